"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference sources are present.  Steps:
  1. build oracle/_ref/ (oracle/ref/build_ref.sh): the reference's own test
     program (test/test.cpp) compiled against the recording canvas;
  2. run it: each of its 76 tests records its call list, including the
     reference's get_image_data / is_point_in_path / measure_text answers;
  3. store each call list zlib-compressed as ref_tests/<name>.trace.z and
     write manifest.json with the golden hash of every test, read from the
     reference's table (test/test.cpp:2185-2261), the hash the reference
     produced here, and the SHA-256 of the PNG file its own writer made of
     the test's image (test.cpp's --pngs, write_png at test.cpp:2415-2511);
  4. run the reference's tiger demo (demos/tiger/tiger.cpp) compiled against
     the same recording canvas: its first canvas's call list goes to
     ref_demos/tiger.trace.z, and the SHA-256 of the tiger.tga its own TGA
     writer made (tiger.cpp:4333-4345) to the manifest's "demos".

Usage: python tests/golden/make_golden.py REFERENCE_ROOT   (or CY_REFERENCE_ROOT set)
"""
import glob
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CY_REFERENCE_ROOT")
    if not ref:
        raise SystemExit(__doc__)
    subprocess.check_call(["sh", os.path.join(REPO, "oracle", "ref", "build_ref.sh"), ref])
    table = {}
    with open(os.path.join(ref, "test", "test.cpp")) as f:
        for m in re.finditer(r'\{\s*0x([0-9a-f]{8}),\s*(\d+),\s*(\d+),\s*(\w+),\s*"(\w+)"\s*\}', f.read()):
            table[m.group(5)] = {"golden_hash": int(m.group(1), 16), "width": int(m.group(2)),
                                 "height": int(m.group(3))}
    out_dir = os.path.join(HERE, "ref_tests")
    os.makedirs(out_dir, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        env = dict(os.environ, CY_RECORD_DIR=tmp)
        log = subprocess.run([os.path.join(REPO, "oracle", "_ref", "ref_recorder"), "--plain", "--pngs"],
                             env=env, cwd=tmp, check=True, capture_output=True, text=True).stdout
        lines = [l for l in log.splitlines() if re.match(r"\s*\d+/\d+ \[", l)]
        traces = sorted(glob.glob(os.path.join(tmp, "trace_*.bin")))
        if len(lines) != len(traces):
            raise SystemExit(f"{len(lines)} results but {len(traces)} call lists")
        manifest = []
        for line, path in zip(lines, traces):
            m = re.match(r"\s*\d+/\d+ \[(PASS|FAIL)\] ([0-9a-f]{8})\s+\S+ms (\w+)", line)
            name = m.group(3)
            with open(path, "rb") as f:
                raw = f.read()
            with open(os.path.join(out_dir, name + ".trace.z"), "wb") as f:
                f.write(zlib.compress(raw, 9))
            with open(os.path.join(tmp, name + ".png"), "rb") as f:
                png = f.read()
            entry = dict(name=name, trace="ref_tests/" + name + ".trace.z",
                         reference_hash=int(m.group(2), 16), reference_passed=m.group(1) == "PASS",
                         reference_png_sha256=hashlib.sha256(png).hexdigest(), reference_png_bytes=len(png))
            entry.update(table[name])
            manifest.append(entry)
    demos = []
    demo_dir = os.path.join(HERE, "ref_demos")
    os.makedirs(demo_dir, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        env = dict(os.environ, CY_RECORD_DIR=tmp)
        subprocess.run([os.path.join(REPO, "oracle", "_ref", "ref_tiger_recorder")], env=env, cwd=tmp, check=True,
                       capture_output=True)
        with open(os.path.join(tmp, "trace_000.bin"), "rb") as f:   # the first trial's canvas
            raw = f.read()
        with open(os.path.join(demo_dir, "tiger.trace.z"), "wb") as f:
            f.write(zlib.compress(raw, 9))
        with open(os.path.join(tmp, "tiger.tga"), "rb") as f:
            tga = f.read()
        demos.append(dict(name="tiger", trace="ref_demos/tiger.trace.z", width=733, height=757,
                          reference_tga_sha256=hashlib.sha256(tga).hexdigest(), reference_tga_bytes=len(tga)))
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"source": "canvas_ity test/test.cpp and demos/tiger/tiger.cpp via oracle/ref/recorder.cpp",
                   "tests": manifest, "demos": demos}, f, indent=1)
    print(f"wrote {len(manifest)} fixtures")


if __name__ == "__main__":
    main()
