"""Device kernels compiled as host C++ (tests/host_kernels/shim.h) and run
once per thread index on the CPU, against the reference's own semantics:
the image file packing against its PNG and TGA writers, the batched hit
test against the sequential is_point_in_path, and the stroke kernels (warp
kernels, run through tests/host_kernels/warp_emu.h) against the host
class's own stroke expansion.  The GPU tests run the
same kernels on the device (tests/test_encode.py, tests/test_points_in_path.py)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")
HERE = os.path.join(ROOT, "tests", "host_kernels")


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


def _run(tmp_path, sources, std="c++17", objects=(), args=(), libs=()):
    inc = _cuda_include()
    if not shutil.which("g++") or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "check")
    cmd = ["g++", "-O2", f"-std={std}", "-ffp-contract=off", "-w", "-I", os.path.join(ROOT, "include"), "-I", inc,
           *sources, *objects, "-o", exe, *libs]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([exe, *args], check=True, capture_output=True, text=True).stdout.strip()


def test_pack_kernels_match_reference_writers(tmp_path):
    out = _run(tmp_path, [os.path.join(HERE, "pack_check.cpp")])
    assert out.endswith("mismatching 0"), out
    assert not out.startswith("cases 0"), out


def test_hit_kernel_matches_sequential_is_point_in_path(tmp_path):
    out = _run(tmp_path, [os.path.join(HERE, "hit_check.cpp"),
                          os.path.join(ROOT, "canvas_ity_gb300", "csrc", "canvas.cpp")])
    assert out.endswith("differing 0"), out
    assert not out.startswith("queries 0"), out


def _stroke_scene(path):
    """Six strokes: every join and cap, dashes (odd pattern, negative offset,
    closed subpaths whose first and last dashes merge), a step shorter than
    1e-4, tight turns, curves, and a scaled, rotated transform."""
    from canvas_ity_gb300 import trace as T
    t = T.TraceWriter(64, 48)

    def stroke(width, join, cap, pts, dash=None, off=0.0, closed=False, curve=False):
        t.set_line_width(width)
        t.set_line_join(join)
        t.set_line_cap(cap)
        t.set_line_dash(dash or [])
        t.set_line_dash_offset(off)
        t.begin_path()
        t.move_to(*pts[0])
        for i, p in enumerate(pts[1:]):
            if curve and i % 2:
                t.bezier_curve_to(p[0] - 9, p[1] + 12, p[0] + 7, p[1] - 8, *p)
            else:
                t.line_to(*p)
        if closed:
            t.close_path()
        t.stroke()

    t.set_color(T.STROKE_STYLE, 0.2, 0.4, 0.8, 0.9)
    stroke(4.0, 0, 0, [(5, 5), (40, 8), (12, 30), (50, 40)])
    stroke(3.0, 2, 2, [(8, 40), (30, 10), (55, 35), (20, 44)], curve=True)
    stroke(2.5, 1, 1, [(10, 10), (54, 12), (50, 40), (14, 38)], dash=[5.0, 3.0], off=-2.0, closed=True)
    stroke(6.0, 2, 0, [(30, 24), (31, 24), (31.00001, 24.00001), (45, 30), (35, 44)], dash=[2.0, 1.0, 4.0],
           closed=True, curve=True)
    stroke(1.0, 0, 2, [(2, 46), (62, 2), (2, 2), (62, 46)])
    t.scale(1.5, 0.75)
    t.rotate(0.4)
    stroke(2.0, 2, 1, [(10, 5), (30, 5), (30, 25), (10, 25)], closed=True, curve=True)
    with open(path, "wb") as f:
        f.write(t.finish(read_back=False))


def test_stroke_kernels_match_host_expansion(tmp_path):
    inc = _cuda_include()
    if not shutil.which("g++") or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    libdir = os.path.join(os.path.dirname(inc), "lib64")
    if not os.path.exists(libdir):
        libdir = os.path.join(os.path.dirname(inc), "lib")
    objs = []
    for name in ("canvas", "capi"):
        obj = str(tmp_path / f"{name}.o")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-include",
                        os.path.join(HERE, "cr_trig.h"), "-I", os.path.join(ROOT, "include"), "-I", inc, "-c",
                        os.path.join(ROOT, "canvas_ity_gb300", "csrc", f"{name}.cpp"), "-o", obj],
                       check=True, capture_output=True, text=True)
        objs.append(obj)
    scene = str(tmp_path / "strokes.trace")
    _stroke_scene(scene)
    # and two canvases of the many-canvas workload: long dashed polylines
    # (dash walks over many 32-segment chunks), every join and cap kind
    from canvas_ity_gb300 import scenes
    workload = []
    for i in (0, 1):
        path = str(tmp_path / f"c3_{i}.trace")
        with open(path, "wb") as f:
            f.write(scenes.c3_canvas(i))
        workload.append(path)
    out = _run(tmp_path, [os.path.join(HERE, "stroke_check.cpp")], std="c++20", objects=objs, args=[scene],
               libs=["-L", libdir, f"-Wl,-rpath,{libdir}", "-lcudart", "-lpthread"])
    assert out == "commands 6, differing 0", out
    out = subprocess.run([str(tmp_path / "check"), *workload], check=True, capture_output=True,
                         text=True).stdout.strip()
    assert out.endswith("differing 0") and not out.startswith("commands 0"), out
