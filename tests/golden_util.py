"""Helpers shared by the parity tests: golden fixtures and image splitting."""
import json
import os
from typing import List, Tuple

import numpy as np

from canvas_ity_gb300 import trace as T

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest() -> List[dict]:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)["tests"]


def demos() -> List[dict]:
    """The reference's demo programs recorded (the tiger): call list, size
    and the SHA-256 of the image file the demo itself wrote."""
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f).get("demos", [])


def load_fixture(entry: dict) -> bytes:
    return T.load(os.path.join(GOLDEN, entry["trace"]))


def final_image(trace_bytes: bytes) -> np.ndarray:
    """The reference's answer to the call list's last get_image_data: for the
    recorded tests and demos, the whole canvas read after drawing."""
    return T.parse(trace_bytes).expected_images()[-1][2]


def split_images(trace_bytes: bytes, raw: bytes) -> List[np.ndarray]:
    """Split concatenated get_image_data outputs by the sizes in the trace."""
    t = T.parse(trace_bytes)
    out, at = [], 0
    for r in t.records:
        if r.op == T.GET_IMAGE_DATA and r.args[4] and r.args[0] > 0 and r.args[1] > 0:
            w, h = r.args[0], r.args[1]
            n = w * h * 4
            out.append(np.frombuffer(raw[at:at + n], np.uint8).reshape(h, w, 4))
            at += n
    assert at == len(raw), "image bytes do not match the trace"
    return out


def compare(a: np.ndarray, b: np.ndarray) -> Tuple[int, float]:
    """(max per-channel difference, fraction of pixels that differ at all)."""
    d = np.abs(a.astype(np.int16) - b.astype(np.int16))
    return int(d.max(initial=0)), float(np.any(d != 0, axis=-1).mean()) if d.size else 0.0


# ---------------------------------------------------------------- tolerance
# The parity contract for RGBA8 reads against the reference (or its
# restatement): at least MIN_IDENTICAL of the pixels identical; the alpha
# byte within MAX_LSB everywhere; the colour bytes within MAX_LSB wherever
# alpha is above LOW_ALPHA / 255.  Below that, get_image_data divides the
# colour by alpha (hpp:3348-3381): a difference in the last bit of a
# premultiplied float is magnified up to 8160x, so those colour bytes of a
# nearly transparent pixel are not bounded.  `strict` additionally bounds
# every colour byte by MAX_LSB (what the exact coverage path meets).
MAX_LSB = 1
MIN_IDENTICAL = 0.995
LOW_ALPHA = 2


def contract_stats(a: np.ndarray, b: np.ndarray) -> dict:
    d = np.abs(a.astype(np.int16) - b.astype(np.int16)).reshape(-1, 4)
    if d.size == 0:
        return {"max": 0, "alpha": 0, "colour_opaque": 0, "frac": 0.0}
    low = np.minimum(a.reshape(-1, 4)[:, 3], b.reshape(-1, 4)[:, 3]) <= LOW_ALPHA
    return {"max": int(d.max()), "alpha": int(d[:, 3].max()),
            "colour_opaque": int(d[~low, :3].max(initial=0)), "frac": float(np.any(d != 0, axis=1).mean())}


def assert_within_contract(got: np.ndarray, want: np.ndarray, what: str, strict: bool = False) -> None:
    assert got.shape == want.shape, what
    s = contract_stats(got, want)
    assert s["alpha"] <= MAX_LSB, f"{what}: alpha differs by {s['alpha']}"
    assert s["colour_opaque"] <= MAX_LSB, f"{what}: colour differs by {s['colour_opaque']} where alpha > {LOW_ALPHA}"
    if strict:
        assert s["max"] <= MAX_LSB, f"{what}: max channel difference {s['max']}"
    assert s["frac"] <= 1.0 - MIN_IDENTICAL, f"{what}: {s['frac']:.4%} of pixels differ"


# -------------------------------------------------------------- render modes
# The GPU path's modes, and the oracle variant each equals bit for bit:
#   tile        tile engine, binned coverage (the default): the oracle's
#               coverage="binned" restatement of the same fixed-point sums;
#   tile_exact  tile engine, sorted-run coverage: the oracle itself;
#   plain       per-draw engine (always sorted runs): the oracle itself.
MODES = {"tile": (0, False), "tile_exact": (0, True), "plain": (1, True)}


def use_mode(mode: str) -> None:
    from canvas_ity_gb300 import native
    engine, exact = MODES[mode]
    native.set_engine(engine)
    native.set_coverage(exact)


def oracle_coverage(mode: str) -> str:
    return "binned" if mode == "tile" else "runs"


def far_point_scene(bad: float) -> bytes:
    """Three fills on a 64 x 48 canvas, two of them with one vertex at `bad`
    (a non-finite value, or a point far off the canvas): one in x, one in y."""
    t = T.TraceWriter(64, 48)
    t.set_color(T.FILL_STYLE, 0.2, 0.4, 0.8, 1.0)
    t.begin_path()
    t.move_to(5, 5)
    t.line_to(50, 8)
    t.line_to(bad, 30)
    t.line_to(40, 44)
    t.line_to(6, 40)
    t.close_path()
    t.fill()
    t.set_color(T.FILL_STYLE, 0.9, 0.3, 0.1, 0.7)
    t.begin_path()
    t.move_to(-20, 10)
    t.line_to(30, bad)
    t.line_to(60, 30)
    t.close_path()
    t.fill()
    t.begin_path()
    t.move_to(10, 10)
    t.line_to(20, 12)
    t.line_to(14, 30)
    t.close_path()
    t.fill()
    return t.finish()
