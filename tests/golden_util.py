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


def load_fixture(entry: dict) -> bytes:
    return T.load(os.path.join(GOLDEN, entry["trace"]))


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
