"""ctypes binding of libcanvas_ity_gb300.so (the C ABI in include/).

Loading never falls back to anything else: if the CUDA library has not been
built, every call raises.  Build it with ``canvas_ity_gb300.build.build()``.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Tuple

import numpy as np

from . import build as _build

_lib: Optional[ctypes.CDLL] = None


def library_path() -> str:
    return _build.LIB


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first "
                           "(python -c 'import canvas_ity_gb300.build as b; b.build()')")
    lib = ctypes.CDLL(path)
    c_size_p = ctypes.POINTER(ctypes.c_size_t)
    c_int_p = ctypes.POINTER(ctypes.c_int)
    lib.cy_replay.restype = ctypes.c_int
    lib.cy_replay.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, c_size_p,
                              ctypes.POINTER(ctypes.c_float), ctypes.c_int, c_int_p]
    lib.cy_replay_linear.restype = ctypes.c_int
    lib.cy_replay_linear.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                                     ctypes.c_size_t, c_int_p, c_int_p]
    lib.cy_set_engine.restype = None
    lib.cy_set_engine.argtypes = [ctypes.c_int]
    _lib = lib
    return lib


def set_engine(engine: int) -> None:
    """0 = tile engine, 1 = plain per-draw engine (this thread)."""
    load().cy_set_engine(int(engine))


def replay(trace: bytes) -> Tuple[bytes, List[float]]:
    """Replay a call list through canvas_ity::canvas on the GPU.

    Returns (concatenated get_image_data bytes, is_point_in_path /
    measure_text results)."""
    lib = load()
    cap, rcap = 1 << 20, 1024
    while True:
        img = ctypes.create_string_buffer(cap)
        res = (ctypes.c_float * rcap)()
        n_img, n_res = ctypes.c_size_t(0), ctypes.c_int(0)
        rc = lib.cy_replay(trace, len(trace), img, cap, ctypes.byref(n_img), res, rcap, ctypes.byref(n_res))
        if rc == -2:
            cap, rcap = max(cap, n_img.value), max(rcap, n_res.value)
            continue
        if rc != 0:
            raise RuntimeError(f"cy_replay failed with status {rc}")
        return img.raw[: n_img.value], [res[i] for i in range(n_res.value)]


def replay_linear(trace: bytes, width: int, height: int) -> np.ndarray:
    """Replay and return the final premultiplied linear float canvas (H, W, 4)."""
    lib = load()
    out = np.zeros((height, width, 4), np.float32)
    w, h = ctypes.c_int(0), ctypes.c_int(0)
    rc = lib.cy_replay_linear(trace, len(trace), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                              out.size, ctypes.byref(w), ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"cy_replay_linear failed with status {rc}")
    return out
