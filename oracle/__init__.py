"""CPU oracle for the canvas_ity render path -- TEST INFRASTRUCTURE ONLY.

`oracle/cy_oracle.cpp` restates the reference CPU algorithm
(src/canvas_ity.hpp); this module builds it with g++ and replays recorded
call lists through it.  `oracle/ref/` builds the reference itself from its
own sources when they are present (not on the GPU host) for pinning.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
use this package; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Optional, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libcy_oracle.so")
# Variants of the same restatement:
#  ties="sign": equal-magnitude, opposite-sign runs of a cell ordered negative
#    first (the GPU's order) instead of std::sort's own choice;
#  trig="cr": round joins take acos and tan in double precision rounded to
#    float (the GPU stroke expansion's choice) instead of libm's acosf/tanf.
ORACLE_SIGN_SO = os.path.join(BUILD_DIR, "libcy_oracle_sign.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libcy_ref.so")
# Where the reference sources lie: CY_REFERENCE_ROOT, or the root passed to
# build_reference().  Unset (as on a machine without them): no reference tools.
REFERENCE_ROOT = os.environ.get("CY_REFERENCE_ROOT")

_FLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"]


def _variant(ties: str, trig: str, coverage: str = "runs") -> Tuple[str, list]:
    name, extra = "libcy_oracle", []
    if ties == "sign":
        name, extra = name + "_sign", extra + ["-DCYO_TIES_BY_SIGN"]
    if trig == "cr":
        name, extra = name + "_cr", extra + ["-DCYO_CR_TRIG"]
    if coverage == "binned":
        name, extra = name + "_binned", extra + ["-DCYO_BINNED"]
    return os.path.join(BUILD_DIR, name + ".so"), extra


def build(force: bool = False, ties: str = "reference", trig: str = "libm", coverage: str = "runs") -> str:
    """Compile the oracle restatement (fast: one translation unit).

    ties="sign" builds the variant whose sort orders equal-magnitude,
    opposite-sign runs of one cell negative first; trig="cr" the variant
    whose round joins use correctly rounded acos/tan; coverage="binned" the
    variant whose draws take the library's sort-free fixed-point coverage
    instead of the reference's sorted runs (its distance from the reference
    is what the tests bound)."""
    src = os.path.join(HERE, "cy_oracle.cpp")
    out, extra = _variant(ties, trig, coverage)
    hdrs = [os.path.join(HERE, "..", "include", h) for h in ("cy_trace.h", "cy_replay.hpp")]
    newest = max(os.path.getmtime(p) for p in [src] + hdrs)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp"
    subprocess.check_call(["g++", *_FLAGS, *extra, "-o", tmp, src])
    os.replace(tmp, out)
    return out


def build_reference(force: bool = False, root: Optional[str] = None) -> Optional[str]:
    """Build the reference tools from the read-only sources under `root` (or
    CY_REFERENCE_ROOT), if they are there; returns the library path or None.
    Tools built earlier are reused when no sources are named."""
    root = root or REFERENCE_ROOT
    if not root or not os.path.isfile(os.path.join(root, "src", "canvas_ity.hpp")):
        return REF_SO if os.path.exists(REF_SO) and not force else None
    ours = [os.path.join(HERE, "ref", f) for f in os.listdir(os.path.join(HERE, "ref"))]
    ours += [os.path.join(HERE, "..", "include", h) for h in ("cy_trace.h", "cy_replay.hpp")]
    stale = not os.path.exists(REF_SO) or os.path.getmtime(REF_SO) < max(os.path.getmtime(p) for p in ours)
    if force or stale:
        subprocess.check_call(["sh", os.path.join(HERE, "ref", "build_ref.sh"), root])
    return REF_SO


class _Lib:
    def __init__(self, path: str, symbol: str):
        self.lib = ctypes.CDLL(path)
        self.fn = getattr(self.lib, symbol)
        self.fn.restype = ctypes.c_int
        self.fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                            ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_float),
                            ctypes.c_int, ctypes.POINTER(ctypes.c_int)]

    def replay(self, trace: bytes) -> Tuple[bytes, List[float]]:
        cap, rcap = 1 << 20, 1024
        while True:
            img = ctypes.create_string_buffer(cap)
            res = (ctypes.c_float * rcap)()
            n_img, n_res = ctypes.c_size_t(0), ctypes.c_int(0)
            rc = self.fn(trace, len(trace), img, cap, ctypes.byref(n_img), res, rcap, ctypes.byref(n_res))
            if rc == -2 and (n_img.value > cap or n_res.value > rcap):
                cap, rcap = max(cap, n_img.value), max(rcap, n_res.value)
                continue
            if rc != 0:
                raise ValueError(f"replay failed with status {rc}")
            return img.raw[: n_img.value], [res[i] for i in range(n_res.value)]


_oracles: dict = {}
_ref: Optional[_Lib] = None


def _get(ties: str, trig: str = "libm", coverage: str = "runs") -> _Lib:
    key = (ties, trig, coverage)
    if key not in _oracles:
        _oracles[key] = _Lib(build(ties=ties, trig=trig, coverage=coverage), "cyo_replay")
    return _oracles[key]


def replay(trace: bytes, ties: str = "reference", trig: str = "libm",
           coverage: str = "runs") -> Tuple[bytes, List[float]]:
    """Replay through the oracle: (concatenated get_image_data bytes, results)."""
    return _get(ties, trig, coverage).replay(trace)


def replay_linear(trace: bytes, width: int, height: int, ties: str = "reference", trig: str = "libm",
                  coverage: str = "runs"):
    """Replay through the oracle; return the final float canvas (H, W, 4)."""
    import numpy as np
    fn = _get(ties, trig, coverage).lib.cyo_replay_linear
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float), ctypes.c_size_t,
                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    out = np.zeros((height, width, 4), np.float32)
    w, h = ctypes.c_int(0), ctypes.c_int(0)
    rc = fn(trace, len(trace), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size,
            ctypes.byref(w), ctypes.byref(h))
    if rc != 0:
        raise ValueError(f"oracle replay failed with status {rc}")
    return out


def reference_available() -> bool:
    return os.path.exists(REF_SO) or build_reference() is not None


def reference_replay(trace: bytes) -> Tuple[bytes, List[float]]:
    """Replay through the reference header itself (needs its sources)."""
    global _ref
    if _ref is None:
        path = build_reference()
        if path is None:
            raise RuntimeError("reference sources are not available here")
        _ref = _Lib(path, "cyr_replay")
    return _ref.replay(trace)
