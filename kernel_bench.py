"""Standalone workloads for the bandwidth-bound kernels, for profiling.

    python kernel_bench.py io [--side 4096] [--reps 3]

`io` replays, on the plain engine, a call list that puts a random RGBA8
image over a whole side x side canvas and reads the canvas back: k_put
(4 B in, 16 B out per pixel) and k_get (16 B in, 4 B out per pixel) each run
once per replay.  It prints one JSON line with the wall time per replay;
per-kernel durations and DRAM bytes come from ncu on this command.
"""
from __future__ import annotations

import argparse
import json
import time

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def io_trace(side: int, seed: int = 0) -> bytes:
    from canvas_ity_gb300 import trace as T
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(side, side, 4), dtype=np.uint8)
    t = T.TraceWriter(side, side)
    t.put_image_data(img, side, side, 0, 0)
    t.get_image_data(side, side, 0, 0)
    return t.finish(read_back=False)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["io"])
    ap.add_argument("--side", type=int, default=4096)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)
    from canvas_ity_gb300 import build, native
    build.build()
    native.set_engine(1)
    tb = io_trace(args.side)
    native.replay(tb)   # warm-up
    t0 = time.perf_counter()
    for _ in range(args.reps):
        native.replay(tb)
    dt = (time.perf_counter() - t0) / args.reps
    px = args.side * args.side
    print(json.dumps({"workload": "io", "side": args.side, "pixels": px, "replay_ms": round(dt * 1e3, 3),
                      "put_bytes": 20 * px, "get_bytes": 20 * px}))


if __name__ == "__main__":
    main()
