"""Standalone workloads of the render path's kernels, for profiling with ncu.

    python kernel_bench.py io [--side 4096] [--reps 3]
    python kernel_bench.py frame [--canvases 64] [--coverage binned|exact] [--reps 2]
    python kernel_bench.py plain [--canvases 8] [--reps 2]
    python kernel_bench.py encode [--side 1024] [--reps 2]
    python kernel_bench.py hit [--points 1048576] [--reps 2]

* `io` replays, on the plain engine, a call list that puts a random RGBA8
  image over a whole side x side canvas and reads the canvas back: k_put
  (4 B in, 16 B out per pixel) and k_get (16 B in, 4 B out per pixel) each
  run once per replay.
* `frame` renders the first N canvases of the many-canvas workload
  (canvas_ity_gb300.scenes.c3_canvas) as one frame on the tile engine and
  runs it again `reps` times: flattening, stroke expansion, clip passes,
  binning or run scan conversion, clip masks, shadows and the strip kernel.
* `plain` renders the first N workload canvases on the plain per-draw
  engine (k_paint and the per-draw kernels).
* `encode` writes a rendered side x side canvas as PNG and as TGA on the
  GPU (k_encode, k_png_rows).
* `hit` asks is_point_in_path of a workload path for many points at once
  (k_points_in_path).

Each prints one JSON line with its sizes and wall time per repetition;
per-kernel durations and DRAM bytes come from ncu run on the same command.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

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
    ap.add_argument("workload", choices=["io", "frame", "plain", "encode", "hit"])
    ap.add_argument("--side", type=int, default=4096)
    ap.add_argument("--canvases", type=int, default=64)
    ap.add_argument("--coverage", choices=["binned", "exact"], default="binned")
    ap.add_argument("--points", type=int, default=1 << 20)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)
    from canvas_ity_gb300 import build, native, scenes
    from canvas_ity_gb300 import trace as T
    build.build()
    out = {"workload": args.workload}
    if args.workload == "io":
        native.set_engine(1)
        tb = io_trace(args.side)
        native.replay(tb)   # warm-up
        t0 = time.perf_counter()
        for _ in range(args.reps):
            native.replay(tb)
        px = args.side * args.side
        out.update(side=args.side, pixels=px, put_bytes=20 * px, get_bytes=20 * px)
    elif args.workload in ("frame", "plain"):
        engine = 0 if args.workload == "frame" else 1
        native.set_coverage(args.coverage == "exact")
        traces = [scenes.c3_canvas(i) for i in range(args.canvases)]
        with native.Frame(traces, engine) as f:
            f.sync()
            t0 = time.perf_counter()
            for _ in range(args.reps):
                f.run()
            f.sync()
            out.update(canvases=len(traces), coverage=args.coverage if engine == 0 else "exact", **f.stats())
    elif args.workload == "encode":
        native.set_engine(0)
        tb = scenes.mixed_canvas(11, args.side, args.side, 40)
        native.encode_image(tb, native.PNG, 0, 0, args.side, args.side)   # warm-up
        t0 = time.perf_counter()
        for _ in range(args.reps):
            native.encode_image(tb, native.PNG, 0, 0, args.side, args.side)
            native.encode_image(tb, native.TGA, 0, 0, args.side, args.side)
        out.update(side=args.side, pixels=args.side * args.side)
    else:
        tb = scenes.mixed_canvas(12, 1024, 1024, 1)
        rng = np.random.default_rng(0)
        q = rng.uniform(0, 1024, size=(args.points, 2)).astype(np.float32)
        native.points_in_path(tb, q)   # warm-up
        t0 = time.perf_counter()
        for _ in range(args.reps):
            native.points_in_path(tb, q)
        out.update(points=args.points)
    out["ms_per_rep"] = round((time.perf_counter() - t0) / max(args.reps, 1) * 1e3, 3)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
