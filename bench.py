"""Benchmark: batched many-canvas rendering on one GB300.

Workload (default): 4096 independent canvases, each side log-uniform in
[64, 1024] px, 8-128 paths per canvas from the c0/c1/c2 mixture (60/30/10),
seeded synthetic call lists (canvas_ity_gb300.scenes.c3).  A step renders
the whole batch.

* value: Mpix/s of the batched tile engine with the batch already uploaded
  (device time of K runs of the prepared frame, CUDA events on its stream);
* e2e: the same through the public C ABI with host buffers: call lists on the
  host are replayed into canvases (path building, stroke expansion), the
  frame is uploaded, rendered and read back as RGBA8, every step;
* plain: Mpix/s of the per-canvas plain engine (per-draw launches over each
  canvas's float bitmap), over a sample of the same canvases;
* cpu_baseline: the CPU oracle on the host cores on a sample of canvases;
* roofline: the dominant kernel's algorithmic bytes / its measured time.

`--impl reference` times the CPU implementation of the path (the reference
build where it exists, else the CPU oracle) on all host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "Mpix/s batched vs plain per-canvas on 1 GB300 at +/-1 LSB; serving p50/p99 ms"
WORKLOAD = ("c3: 4096 canvases, sides log-uniform 64-1024 px, 8-128 paths each from the "
            "c0/c1/c2 mixture 60/30/10 (fills, strokes, gradients, patterns, 11 ops, shadows, clips)")


def _gen_chunk(args):
    first, count, base = args
    from canvas_ity_gb300 import scenes
    return [scenes.c3_canvas(i, base) for i in range(first, first + count)]


def _gen_requests(args):
    first, count, base = args
    from canvas_ity_gb300 import scenes
    return [scenes.c4_request(i, base) for i in range(first, first + count)]


def generate(count, base_seed, workers, fn=_gen_chunk):
    """Seeded call lists, generated in a spawn pool (before any GPU use)."""
    import multiprocessing as mp
    chunk = max(1, count // (workers * 4))
    jobs = [(i, min(chunk, count - i), base_seed) for i in range(0, count, chunk)]
    if workers <= 1:
        return [t for j in jobs for t in fn(j)]
    with mp.get_context("spawn").Pool(workers) as pool:
        parts = pool.map(fn, jobs)
    return [t for p in parts for t in p]


def pixels_of(traces):
    from canvas_ity_gb300 import trace as T
    total = 0
    for t in traces:
        w, h = T.canvas_size(t)
        total += w * h
    return total


def canvas_cost(trace):
    """Work estimate of one call list: canvas pixels times recorded bytes."""
    from canvas_ity_gb300 import trace as T
    w, h = T.canvas_size(trace)
    return w * h * len(trace)


def cpu_render(traces, threads):
    """Render call lists with the CPU implementation of the path, one canvas
    per task on `threads` threads, the costliest canvases first so the last
    tasks are short; returns (seconds, kind)."""
    import oracle
    kind = "port"
    fn = oracle.replay
    if oracle.reference_available():
        kind, fn = "reference", oracle.reference_replay
    fn(traces[0])  # load the library outside the timed region
    order = sorted(traces, key=canvas_cost, reverse=True)
    t0 = time.perf_counter()
    if threads <= 1:
        for t in order:
            fn(t)
    else:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(fn, order))
    return time.perf_counter() - t0, kind


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """(DRAM bytes per canvas pixel, issue %, FP32-pipe %) of a kernel from the
    committed ncu summary profiles/ncu_traffic.md, or None."""
    path = os.path.join(HERE, "profiles", "ncu_traffic.md")
    try:
        with open(path) as f:
            for line in f:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if len(cells) == 4 and cells[0] == kernel:
                    return float(cells[1]), float(cells[2]), float(cells[3])
    except (OSError, ValueError):
        return None
    return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value, world, backend):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value, world, backend):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reference_arm(args, world, rank):
    """CPU implementation of the path on all host cores, same metric/config."""
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    cores = os.cpu_count() or 1
    # The GPU arm's canvas list (same seed, same count); the K timed steps
    # render it once between them, step i taking canvases i::K, so the
    # figure covers exactly the canvases the GPU arm renders.
    traces = generate(args.canvases, args.seed, min(cores, 16))
    px_all = pixels_of(traces)
    steps = max(1, args.steps)
    for _ in range(args.warmup):
        cpu_render(traces[:16], cores)
    t_total, kind = 0.0, "port"
    for i in range(steps):
        t, kind = cpu_render(traces[i::steps], cores)
        t_total += t
    value = px_all / t_total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mpix/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": round(t_total / steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "canvases": len(traces), "pixels": px_all,
                   "per_step": f"canvases i::{steps} of the batch (all {len(traces)} once over the timed steps)"},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mpix/s", "cores": cores, "kind": kind,
                         "sample": f"the whole {len(traces)}-canvas batch ({px_all} px), 1/{steps} per step, "
                                   "one canvas per thread, costliest first"},
        "e2e": {"value": round(value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def time_frame(frame, runs, torch):
    """Device milliseconds per run of a captured frame (CUDA events on the
    frame's stream, after warm-up)."""
    stream = torch.cuda.ExternalStream(frame.stream())
    frame.capture()
    for _ in range(3):
        frame.run()
    frame.sync()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(runs):
        frame.run()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / runs


def tiger_bench(args, native, T, torch):
    """The reference's own demo drawing (demos/tiger/tiger.cpp: a 733 x 757
    tiger, about 300 fills and strokes), from its recorded call list: one
    tiger per frame (latency), a batch of tigers in one frame (throughput),
    the public replay call end to end, and the oracle port on one host
    thread (best of 5), beside the reference's own time for it."""
    import numpy as np
    import oracle
    tb = T.load(os.path.join(HERE, "tests", "golden", "ref_demos", "tiger.trace.z"))
    w, h = T.canvas_size(tb)
    want = np.frombuffer(T.parse(tb).expected_images()[-1][2].tobytes(), np.uint8).reshape(-1, 4).astype(np.int16)
    cpu_best = min(_timed(lambda: oracle.replay(tb)) for _ in range(5))
    f = native.Frame([tb], 0)
    single_ms = time_frame(f, 20, torch)
    f.finish()
    f.close()
    native.replay(tb)
    e2e_s = min(_timed(lambda: native.replay(tb)) for _ in range(10))
    n = args.tiger_canvases
    f = native.Frame([tb] * n, 0)
    batch_ms = time_frame(f, max(args.steps, 3), torch)
    outs = f.finish()
    f.close()
    d = np.abs(np.frombuffer(outs[0], np.uint8).reshape(-1, 4).astype(np.int16) - want)
    same = all(o == outs[0] for o in outs)
    return {"canvas": f"{w}x{h}, the reference's demos/tiger/tiger.cpp as recorded (tests/golden/ref_demos)",
            "single_ms": round(single_ms, 3), "single_e2e_ms": round(e2e_s * 1e3, 3),
            "batch": {"canvases": n, "ms_per_frame": round(batch_ms, 3),
                      "ms_per_tiger": round(batch_ms / n, 4),
                      "mpix_s": round(n * w * h / (batch_ms / 1e3) / 1e6, 1)},
            "cpu_single_thread_ms": round(cpu_best * 1e3, 2), "cpu_kind": "port",
            "parity_vs_reference": {"max_lsb": int(d.max(initial=0)),
                                    "pixels_differing": int(np.any(d != 0, axis=1).sum()),
                                    "all_batch_canvases_identical": same},
            "coverage": args.coverage}


def _timed(fn):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


def gpu_arm(args, world, rank, local):
    import numpy as np

    cores = os.cpu_count() or 1
    base_seed = args.seed + 100003 * rank
    t_gen = time.perf_counter()
    traces = generate(args.canvases, base_seed, min(cores, 16))
    requests = generate(args.serve_requests, base_seed, min(cores, 16), _gen_requests) if (
        rank == 0 and args.serve_requests > 0) else []
    gen_s = time.perf_counter() - t_gen
    # CPU baseline on a bounded sample (rank 0 only), before the GPU is used.
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        sample = traces[: args.cpu_sample]
        t, kind = cpu_render(sample, cores)
        spx = pixels_of(sample)
        cpu = {"value": round(spx / t / 1e6, 3), "unit": "Mpix/s", "cores": cores, "kind": kind,
               "sample": f"first {len(sample)} canvases of the batch ({spx} px), one render per thread, "
                         f"costliest first, {t:.1f} s"}
        if args.single_sample > 0:
            one = traces[: args.single_sample]
            t1, _ = cpu_render(one, 1)
            opx = pixels_of(one)
            cpu["single_thread"] = {"value": round(opx / t1 / 1e6, 3), "unit": "Mpix/s", "cores": 1,
                                    "sample": f"first {len(one)} canvases of the batch ({opx} px), "
                                              f"one after another on one thread, {t1:.1f} s"}
    import torch
    torch.cuda.set_device(local)
    backend = "nccl"
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend, device_id=torch.device("cuda", local))
    from canvas_ity_gb300 import native, build
    from canvas_ity_gb300 import trace as T
    build.build()
    native.set_coverage(args.coverage == "exact")
    if args.strip_pixels:
        native.set_strip_config(args.strip_pixels, args.strip_threads)
    px = pixels_of(traces)
    # Parity spot check: canvases spread over the batch against the CPU
    # oracle (the reference restatement) under the contract, and bit for bit
    # against the oracle computing the library's coverage.
    import oracle
    parity_set = traces[:: max(1, len(traces) // args.parity_sample)][: args.parity_sample]
    outs = native.render_batch(parity_set, 0)
    oracle.replay(parity_set[0])
    oracle.replay(parity_set[0], ties="sign", trig="cr", coverage="binned" if args.coverage == "binned" else "runs")

    def _parity_one(i):
        tb, raw = parity_set[i], outs[i]
        a = np.frombuffer(raw, np.uint8).reshape(-1, 4).astype(np.int16)
        b = np.frombuffer(oracle.replay(tb)[0], np.uint8).reshape(-1, 4).astype(np.int16)
        same = raw == oracle.replay(tb, ties="sign", trig="cr",
                                    coverage="binned" if args.coverage == "binned" else "runs")[0]
        d = np.abs(a - b)
        low = np.minimum(a[:, 3], b[:, 3]) <= 2
        return (int(d.max(initial=0)), int(d[:, 3].max(initial=0)), int(d[~low, :3].max(initial=0)),
                int(np.any(d != 0, axis=1).sum()), len(a), same)

    with ThreadPoolExecutor(min(cores, 16)) as ex:
        pres = list(ex.map(_parity_one, range(len(parity_set))))
    parity = {"canvases": len(parity_set), "pixels": sum(r[4] for r in pres),
              "max_lsb": max(r[0] for r in pres), "max_lsb_alpha": max(r[1] for r in pres),
              "max_lsb_colour_alpha_above_2": max(r[2] for r in pres),
              "pixels_differing": sum(r[3] for r in pres),
              "max_frac_pixels_differing": round(max(r[3] / r[4] for r in pres), 6),
              "identical_to_coverage_oracle": sum(1 for r in pres if r[5]),
              "against": "oracle (reference restatement); identical_to_coverage_oracle counts canvases equal "
                         "byte for byte to the oracle variant computing this coverage"}
    # Prepared frame: device-resident inputs.
    frame = native.Frame(traces, 0)
    stats = frame.stats()
    stream = torch.cuda.ExternalStream(frame.stream())
    tuned = frame.autotune() if args.autotune else None
    frame.capture()   # every later run is one CUDA graph launch
    for _ in range(max(args.warmup, 3)):
        frame.run()
    frame.sync()
    barrier(world)
    with ClockSampler(local) as clocks:
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(args.steps):
            frame.run()
        stop.record(stream)
        stop.synchronize()
        elapsed_ms = start.elapsed_time(stop)
    torch.cuda.synchronize()
    barrier(world)
    t_max = reduce_max(elapsed_ms / 1e3, world, backend)
    px_all = reduce_sum(float(px), world, backend)
    value = px_all * args.steps / t_max / 1e6
    # Phase profile of one run (CUDA events on the frame's stream).
    frame.set_profiling(True)
    frame.run()
    phases = frame.profile()
    frame.set_profiling(False)
    frame.finish()
    frame.close()
    # End to end through the public C ABI (cy_render_traces): call lists in
    # host memory to RGBA8 reads in host memory, every step replaying,
    # uploading, rendering and reading back all canvases; frames of about
    # 32 Mpx are pipelined so host work overlaps device work.  The output
    # buffer and its per-canvas offsets (the sizes of the recorded
    # get_image_data calls) are the caller's, prepared once.
    t_e2e = 0.0
    h2d = d2h = 0
    e2e_parts = {}
    e2e_steps = args.steps if args.e2e_steps < 0 else args.e2e_steps
    if e2e_steps > 0:
        offsets = np.zeros(len(traces) + 1, np.uint64)
        offsets[1:] = np.cumsum([T.read_bytes(t) for t in traces], dtype=np.uint64)
        out_buf = np.zeros(max(int(offsets[-1]), 1), np.uint8)
        views, _ = native.render_traces(traces, 0, 0, out_buf, offsets)   # warm-up: frame workspaces
        check = native.render_batch(traces[:4], 0)
        for a, b in zip(views[:4], check):
            if bytes(a) != b:
                raise RuntimeError("cy_render_traces differs from the frame path")
        frames = 0
        for i in range(e2e_steps):
            t0 = time.perf_counter()
            views, st = native.render_traces(traces, 0, 0, out_buf, offsets)
            t_e2e += time.perf_counter() - t0
            h2d, d2h, frames = st["upload_bytes"], st["read_bytes"], st["frames"]
        e2e_parts = {"api": "cy_render_traces", "frames": frames}
    e2e_s = reduce_max(t_e2e / max(e2e_steps, 1), world, backend)
    e2e = px_all / e2e_s / 1e6 if e2e_s > 0 else None
    # Plain per-canvas path on a sample of the same canvases.
    sample = traces[: args.plain_sample]
    plain_ms = 0.0
    for tb in sample:
        f = native.Frame([tb], 1)
        s0 = torch.cuda.ExternalStream(f.stream())
        f.run()
        f.sync()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s0)
        f.run()
        b.record(s0)
        b.synchronize()
        plain_ms += a.elapsed_time(b)
        f.finish()
        f.close()
    plain = pixels_of(sample) / (plain_ms / 1e3) / 1e6 if plain_ms > 0 else None
    tiger = tiger_bench(args, native, T, torch) if rank == 0 and args.tiger_canvases > 0 else None
    # Serving: Poisson arrivals of mixed-size requests (cycled from the
    # generated pool), continuous batching under a 150 GB admission budget
    # (rank 0).  Each stated rate is offered for --serve-seconds of arrivals
    # at steady state; a rate the server cannot carry builds a backlog, and
    # its completion rate is then the measured capacity.  Latency is also
    # reported at 80% of that capacity.
    serving_out = None
    if requests:
        from canvas_ity_gb300 import serving
        serving_out = {"request_pool": len(requests), "budget_gb": 150, "workers": args.serve_workers,
                       "max_frame_pixels": args.serve_frame_pixels, "offer_seconds": args.serve_seconds,
                       "workload": "c4: sides log-uniform 32-2048 px, 1-512 paths from the c0/c1/c2 mixture",
                       "rates": []}
        with serving.Server(budget_bytes=150 * 10**9, workers=args.serve_workers,
                            max_pixels=args.serve_frame_pixels) as srv:
            serving.run_poisson(srv, requests[: max(1, len(requests) // 8)], 2000.0, seed=0)   # warm-up
            for rate in (2000.0, 10000.0, 20000.0):
                serving_out["rates"].append(serving.run_steady(srv, requests, rate, args.serve_seconds,
                                                               seed=int(rate)))
            sat = [r["achieved_req_s"] for r in serving_out["rates"] if r["saturated"]]
            if sat:
                cap = max(sat)
                serving_out["capacity_req_s"] = cap
                serving_out["at_80pct_capacity"] = serving.run_steady(srv, requests, 0.8 * cap, args.serve_seconds,
                                                                      seed=7)
            st = srv.stats()
        serving_out["frames"] = st["frames"]
        serving_out["max_batch"] = st["max_batch"]
        serving_out["max_admitted_gb"] = round(st["max_bytes_admitted"] / 1e9, 2)
    # Roofline of the dominant kernel.  Algorithmic bytes of one step are
    # what the render must move at least: the call data uploaded (points,
    # subpaths, paint records, stops and texels, commands), the float canvas
    # state every canvas keeps (16 B per pixel written) and the RGBA8 reads
    # (4 B per pixel).  The paint kernel (k_strips) reads the prepared inputs
    # and writes every output, so the step's bytes are its algorithmic bytes;
    # the rest of the step is scan conversion, shadows and masks.
    peak, peak_kind = measured_peaks()
    in_b, out_b, state_b = stats["upload_bytes"], stats["read_bytes"], 16 * stats["pixels"]
    alg = in_b + out_b + state_b
    kernel = "k_strips"
    kms = phases.get("paint", 0.0)
    achieved = alg / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    prof = ncu_traffic(kernel + (" binned" if args.coverage == "binned" else " exact"))
    # Intermediates that stay on the device between kernels, written once
    # and read once: binned segment entries (16 B) and, for shadows and
    # clips, runs with their sums (12 B).
    inter = 2 * (16 * stats.get("bin_entries", 0) + 12 * stats["runs"])
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "peak_source": peak_kind,
                "traffic": (round(prof[0] * stats["pixels"]) if prof else None),
                "traffic_source": ("ncu DRAM bytes per canvas pixel of a 64-canvas capture of this kernel "
                                   "(profiles/ncu_traffic.md), scaled by the step's pixels") if prof else None,
                "algorithmic_bytes": alg,
                "algorithmic_parts": {"inputs": in_b, "rgba8_out": out_b, "canvas_state": state_b},
                "traffic_intermediate": inter, "kernel_ms": round(kms, 3),
                "step_achieved": round(alg / (elapsed_ms / args.steps / 1e3) / 1e9, 1),
                "note": "compute/latency-bound: see issue/fp32 utilisation (ncu, profiles/)",
                "issue_pct": prof[1] if prof else None, "fp32_pipe_pct": prof[2] if prof else None}
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(t_max * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "canvases": len(traces), "pixels": px, "engine": "tile",
                   "strip_pixels": tuned["strip_pixels"] if tuned else (args.strip_pixels or 4096),
                   "strip_threads": tuned["threads"] if tuned else (args.strip_threads or 256),
                   "autotuned": bool(tuned), "cuda_graph": True, "commands": stats["commands"],
                   "coverage": args.coverage, "segments": stats["segments"], "runs": stats["runs"],
                   "bin_entries": stats.get("bin_entries"), "shadows": stats["shadows"],
                   "clips": stats["clips"], "l2": "inputs larger than L2 (runs and outputs are GBs)",
                   "parallelism": f"replicas x{world}", "generate_s": round(gen_s, 1)},
        "e2e": {"value": round(e2e, 2) if e2e else None, "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "host_threads": cores,
                **e2e_parts},
        "plain_per_canvas": {"value": round(plain, 2) if plain else None, "unit": "Mpix/s",
                             "sample_canvases": len(sample)},
        "batched_over_plain": round(value / plain, 2) if plain else None,
        "tiger": tiger,
        "phases_ms": {k: round(v, 3) for k, v in phases.items()},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "parity": parity,
        "serving": serving_out,
        "clocks": clocks.summary(),
        "gpu_launches": stats["launches"] * args.steps,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--canvases", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-sample", type=int, default=128)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--parity-sample", type=int, default=32)
    ap.add_argument("--single-sample", type=int, default=24, help="canvases of the single-thread CPU baseline")
    ap.add_argument("--tiger-canvases", type=int, default=256, help="tigers per frame in the demo timing (0: none)")
    ap.add_argument("--autotune", type=int, default=1, help="pick the strip configuration by timing (1) or not (0)")
    ap.add_argument("--serve-requests", type=int, default=240, help="requests per arrival rate (0: no serving run)")
    ap.add_argument("--serve-workers", type=int, default=4)
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="seconds of arrivals offered per rate")
    ap.add_argument("--serve-frame-pixels", type=int, default=32 << 20, help="canvas pixels per server frame")
    ap.add_argument("--e2e-steps", type=int, default=-1, help="end-to-end calls timed (-1: --steps)")
    ap.add_argument("--strip-pixels", type=int, default=0)
    ap.add_argument("--strip-threads", type=int, default=256)
    ap.add_argument("--coverage", choices=["binned", "exact"], default="binned",
                    help="tile engine coverage: binned fixed-point sums (default) or exact sorted runs")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        gpu_arm(args, world, rank, local)


if __name__ == "__main__":
    main()
