"""Continuous-batching render server (include/cy_serve.h) and a Poisson load
driver for it.

A request is a recorded call list; its result is the bytes of its
get_image_data reads.  The native server admits waiting requests against a
device-memory budget and renders them in frames on several worker streams;
this module only submits, polls and measures.
"""
from __future__ import annotations

import ctypes
import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import native

STAT_NAMES = ("frames", "requests", "pixels", "waiting", "bytes_admitted", "max_bytes_admitted",
              "max_batch", "budget")


def _lib() -> ctypes.CDLL:
    lib = native.load()
    if getattr(lib, "_serve_ready", False):
        return lib
    vp = ctypes.c_void_p
    lib.cy_server_create.restype = ctypes.c_int
    lib.cy_server_create.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_longlong, ctypes.POINTER(vp)]
    lib.cy_server_submit.restype = ctypes.c_int
    lib.cy_server_submit.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.cy_server_poll.restype = ctypes.c_int
    lib.cy_server_poll.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_int),
                                   vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                   ctypes.POINTER(ctypes.c_double)]
    lib.cy_server_stats.restype = ctypes.c_int
    lib.cy_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
    lib.cy_server_destroy.restype = None
    lib.cy_server_destroy.argtypes = [vp]
    lib._serve_ready = True
    return lib


@dataclass
class Result:
    id: int
    status: int
    images: bytes
    latency_ms: float


class Server:
    """Worker threads on the current device; `budget_bytes` of device memory
    may be admitted at once (150 GB by default)."""

    def __init__(self, budget_bytes: int = 150 * 10**9, workers: int = 3, host_threads: int = 0,
                 max_batch: int = 256, max_pixels: int = 16 << 20):
        self.lib = _lib()
        self.handle = ctypes.c_void_p()
        rc = self.lib.cy_server_create(int(budget_bytes), int(workers), int(host_threads), int(max_batch),
                                       int(max_pixels), ctypes.byref(self.handle))
        if rc != 0:
            raise RuntimeError(f"cy_server_create failed with status {rc}")
        self._buf = ctypes.create_string_buffer(1 << 20)

    def submit(self, trace: bytes) -> int:
        rid = ctypes.c_ulonglong(0)
        rc = self.lib.cy_server_submit(self.handle, trace, len(trace), ctypes.byref(rid))
        if rc != 0:
            raise RuntimeError(f"cy_server_submit failed with status {rc}")
        return rid.value

    def poll(self, wait_ms: int = -1) -> Optional[Result]:
        rid, st, n, lat = ctypes.c_ulonglong(0), ctypes.c_int(0), ctypes.c_size_t(0), ctypes.c_double(0.0)
        while True:
            rc = self.lib.cy_server_poll(self.handle, int(wait_ms), ctypes.byref(rid), ctypes.byref(st), self._buf,
                                         len(self._buf), ctypes.byref(n), ctypes.byref(lat))
            if rc == -2:
                self._buf = ctypes.create_string_buffer(max(n.value, 2 * len(self._buf)))
                continue
            if rc == 1:
                return None
            if rc != 0:
                raise RuntimeError(f"cy_server_poll failed with status {rc}")
            return Result(rid.value, st.value, self._buf.raw[: n.value], lat.value)

    def stats(self) -> Dict[str, int]:
        arr = (ctypes.c_longlong * len(STAT_NAMES))()
        k = self.lib.cy_server_stats(self.handle, arr, len(STAT_NAMES))
        return {STAT_NAMES[i]: int(arr[i]) for i in range(k)}

    def close(self) -> None:
        if self.handle:
            self.lib.cy_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_poisson(server: Server, traces: Sequence[bytes], rate: float, seed: int = 0,
                keep_results: bool = False) -> dict:
    """Submit `traces` with exponential inter-arrival times of mean 1/rate
    (seconds) from a driver thread, collect every result, and return the
    latency percentiles (ms, submission to completion) and throughput."""
    from . import trace as T
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(traces))
    pixels = {}
    results: Dict[int, Result] = {}
    order: List[int] = []
    t_first = [0.0]

    def drive():
        t = time.perf_counter()
        t_first[0] = t
        due = t
        for tb, g in zip(traces, gaps):
            due += g
            while time.perf_counter() < due:
                pass
            rid = server.submit(tb)
            w, h = T.canvas_size(tb)
            pixels[rid] = w * h
            order.append(rid)

    driver = threading.Thread(target=drive)
    driver.start()
    lat = []
    failed = 0
    while len(lat) < len(traces):
        r = server.poll(1000)
        if r is None:
            continue
        lat.append(r.latency_ms)
        failed += r.status != 0
        if keep_results:
            results[r.id] = r
    t_end = time.perf_counter()
    driver.join()
    lat_a = np.asarray(lat)
    total_px = sum(pixels.values())
    out = {
        "rate_req_s": rate,
        "requests": len(traces),
        "offered_s": round(float(gaps.sum()), 4),
        "p50_ms": round(float(np.percentile(lat_a, 50)), 3),
        "p99_ms": round(float(np.percentile(lat_a, 99)), 3),
        "mean_ms": round(float(lat_a.mean()), 3),
        "mpix_s": round(total_px / (t_end - t_first[0]) / 1e6, 2),
        "failed": failed,
    }
    if keep_results:
        out["results"] = [results[i] for i in order]
    return out


def run_steady(server: Server, pool: Sequence[bytes], rate: float, duration_s: float = 5.0, seed: int = 0,
               max_backlog: int = 2000) -> dict:
    """Offer requests (cycling through `pool`) with exponential inter-arrival
    times of mean 1/rate for `duration_s` seconds of arrivals, and measure
    the server at that load: latency percentiles (ms, submission to
    completion) of every request, and the rate it actually completed them
    at.  A server that cannot keep up builds a backlog; once `max_backlog`
    requests wait unanswered, arrivals stop early (the run is then marked
    saturated, and its completion rate is the server's capacity)."""
    from . import trace as T
    rng = np.random.default_rng(seed)
    n_max = max(1, int(rate * duration_s))
    gaps = rng.exponential(1.0 / rate, size=n_max)
    picks = rng.integers(0, len(pool), size=n_max)
    px_of = [T.canvas_size(tb)[0] * T.canvas_size(tb)[1] for tb in pool]
    submitted = [0]
    stopped_early = [False]
    done_count = [0]
    lock = threading.Lock()
    t0 = [0.0]

    def drive():
        t = time.perf_counter()
        t0[0] = t
        due = t
        for i in range(n_max):
            due += gaps[i]
            while time.perf_counter() < due:
                pass
            with lock:
                if submitted[0] - done_count[0] >= max_backlog:
                    stopped_early[0] = True
                    break
            server.submit(pool[picks[i]])
            with lock:
                submitted[0] += 1

    driver = threading.Thread(target=drive)
    driver.start()
    lat, failed, px = [], 0, 0
    t_last = 0.0
    while True:
        with lock:
            finished_all = not driver.is_alive() and done_count[0] >= submitted[0]
        if finished_all:
            break
        r = server.poll(200)
        if r is None:
            continue
        lat.append(r.latency_ms)
        failed += r.status != 0
        t_last = time.perf_counter()
        with lock:
            done_count[0] += 1
    driver.join()
    n = len(lat)
    lat_a = np.asarray(lat) if n else np.zeros(1)
    span = max(t_last - t0[0], 1e-9)
    mean_px = float(np.mean([px_of[i] for i in picks[:n]])) if n else 0.0
    return {
        "offered_req_s": rate,
        "requests": n,
        "offered_for_s": round(float(gaps[:n].sum()), 3),
        "achieved_req_s": round(n / span, 1),
        "saturated": bool(stopped_early[0]),
        "p50_ms": round(float(np.percentile(lat_a, 50)), 3),
        "p99_ms": round(float(np.percentile(lat_a, 99)), 3),
        "mean_ms": round(float(lat_a.mean()), 3),
        "mpix_s": round(n * mean_px / span / 1e6, 2),
        "failed": failed,
    }
