"""ctypes binding of libcanvas_ity_gb300.so (the C ABI in include/).

Loading never falls back to anything else: if the CUDA library has not been
built, every call raises.  Build it with ``canvas_ity_gb300.build.build()``.
"""
from __future__ import annotations

import ctypes
import os
import time
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


def set_coverage(exact: bool) -> None:
    """Coverage of the tile engine's draws for frames prepared afterwards:
    binned fixed-point accumulation (False, the default; within the parity
    tolerance) or the exact row-sorted runs (True; the float canvas is the
    reference's bit for bit).  Applies to the whole process."""
    lib = load()
    lib.cy_set_coverage.restype = None
    lib.cy_set_coverage.argtypes = [ctypes.c_int]
    lib.cy_set_coverage(1 if exact else 0)


def coverage_exact() -> bool:
    lib = load()
    lib.cy_get_coverage.restype = ctypes.c_int
    lib.cy_get_coverage.argtypes = []
    return bool(lib.cy_get_coverage())


def set_device_stroke(on: bool) -> None:
    """Expand strokes on the GPU (True, the default) or on the host with the
    reference's own acosf/tanf (False); applies to the whole process."""
    lib = load()
    lib.cy_set_device_stroke.restype = None
    lib.cy_set_device_stroke.argtypes = [ctypes.c_int]
    lib.cy_set_device_stroke(1 if on else 0)


def device_stroke() -> bool:
    lib = load()
    lib.cy_device_stroke.restype = ctypes.c_int
    lib.cy_device_stroke.argtypes = []
    return bool(lib.cy_device_stroke())


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
        if rc == -2 and (n_img.value > cap or n_res.value > rcap):
            # the outputs did not fit: retry with the sizes reported
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


# ------------------------------------------------------------ batched frames
def _batch_lib() -> ctypes.CDLL:
    lib = load()
    if getattr(lib, "_batch_ready", False):
        return lib
    vp, c_int_p, c_size_p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)
    lib.cy_canvas_from_trace.restype = vp
    lib.cy_canvas_from_trace.argtypes = [vp, ctypes.c_size_t, c_int_p]
    lib.cy_canvas_ctx.restype = vp
    lib.cy_canvas_ctx.argtypes = [vp]
    lib.cy_canvas_delete.restype = None
    lib.cy_canvas_delete.argtypes = [vp]
    lib.cy_frame_create.restype = ctypes.c_int
    lib.cy_frame_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    for name in ("cy_frame_run", "cy_frame_sync", "cy_frame_finish", "cy_frame_capture"):
        getattr(lib, name).restype = ctypes.c_int
        getattr(lib, name).argtypes = [vp]
    lib.cy_frame_destroy.restype = None
    lib.cy_frame_destroy.argtypes = [vp]
    lib.cy_frame_stream.restype = vp
    lib.cy_frame_stream.argtypes = [vp]
    lib.cy_ctx_take_reads.restype = ctypes.c_int
    lib.cy_ctx_take_reads.argtypes = [vp, vp, ctypes.c_size_t, c_size_p]
    lib.cy_set_strip_config.restype = None
    lib.cy_set_strip_config.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.cy_frame_set_profiling.restype = ctypes.c_int
    lib.cy_frame_set_profiling.argtypes = [vp, ctypes.c_int]
    lib.cy_frame_profile.restype = ctypes.c_int
    lib.cy_frame_profile.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
    lib.cy_frame_collect.restype = ctypes.c_int
    lib.cy_frame_collect.argtypes = [vp, vp, ctypes.c_size_t, c_size_p]
    lib.cy_frame_autotune.restype = ctypes.c_int
    lib.cy_frame_autotune.argtypes = [vp, c_int_p, c_int_p, ctypes.POINTER(ctypes.c_float)]
    lib.cy_canvases_from_traces.restype = ctypes.c_int
    lib.cy_canvases_from_traces.argtypes = [ctypes.POINTER(vp), c_size_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.POINTER(vp)]
    lib.cy_frame_stats.restype = ctypes.c_int
    lib.cy_frame_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
    lib._batch_ready = True
    return lib


def set_strip_config(strip_pixels: int, threads: int) -> None:
    _batch_lib().cy_set_strip_config(int(strip_pixels), int(threads))


class Frame:
    """Many canvases rendered together: each call list is replayed on the
    host into a canvas whose reads are deferred, then one frame renders all
    of them (engine 0: persistent strip kernel; 1: per-draw launches)."""

    def __init__(self, traces, engine: int = 0, threads: int = 0):
        self.lib = _batch_lib()
        self.canvases = []
        self.frame = ctypes.c_void_p()
        try:
            n = len(traces)
            bufs = (ctypes.c_void_p * n)(*[ctypes.cast(ctypes.c_char_p(t), ctypes.c_void_p).value
                                           for t in traces])
            lens = (ctypes.c_size_t * n)(*[len(t) for t in traces])
            out = (ctypes.c_void_p * n)()
            t0 = time.perf_counter()
            rc = self.lib.cy_canvases_from_traces(bufs, lens, n, int(engine), int(threads), out)
            if rc != 0:
                raise RuntimeError(f"replay into deferred canvases failed with status {rc}")
            self.canvases = [out[i] for i in range(n)]
            t1 = time.perf_counter()
            ctxs = (ctypes.c_void_p * len(self.canvases))(*[self.lib.cy_canvas_ctx(c) for c in self.canvases])
            rc = self.lib.cy_frame_create(ctxs, len(self.canvases), int(engine), ctypes.byref(self.frame))
            if rc != 0:
                raise RuntimeError(f"cy_frame_create failed with status {rc}")
            # host seconds: replaying the call lists, building + first run of the frame
            self.timing = {"replay_s": t1 - t0, "create_s": time.perf_counter() - t1}
            self.ctxs = [ctxs[i] for i in range(len(self.canvases))]
        except Exception:
            self.close()
            raise

    def run(self) -> None:
        rc = self.lib.cy_frame_run(self.frame)
        if rc != 0:
            raise RuntimeError(f"cy_frame_run failed with status {rc}")

    def autotune(self) -> dict:
        """Pick the fastest strip size / block size for this frame's paint
        stage; it also becomes the process's strip configuration."""
        p, t, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_float(0.0)
        rc = self.lib.cy_frame_autotune(self.frame, ctypes.byref(p), ctypes.byref(t), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError(f"cy_frame_autotune failed with status {rc}")
        return {"strip_pixels": p.value, "threads": t.value, "paint_ms": round(ms.value, 3)}

    def capture(self) -> None:
        """Capture a device-only run into a CUDA graph; later runs launch it."""
        rc = self.lib.cy_frame_capture(self.frame)
        if rc != 0:
            raise RuntimeError(f"cy_frame_capture failed with status {rc}")

    def sync(self) -> None:
        rc = self.lib.cy_frame_sync(self.frame)
        if rc != 0:
            raise RuntimeError(f"cy_frame_sync failed with status {rc}")

    def stream(self) -> int:
        return int(self.lib.cy_frame_stream(self.frame) or 0)

    STAT_NAMES = ("pixels", "commands", "segments", "runs", "rows", "draw_runs", "draw_rows",
                  "shadow_floats", "read_bytes", "upload_bytes", "launches", "shadows", "clips",
                  "bin_entries", "binned")

    def stats(self) -> dict:
        arr = (ctypes.c_longlong * len(self.STAT_NAMES))()
        n = self.lib.cy_frame_stats(self.frame, arr, len(self.STAT_NAMES))
        return {k: int(arr[i]) for i, k in enumerate(self.STAT_NAMES[:n])}

    PHASES = ("flatten_stroke", "scan_convert", "masks_shadows", "paint")

    def set_profiling(self, on: bool) -> None:
        self.lib.cy_frame_set_profiling(self.frame, 1 if on else 0)

    def profile(self) -> dict:
        arr = (ctypes.c_float * 8)()
        n = self.lib.cy_frame_profile(self.frame, arr, 8)
        return {self.PHASES[i]: float(arr[i]) for i in range(min(n, len(self.PHASES)))}

    def finish(self, copy: bool = True) -> list:
        """Copy the reads back; returns each canvas's get_image_data bytes.
        With copy=False they are memoryviews into the frame's pinned
        read-back buffer (no host copy), valid until the frame is closed."""
        if not copy:
            return self._finish_views()
        t0 = time.perf_counter()
        rc = self.lib.cy_frame_finish(self.frame)
        if rc != 0:
            raise RuntimeError(f"cy_frame_finish failed with status {rc}")
        t1 = time.perf_counter()
        n = len(self.ctxs)
        offs = (ctypes.c_size_t * (n + 1))()
        rc = self.lib.cy_frame_collect(self.frame, None, 0, offs)
        total = offs[n]
        buf = bytearray(total)
        if total:
            cbuf = (ctypes.c_char * total).from_buffer(buf)
            rc = self.lib.cy_frame_collect(self.frame, ctypes.addressof(cbuf), total, offs)
            if rc != 0:
                raise RuntimeError(f"cy_frame_collect failed with status {rc}")
            del cbuf
        mv = memoryview(buf)
        out = [mv[offs[i]:offs[i + 1]] for i in range(n)]
        if copy:
            out = [bytes(o) for o in out]
        self.timing["finish_s"] = t1 - t0
        self.timing["reads_s"] = time.perf_counter() - t1
        return out

    def _finish_views(self) -> list:
        t0 = time.perf_counter()
        n = len(self.ctxs)
        offs = (ctypes.c_size_t * (n + 1))()
        data = ctypes.c_void_p()
        self.lib.cy_frame_finish_views.restype = ctypes.c_int
        self.lib.cy_frame_finish_views.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                   ctypes.POINTER(ctypes.c_size_t)]
        rc = self.lib.cy_frame_finish_views(self.frame, ctypes.byref(data), offs)
        if rc != 0:
            raise RuntimeError(f"cy_frame_finish_views failed with status {rc}")
        t1 = time.perf_counter()
        total = offs[n]
        mv = memoryview((ctypes.c_ubyte * total).from_address(data.value)).cast("B") if total else memoryview(b"")
        out = [mv[offs[i]:offs[i + 1]] for i in range(n)]
        self.timing["finish_s"] = t1 - t0
        self.timing["reads_s"] = time.perf_counter() - t1
        return out

    def close(self) -> None:
        if self.frame:
            self.lib.cy_frame_destroy(self.frame)
            self.frame = ctypes.c_void_p()
        for c in self.canvases:
            self.lib.cy_canvas_delete(c)
        self.canvases = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def points_in_path(trace: bytes, queries) -> np.ndarray:
    """Replay a call list into a canvas, then test (x, y) query points
    against its current path on the GPU (cy_canvas_points_in_path, the
    batched is_point_in_path).  Returns a uint8 array of 0/1."""
    lib = _batch_lib()
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 2)
    st = ctypes.c_int(0)
    c = lib.cy_canvas_from_trace(ctypes.cast(ctypes.c_char_p(trace), ctypes.c_void_p), len(trace), ctypes.byref(st))
    if not c:
        raise RuntimeError(f"replay failed with status {st.value}")
    try:
        fn = lib.cy_canvas_points_in_path
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        out = np.zeros(len(q), np.uint8)
        rc = fn(c, q.ctypes.data, len(q), out.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"cy_canvas_points_in_path failed with status {rc}")
        return out
    finally:
        lib.cy_canvas_delete(c)


TGA, PNG = 0, 1


def encode_image(trace: bytes, fmt: int, x: int, y: int, w: int, h: int) -> bytes:
    """Replay a call list into a canvas, then pack the w x h rectangle at
    (x, y) into a TGA or PNG file on the GPU (cy_encode_image)."""
    lib = _batch_lib()
    st = ctypes.c_int(0)
    c = lib.cy_canvas_from_trace(ctypes.cast(ctypes.c_char_p(trace), ctypes.c_void_p), len(trace), ctypes.byref(st))
    if not c:
        raise RuntimeError(f"replay failed with status {st.value}")
    try:
        fn = lib.cy_encode_image
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                       ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        size = ctypes.c_size_t(0)
        ctx = lib.cy_canvas_ctx(c)
        fn(ctx, int(fmt), int(x), int(y), int(w), int(h), None, 0, ctypes.byref(size))
        buf = ctypes.create_string_buffer(max(size.value, 1))
        rc = fn(ctx, int(fmt), int(x), int(y), int(w), int(h), buf, size.value, ctypes.byref(size))
        if rc != 0:
            raise RuntimeError(f"cy_encode_image failed with status {rc}")
        return buf.raw[: size.value]
    finally:
        lib.cy_canvas_delete(c)


def render_traces(traces, engine: int = 0, frame_pixels: int = 0, out=None, offsets=None):
    """End to end through cy_render_traces: call lists in host memory to
    RGBA8 reads in host memory, frames pipelined (host work of one frame
    under the device work of the previous).  `out` (a writable buffer) and
    `offsets` (n + 1 entries) can be given to reuse them; returns
    (per-canvas memoryviews into out, stats dict)."""
    from . import trace as T
    lib = _batch_lib()
    lib.cy_render_traces.restype = ctypes.c_int
    lib.cy_render_traces.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
    n = len(traces)
    if offsets is None:
        offsets = np.zeros(n + 1, np.uint64)
        offsets[1:] = np.cumsum([T.read_bytes(t) for t in traces], dtype=np.uint64)
    total = int(offsets[n])
    if out is None:
        out = np.zeros(max(total, 1), np.uint8)
    bufs = (ctypes.c_void_p * n)(*[ctypes.cast(ctypes.c_char_p(t), ctypes.c_void_p).value for t in traces])
    lens = (ctypes.c_size_t * n)(*[len(t) for t in traces])
    offs = np.ascontiguousarray(offsets, np.uint64)
    stats = (ctypes.c_longlong * 3)()
    out_arr = np.frombuffer(out, np.uint8)
    rc = lib.cy_render_traces(bufs, lens, n, int(engine), int(frame_pixels), out_arr.ctypes.data,
                              offs.ctypes.data, stats)
    if rc != 0:
        raise RuntimeError(f"cy_render_traces failed with status {rc}")
    mv = memoryview(out_arr)
    views = [mv[int(offs[i]):int(offs[i + 1])] for i in range(n)]
    return views, {"frames": stats[0], "upload_bytes": stats[1], "read_bytes": stats[2]}


def render_batch(traces, engine: int = 0) -> List[bytes]:
    """Render call lists together; returns each one's get_image_data bytes."""
    with Frame(traces, engine) as f:
        return f.finish()
