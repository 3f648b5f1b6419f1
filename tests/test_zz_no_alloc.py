"""cy_get_image_noalloc: get_image_data without any allocation.

Some callers cannot allocate GPU memory when they read pixels back: a serving
loop that admits work against a fixed HBM budget, or a program whose device
memory is reserved by another framework's pool, and any latency-bound path
where cudaMalloc/cudaFree would make the device synchronise.  This entry point
stages the RGBA8 conversion in one fixed device array of the library instead.

It runs the same conversion kernel as cy_get_image, so its bytes must equal
cy_get_image's exactly; both must also equal the CPU oracle's get_image_data
of the same calls (the oracle variant that computes what the render mode
computes, itself held to the reference by the other tests).

This file is named so that pytest collects it last: if it fails, a run that
stops at the first failure has already run every other test.  It must pass on
its own in a fresh process as well as after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import native
from canvas_ity_gb300 import trace as T
import golden_util as G

pytestmark = pytest.mark.gpu

CY_EINVAL = -1
MAX_PIXELS = 1024 * 1024   # CY_GET_IMAGE_NOALLOC_MAX_PIXELS in include/cy_gpu.h


def _lib():
    lib = native.load()
    P, F, I = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    sigs = {
        "cy_canvas_new": (P, [I, I]),
        "cy_canvas_delete": (None, [P]),
        "cy_canvas_ctx": (P, [P]),
        "cy_canvas_set_color": (None, [P, I, F, F, F, F]),
        "cy_canvas_set_shadow_color": (None, [P, F, F, F, F]),
        "cy_canvas_set_shadow_blur": (None, [P, F]),
        "cy_canvas_set_shadow_offset_x": (None, [P, F]),
        "cy_canvas_set_global_alpha": (None, [P, F]),
        "cy_canvas_set_linear_gradient": (None, [P, I, F, F, F, F]),
        "cy_canvas_add_color_stop": (None, [P, I, F, F, F, F, F]),
        "cy_canvas_begin_path": (None, [P]),
        "cy_canvas_move_to": (None, [P, F, F]),
        "cy_canvas_line_to": (None, [P, F, F]),
        "cy_canvas_bezier_curve_to": (None, [P, F, F, F, F, F, F]),
        "cy_canvas_close_path": (None, [P]),
        "cy_canvas_fill": (None, [P]),
        "cy_canvas_set_line_width": (None, [P, F]),
        "cy_canvas_stroke": (None, [P]),
        "cy_canvas_fill_rectangle": (None, [P, F, F, F, F]),
        "cy_flush": (I, [P]),
        "cy_get_image": (I, [P, P, I, I, I, I, I]),
        "cy_get_image_noalloc": (I, [P, P, I, I, I, I, I]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def _scene(w, h):
    """A shadowed gradient cubic and a translucent stroke, as (method, args)
    calls that the C binding and the call-list writer both take."""
    return [
        ("set_linear_gradient", (0, 0.0, 0.0, float(w), float(h))),
        ("add_color_stop", (0, 0.0, 0.9, 0.2, 0.1, 1.0)),
        ("add_color_stop", (0, 1.0, 0.1, 0.3, 0.9, 0.6)),
        ("set_shadow_color", (0.0, 0.0, 0.0, 0.5)),
        ("set_shadow_blur", (6.0,)),
        ("set_shadow_offset_x", (4.0,)),
        ("begin_path", ()),
        ("move_to", (0.1 * w, 0.2 * h)),
        ("bezier_curve_to", (0.9 * w, -0.1 * h, 1.1 * w, 0.9 * h, 0.3 * w, 0.8 * h)),
        ("line_to", (0.05 * w, 0.95 * h)),
        ("close_path", ()),
        ("fill", ()),
        ("set_shadow_color", (0.0, 0.0, 0.0, 0.0)),
        ("set_color", (1, 0.2, 0.7, 0.3, 0.8)),
        ("set_line_width", (3.5,)),
        ("stroke", ()),
    ]


def _draw(lib, cv, calls):
    for name, args in calls:
        getattr(lib, "cy_canvas_" + name)(cv, *args)


def _oracle_read(w, h, calls, reads, mode="tile"):
    """The oracle's get_image_data of each (rw, rh, rx, ry) after `calls`,
    from the oracle variant that computes what the mode computes (strokes
    expanded on the GPU round their joins' acos/tan from double)."""
    tw = T.TraceWriter(w, h)
    for name, args in calls:
        getattr(tw, name)(*args)
    for rw, rh, rx, ry in reads:
        tw.get_image_data(rw, rh, rx, ry)
    raw = oracle.replay(tw.finish(read_back=False), ties="sign", trig="cr", coverage=G.oracle_coverage(mode))[0]
    out, at = [], 0
    for rw, rh, _, _ in reads:
        n = rw * rh * 4
        out.append(np.frombuffer(raw[at:at + n], np.uint8).reshape(rh, rw, 4))
        at += n
    return out


def _read(fn, ctx, w, h, x, y):
    stride = w * 4 + 12   # padded rows: the stride is honoured
    buf = (ctypes.c_ubyte * (stride * h))()
    rc = fn(ctx, buf, w, h, stride, x, y)
    img = np.frombuffer(buf, np.uint8).reshape(h, stride)[:, : w * 4].reshape(h, w, 4).copy()
    return rc, img


def _free_bytes():
    import torch
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("mode", ["tile", "plain"])
def test_no_alloc_readback_matches_get_image(mode):
    lib = _lib()
    G.use_mode(mode)
    w, h = 300, 200
    cv = lib.cy_canvas_new(w, h)
    assert cv
    # Two calls in a row: the whole canvas, then a rectangle hanging off the
    # top-left corner (pixels outside the canvas read as zero).
    reads = ((w, h, 0, 0), (170, 90, -13, -7))
    calls = _scene(w, h)
    try:
        _draw(lib, cv, calls)
        ctx = lib.cy_canvas_ctx(cv)
        assert lib.cy_flush(ctx) == 0
        for (rw, rh, rx, ry), ref in zip(reads, _oracle_read(w, h, calls, reads, mode)):
            rc_a, want = _read(lib.cy_get_image, ctx, rw, rh, rx, ry)
            rc_b, got = _read(lib.cy_get_image_noalloc, ctx, rw, rh, rx, ry)
            assert rc_a == 0 and rc_b == 0
            # the same conversion kernel on the same canvas: identical bytes,
            # and those of the oracle restating this coverage
            assert np.array_equal(got, want), (rw, rh, rx, ry)
            assert np.array_equal(got, ref), (rw, rh, rx, ry)
            assert got.any()
    finally:
        lib.cy_canvas_delete(cv)
        G.use_mode("tile")


def test_no_alloc_readback_full_size_and_never_painted():
    """A read of exactly the largest size the array holds, from a canvas of
    that size, and reads of a canvas that was never painted."""
    lib = _lib()
    G.use_mode("tile")
    side = 1024
    assert side * side == MAX_PIXELS
    cv = lib.cy_canvas_new(side, side)
    blank = lib.cy_canvas_new(64, 48)
    assert cv and blank
    calls = _scene(side, side)
    try:
        # never painted: all zero, as the oracle says
        bctx = lib.cy_canvas_ctx(blank)
        assert lib.cy_flush(bctx) == 0
        rc, got = _read(lib.cy_get_image_noalloc, bctx, 64, 48, 0, 0)
        assert rc == 0 and not got.any()
        want = _oracle_read(64, 48, [], [(64, 48, 0, 0)])[0]
        assert np.array_equal(got, want)
        # the full 1024 x 1024 rectangle
        _draw(lib, cv, calls)
        ctx = lib.cy_canvas_ctx(cv)
        assert lib.cy_flush(ctx) == 0
        ref = _oracle_read(side, side, calls, [(side, side, 0, 0)])[0]
        for _ in range(2):
            rc_a, want = _read(lib.cy_get_image, ctx, side, side, 0, 0)
            rc_b, got = _read(lib.cy_get_image_noalloc, ctx, side, side, 0, 0)
            assert rc_a == 0 and rc_b == 0
            assert np.array_equal(got, want)
            assert np.array_equal(got, ref)
    finally:
        lib.cy_canvas_delete(cv)
        lib.cy_canvas_delete(blank)


def test_no_alloc_readback_allocates_nothing():
    """After a first call, repeated calls leave the device's free memory
    exactly as it was: no allocation by the call or by anything it calls."""
    lib = _lib()
    native.set_engine(0)
    w, h = 512, 384
    cv = lib.cy_canvas_new(w, h)
    assert cv
    try:
        _draw(lib, cv, _scene(w, h))
        ctx = lib.cy_canvas_ctx(cv)
        assert lib.cy_flush(ctx) == 0
        stride = w * 4
        buf = (ctypes.c_ubyte * (stride * h))()
        assert lib.cy_get_image_noalloc(ctx, buf, w, h, stride, 0, 0) == 0
        before = _free_bytes()
        for i in range(20):
            assert lib.cy_get_image_noalloc(ctx, buf, w - i, h - i, stride, i, i) == 0
        assert _free_bytes() == before
    finally:
        lib.cy_canvas_delete(cv)


def test_no_alloc_readback_rejects_what_it_cannot_do():
    lib = _lib()
    native.set_engine(0)
    cv = lib.cy_canvas_new(64, 64)
    try:
        ctx = lib.cy_canvas_ctx(cv)
        assert lib.cy_flush(ctx) == 0
        buf = (ctypes.c_ubyte * 16)()
        # larger than the fixed array
        assert lib.cy_get_image_noalloc(ctx, buf, 1025, 1024, 1025 * 4, 0, 0) == CY_EINVAL
        # stride shorter than a row
        assert lib.cy_get_image_noalloc(ctx, buf, 2, 2, 7, 0, 0) == CY_EINVAL
        # queued draws need a flush (which may allocate) first
        lib.cy_canvas_set_color(cv, 0, 1.0, 0.0, 0.0, 1.0)
        lib.cy_canvas_fill_rectangle(cv, 1.0, 1.0, 10.0, 10.0)
        assert lib.cy_get_image_noalloc(ctx, buf, 2, 2, 8, 0, 0) == CY_EINVAL
        assert lib.cy_flush(ctx) == 0
        assert lib.cy_get_image_noalloc(ctx, buf, 2, 2, 8, 2, 2) == 0
        assert bytes(buf[:4]) == bytes([255, 0, 0, 255])
    finally:
        lib.cy_canvas_delete(cv)
