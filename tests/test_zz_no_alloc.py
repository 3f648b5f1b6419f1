"""cy_get_image_noalloc: get_image_data without any allocation.

Some callers cannot allocate GPU memory when they read pixels back: a serving
loop that admits work against a fixed HBM budget, or a program whose device
memory is reserved by another framework's pool, and any latency-bound path
where cudaMalloc/cudaFree would make the device synchronise.  This entry point
stages the RGBA8 conversion in one fixed device array of the library instead.

This file is named so that pytest collects it last: if it fails, a run that
stops at the first failure has already run every other test.  It must pass on
its own in a fresh process as well as after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

from canvas_ity_gb300 import native
import golden_util as G

pytestmark = pytest.mark.gpu

MAX_LSB = 1            # the parity tolerance of the other GPU tests
MIN_IDENTICAL = 0.995
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


def _draw(lib, cv, w, h):
    """A few draws: a shadowed gradient cubic, a translucent stroke."""
    lib.cy_canvas_set_linear_gradient(cv, 0, 0.0, 0.0, float(w), float(h))
    lib.cy_canvas_add_color_stop(cv, 0, 0.0, 0.9, 0.2, 0.1, 1.0)
    lib.cy_canvas_add_color_stop(cv, 0, 1.0, 0.1, 0.3, 0.9, 0.6)
    lib.cy_canvas_set_shadow_color(cv, 0.0, 0.0, 0.0, 0.5)
    lib.cy_canvas_set_shadow_blur(cv, 6.0)
    lib.cy_canvas_set_shadow_offset_x(cv, 4.0)
    lib.cy_canvas_begin_path(cv)
    lib.cy_canvas_move_to(cv, 0.1 * w, 0.2 * h)
    lib.cy_canvas_bezier_curve_to(cv, 0.9 * w, -0.1 * h, 1.1 * w, 0.9 * h, 0.3 * w, 0.8 * h)
    lib.cy_canvas_line_to(cv, 0.05 * w, 0.95 * h)
    lib.cy_canvas_close_path(cv)
    lib.cy_canvas_fill(cv)
    lib.cy_canvas_set_shadow_color(cv, 0.0, 0.0, 0.0, 0.0)
    lib.cy_canvas_set_color(cv, 1, 0.2, 0.7, 0.3, 0.8)
    lib.cy_canvas_set_line_width(cv, 3.5)
    lib.cy_canvas_stroke(cv)


def _read(fn, ctx, w, h, x, y):
    stride = w * 4 + 12   # padded rows: the stride is honoured
    buf = (ctypes.c_ubyte * (stride * h))()
    rc = fn(ctx, buf, w, h, stride, x, y)
    img = np.frombuffer(buf, np.uint8).reshape(h, stride)[:, : w * 4].reshape(h, w, 4).copy()
    return rc, img


@pytest.mark.parametrize("engine", [0, 1], ids=["tile", "plain"])
def test_no_alloc_readback_matches_get_image(engine):
    lib = _lib()
    native.set_engine(engine)
    w, h = 300, 200
    cv = lib.cy_canvas_new(w, h)
    assert cv
    try:
        _draw(lib, cv, w, h)
        ctx = lib.cy_canvas_ctx(cv)
        assert lib.cy_flush(ctx) == 0
        # Two calls in a row: the whole canvas, then a rectangle hanging off
        # the top-left corner (pixels outside the canvas read as zero).
        for (rw, rh, rx, ry) in ((w, h, 0, 0), (170, 90, -13, -7)):
            rc_a, want = _read(lib.cy_get_image, ctx, rw, rh, rx, ry)
            rc_b, got = _read(lib.cy_get_image_noalloc, ctx, rw, rh, rx, ry)
            assert rc_a == 0 and rc_b == 0
            maxd, frac = G.compare(got, want)
            assert maxd <= MAX_LSB and frac <= 1.0 - MIN_IDENTICAL, (rw, rh, rx, ry, maxd, frac)
            assert got.any()
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
