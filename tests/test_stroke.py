"""Stroke expansion on the GPU (cy_stroke_path): dash_lines, add_half_stroke
and stroke_lines (src/canvas_ity.hpp:1858-2100) run as one thread per
subpath.

The GPU takes a round join's acos and tan in double precision rounded to
float where the reference calls libm's acosf/tanf.  The oracle built with
trig="cr" does the same, and pins the GPU's float canvas bit for bit; the
CPU tests here bound what the choice changes against the reference's own
trigonometry (RGBA8 identical on the reference's suite and the workload).
"""
import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import scenes
from canvas_ity_gb300 import trace as T
import golden_util as G

DASHES = [None, [6.0, 3.0], [4.0, 2.0, 1.0], [0.0, 5.0], [0.0, 0.0], [12.0, 0.5, 0.0, 3.0], [0.25, 0.25]]


def stroke_scene(seed: int, w: int = 224, h: int = 160) -> bytes:
    """Strokes of every join, cap and dash kind over curves, arcs, closed and
    open subpaths, zero-length segments, tight turns and skewed transforms."""
    rng = np.random.default_rng(7000 + seed)
    t = T.TraceWriter(w, h)
    for k in range(14):
        t.save()
        if rng.random() < 0.5:
            t.translate(float(rng.uniform(0, w)), float(rng.uniform(0, h)))
            t.rotate(float(rng.uniform(-3.2, 3.2)))
            t.transform(float(rng.uniform(0.4, 1.8)), float(rng.uniform(-0.4, 0.4)),
                        float(rng.uniform(-0.4, 0.4)), float(rng.uniform(0.4, 1.8)),
                        float(rng.uniform(-w / 2, 0)), float(rng.uniform(-h / 2, 0)))
        t.set_line_width(float(rng.choice([0.05, 0.6, 1.0, 2.5, 7.0, 19.0, 43.0])))
        t.set_line_join(int(rng.integers(0, 3)))
        t.set_line_cap(int(rng.integers(0, 3)))
        t.set_miter_limit(float(rng.choice([1.0, 2.0, 4.0, 10.0, 100.0])))
        dash = DASHES[int(rng.integers(0, len(DASHES)))]
        if dash is not None:
            t.set_line_dash(dash)
            t.set_line_dash_offset(float(rng.choice([0.0, 2.5, -7.25, 100.0, 13.0])))
        c = rng.uniform(0, 1, 4)
        t.set_color(T.STROKE_STYLE, float(c[0]), float(c[1]), float(c[2]), float(0.35 + 0.65 * c[3]))
        if k == 5:
            t.set_shadow_color(0.1, 0.1, 0.2, 0.8)
            t.set_shadow_blur(4.0)
            t.set_shadow_offset_x(3.0)
        if k == 9:
            t.set_global_composite_operation(T.DESTINATION_OVER)
        t.begin_path()
        for sub in range(int(rng.integers(1, 4))):
            p = rng.uniform((-20, -20), (w + 20, h + 20))
            t.move_to(*p)
            for _ in range(int(rng.integers(0, 7))):
                r = rng.random()
                q = rng.uniform((-20, -20), (w + 20, h + 20))
                if r < 0.3:
                    t.line_to(*q)
                elif r < 0.4:
                    t.line_to(*p)            # back to the start: a tight turn
                elif r < 0.5:
                    t.line_to(*q)
                    t.line_to(*q)            # zero-length segment
                elif r < 0.75:
                    c1 = q + rng.normal(0, 40, 2)
                    c2 = q + rng.normal(0, 40, 2)
                    e = rng.uniform((0, 0), (w, h))
                    t.bezier_curve_to(c1[0], c1[1], c2[0], c2[1], e[0], e[1])
                elif r < 0.85:
                    t.quadratic_curve_to(q[0], q[1], *rng.uniform((0, 0), (w, h)))
                else:
                    t.arc(q[0], q[1], float(rng.uniform(2, 40)), float(rng.uniform(0, 6.3)),
                          float(rng.uniform(0, 6.3)), bool(rng.random() < 0.5))
                p = q
            if rng.random() < 0.5:
                t.close_path()
        t.stroke()
        t.restore()
    t.get_image_data(w, h, 0, 0)
    return t.finish(read_back=False)


def test_cr_trig_keeps_reference_suite_bytes():
    """Round joins from correctly rounded acos/tan leave every get_image_data
    byte of the reference's own suite as the reference recorded it."""
    for entry in G.manifest():
        tb = G.load_fixture(entry)
        got = G.split_images(tb, oracle.replay(tb, ties="sign", trig="cr")[0])
        want = [img for _, _, img in T.parse(tb).expected_images()]
        for i, (g, w) in enumerate(zip(got, want)):
            assert np.array_equal(g, w), f"{entry['name']} read {i}"


@pytest.mark.parametrize("seed", range(4))
def test_cr_trig_close_to_libm_on_workload(seed):
    """On many-canvas workload canvases the two round-join choices give the
    same RGBA8 and differ in few float values."""
    tb = scenes.c3_canvas(40 + seed)
    w, h = T.canvas_size(tb)
    assert oracle.replay(tb, ties="sign", trig="cr")[0] == oracle.replay(tb, ties="sign")[0]
    a = oracle.replay_linear(tb, w, h, ties="sign")
    b = oracle.replay_linear(tb, w, h, ties="sign", trig="cr")
    assert (a != b).sum() <= 1e-4 * a.size


@pytest.mark.parametrize("seed", range(6))
def test_cr_trig_close_to_libm_on_stroke_scenes(seed):
    tb = stroke_scene(seed)
    a = G.split_images(tb, oracle.replay(tb, ties="sign")[0])[-1]
    b = G.split_images(tb, oracle.replay(tb, ties="sign", trig="cr")[0])[-1]
    maxd, frac = G.compare(a, b)
    assert maxd <= 1 and frac <= 0.005


@pytest.mark.gpu
@pytest.mark.parametrize("mode", sorted(G.MODES))
@pytest.mark.parametrize("seed", range(10))
def test_device_stroke_float_canvas_bit_exact(mode, seed):
    from canvas_ity_gb300 import native
    G.use_mode(mode)
    native.set_device_stroke(True)
    try:
        tb = stroke_scene(seed)
        w, h = T.canvas_size(tb)
        got = native.replay_linear(tb, w, h)
    finally:
        G.use_mode("tile")
    want = oracle.replay_linear(tb, w, h, ties="sign", trig="cr", coverage=G.oracle_coverage(mode))
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} float values differ, first at {bad[0].tolist()}"


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(10))
def test_device_stroke_rgba8_vs_reference_trig(seed):
    """Against the oracle with libm's round joins (the reference's own
    arithmetic): within one LSB, nearly every pixel identical."""
    from canvas_ity_gb300 import native
    native.set_engine(0)
    native.set_device_stroke(True)
    tb = stroke_scene(seed)
    got = G.split_images(tb, native.replay(tb)[0])[-1]
    want = G.split_images(tb, oracle.replay(tb, ties="sign")[0])[-1]
    G.assert_within_contract(got, want, f"stroke scene {seed}")


@pytest.mark.gpu
def test_device_and_host_stroke_agree_on_workload():
    """A frame of workload canvases: strokes expanded on the GPU and on the
    host give the same RGBA8."""
    from canvas_ity_gb300 import native
    traces = [scenes.c3_canvas(60 + s) for s in range(6)]
    native.set_device_stroke(True)
    dev = native.render_batch(traces, 0)
    native.set_device_stroke(False)
    try:
        host = native.render_batch(traces, 0)
    finally:
        native.set_device_stroke(True)
    assert dev == host


@pytest.mark.gpu
def test_dash_too_fine_fails_cleanly():
    """A pattern that would dash one subpath into more than 2^22 points makes
    the canvas report CY_ENOMEM (the reference would not finish); the
    context stays usable for reading its status."""
    import ctypes
    from canvas_ity_gb300 import native
    native.set_device_stroke(True)
    t = T.TraceWriter(64, 64)
    t.set_line_dash([1.0e-5, 1.0e-5])   # about 2.3e7 dashed points
    t.begin_path()
    t.move_to(0, 0)
    t.line_to(60, 60)
    t.line_to(0, 60)
    t.line_to(60, 0)
    t.stroke()
    t.get_image_data(64, 64, 0, 0)
    tb = t.finish(read_back=False)
    with pytest.raises(RuntimeError, match="status -2"):
        native.replay(tb)
