"""Seeded synthetic scenes for the five benchmark configurations.

The scenes are call lists (see `trace.py`) replayed identically by the GB300
canvas, the CPU oracle and the reference.  Each canvas is drawn from
``numpy.random.Generator(PCG64(base_seed + canvas_index))`` so any canvas of a
batch can be regenerated on its own.

Configurations (sizes and distributions as specified for the benchmark):

* ``c0`` 512x512: 64 closed polygons of 3-32 vertices uniform over the
  canvas, nonzero fill, solid colour (RGB U[0,1], alpha U[0.3,1]),
  source-over, identity transform.
* ``c1`` 1024x1024: 240 paths of 4-40 cubic Beziers; anchors uniform over the
  canvas, control points = anchor + N(0, 40 px).  Even paths filled, odd
  paths stroked (width U[0.5,6]; joins cycle miter/round/bevel, caps cycle
  butt/round/square; a 2-entry dash U[2,20] on 25% of strokes).  A global
  transform scales by 1.8 and rotates by 17 degrees about the canvas centre.
* ``c2`` 2048x2048: 500 paths as in c1, each painted with a linear or radial
  gradient of 2-8 uniform stops or a 64x64 uniform random RGBA8 pattern
  (repeat); composite operations cycle through all 11 per path, global alpha
  U[0.2,1], one random 16-vertex clip polygon first, and 20% of paths cast a
  shadow (blur U[0,16], offset N(0, 8 px)).
* ``c3`` batch: 4096 canvases, each side log-uniform in [64,1024], 8-128
  paths per canvas drawn from the c0/c1/c2 path kinds at 60/30/10 (control
  point spread scaled by side/1024, transform about the canvas centre).
* ``c4`` serving: requests with sides log-uniform in [32,2048] and 1-512
  paths from the same mixture.
"""
from __future__ import annotations

import math
from typing import List, Optional

import numpy as np

from . import trace as T

BASE_SEED = 20261203
_JOINS = (T.MITER, T.ROUNDED, T.BEVEL)
_CAPS = (T.BUTT, T.CIRCLE, T.SQUARE)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _polygon(t: T.TraceWriter, pts: np.ndarray) -> None:
    t.begin_path()
    t.move_to(pts[0, 0], pts[0, 1])
    for x, y in pts[1:]:
        t.line_to(x, y)
    t.close_path()


def _cubic_path(t: T.TraceWriter, rng, w: int, h: int, n: int, spread: float) -> None:
    anchors = rng.uniform((0.0, 0.0), (w, h), size=(n + 1, 2))
    c1 = anchors[:-1] + rng.normal(0.0, spread, size=(n, 2))
    c2 = anchors[1:] + rng.normal(0.0, spread, size=(n, 2))
    t.begin_path()
    t.move_to(anchors[0, 0], anchors[0, 1])
    for i in range(n):
        t.bezier_curve_to(c1[i, 0], c1[i, 1], c2[i, 0], c2[i, 1], anchors[i + 1, 0], anchors[i + 1, 1])


def _solid(t: T.TraceWriter, rng, style: int) -> None:
    r, g, b = rng.uniform(0.0, 1.0, 3)
    t.set_color(style, r, g, b, rng.uniform(0.3, 1.0))


def _global_transform(t: T.TraceWriter, w: int, h: int) -> None:
    t.translate(w * 0.5, h * 0.5)
    t.rotate(math.radians(17.0))
    t.scale(1.8, 1.8)
    t.translate(-w * 0.5, -h * 0.5)


def _stroke_style(t: T.TraceWriter, rng, k: int) -> None:
    t.set_line_width(rng.uniform(0.5, 6.0))
    t.set_line_join(_JOINS[k % 3])
    t.set_line_cap(_CAPS[k % 3])
    if rng.uniform() < 0.25:
        t.set_line_dash([rng.uniform(2.0, 20.0), rng.uniform(2.0, 20.0)])
    else:
        t.set_line_dash(None, 0)


def _fancy_paint(t: T.TraceWriter, rng, style: int, w: int, h: int) -> None:
    kind = rng.integers(0, 3)
    if kind == 2:
        img = rng.integers(0, 256, size=(64, 64, 4), dtype=np.uint8)
        t.set_pattern(style, img, 64, 64, T.REPEAT)
        return
    if kind == 0:
        x0, y0, x1, y1 = rng.uniform(0, 1, 4) * (w, h, w, h)
        t.set_linear_gradient(style, x0, y0, x1, y1)
    else:
        x0, y0, x1, y1 = rng.uniform(0, 1, 4) * (w, h, w, h)
        r0, r1 = rng.uniform(0.0, 0.5 * max(w, h), 2)
        t.set_radial_gradient(style, x0, y0, r0, x1, y1, r1)
    for _ in range(int(rng.integers(2, 9))):
        r, g, b, a = rng.uniform(0.0, 1.0, 4)
        t.add_color_stop(style, rng.uniform(0.0, 1.0), r, g, b, a)


def _c0_path(t, rng, w, h, k):
    n = int(rng.integers(3, 33))
    _solid(t, rng, T.FILL_STYLE)
    _polygon(t, rng.uniform((0.0, 0.0), (w, h), size=(n, 2)))
    t.fill()


def _c1_path(t, rng, w, h, k, spread, transformed=True):
    n = int(rng.integers(4, 41))
    if transformed:
        t.save()
        _global_transform(t, w, h)
    if k % 2 == 0:
        _solid(t, rng, T.FILL_STYLE)
        _cubic_path(t, rng, w, h, n, spread)
        t.fill()
    else:
        _solid(t, rng, T.STROKE_STYLE)
        _stroke_style(t, rng, k // 2)
        _cubic_path(t, rng, w, h, n, spread)
        t.stroke()
    if transformed:
        t.restore()


def _c2_path(t, rng, w, h, k, spread, transformed=True):
    n = int(rng.integers(4, 41))
    if transformed:
        t.save()
        _global_transform(t, w, h)
    stroked = k % 2 == 1
    style = T.STROKE_STYLE if stroked else T.FILL_STYLE
    _fancy_paint(t, rng, style, w, h)
    t.set_global_composite_operation(T.COMPOSITE_OPS[k % 11])
    t.set_global_alpha(rng.uniform(0.2, 1.0))
    shadow = rng.uniform() < 0.2
    if shadow:
        r, g, b = rng.uniform(0.0, 1.0, 3)
        t.set_shadow_color(r, g, b, rng.uniform(0.3, 1.0))
        t.set_shadow_blur(rng.uniform(0.0, 16.0))
        t.set_shadow_offset_x(rng.normal(0.0, 8.0))
        t.set_shadow_offset_y(rng.normal(0.0, 8.0))
    if stroked:
        _stroke_style(t, rng, k // 2)
    _cubic_path(t, rng, w, h, n, spread)
    if stroked:
        t.stroke()
    else:
        t.fill()
    if shadow:
        t.set_shadow_color(0.0, 0.0, 0.0, 0.0)
    if transformed:
        t.restore()


def _clip_polygon(t, rng, w, h, n=16):
    _polygon(t, rng.uniform((0.0, 0.0), (w, h), size=(n, 2)))
    t.clip()


def c0(seed: int = BASE_SEED, w: int = 512, h: int = 512, paths: int = 64) -> bytes:
    rng = _rng(seed)
    t = T.TraceWriter(w, h)
    for k in range(paths):
        _c0_path(t, rng, w, h, k)
    return t.finish()


def c1(seed: int = BASE_SEED, w: int = 1024, h: int = 1024, paths: int = 240) -> bytes:
    rng = _rng(seed)
    t = T.TraceWriter(w, h)
    _global_transform(t, w, h)
    for k in range(paths):
        _c1_path(t, rng, w, h, k, 40.0, transformed=False)
    return t.finish()


def c2(seed: int = BASE_SEED, w: int = 2048, h: int = 2048, paths: int = 500) -> bytes:
    rng = _rng(seed)
    t = T.TraceWriter(w, h)
    _clip_polygon(t, rng, w, h)
    _global_transform(t, w, h)
    for k in range(paths):
        _c2_path(t, rng, w, h, k, 40.0, transformed=False)
    return t.finish()


def mixed_canvas(seed: int, w: int, h: int, paths: int, clip: bool = False) -> bytes:
    """One canvas of the batched / serving mixture (60/30/10 of c0/c1/c2 paths)."""
    rng = _rng(seed)
    t = T.TraceWriter(w, h)
    spread = 40.0 * max(w, h) / 1024.0
    if clip:
        _clip_polygon(t, rng, w, h)
    for k in range(paths):
        u = rng.uniform()
        if u < 0.6:
            _c0_path(t, rng, w, h, k)
        elif u < 0.9:
            _c1_path(t, rng, w, h, k, spread)
        else:
            _c2_path(t, rng, w, h, k, spread)
    return t.finish()


def _log_uniform(rng, lo: float, hi: float) -> int:
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def c3_canvas(index: int, base_seed: int = BASE_SEED) -> bytes:
    rng = _rng(base_seed * 7 + index)
    w, h = _log_uniform(rng, 64, 1024), _log_uniform(rng, 64, 1024)
    paths = int(rng.integers(8, 129))
    clip = rng.uniform() < 0.1
    return mixed_canvas(base_seed + index, w, h, paths, clip)


def c3(count: int = 4096, base_seed: int = BASE_SEED) -> List[bytes]:
    return [c3_canvas(i, base_seed) for i in range(count)]


def c4_request_shape(index: int, base_seed: int = BASE_SEED):
    """(width, height, paths, clip) of c4_request(index) without building it."""
    rng = _rng(base_seed * 11 + index)
    w, h = _log_uniform(rng, 32, 2048), _log_uniform(rng, 32, 2048)
    paths = int(rng.integers(1, 513))
    return w, h, paths, bool(rng.uniform() < 0.1)


def c4_request(index: int, base_seed: int = BASE_SEED) -> bytes:
    w, h, paths, clip = c4_request_shape(index, base_seed)
    return mixed_canvas(base_seed + 1000003 + index, w, h, paths, clip)


def c4_parity_sample(count: int = 16, pool: int = 4000, base_seed: int = BASE_SEED):
    """Indices of c4 requests that cover the distribution's extremes: the
    largest canvases, the most paths, clipped ones, and the rest spread over
    the pool."""
    shapes = [c4_request_shape(i, base_seed) for i in range(pool)]
    by_px = sorted(range(pool), key=lambda i: -shapes[i][0] * shapes[i][1])
    by_paths = sorted(range(pool), key=lambda i: -shapes[i][2])
    clipped = [i for i in range(pool) if shapes[i][3]]
    chosen = []
    for i in by_px[:count // 4] + by_paths[:count // 4] + clipped[:count // 8]:
        if i not in chosen:
            chosen.append(i)
    step = max(1, pool // count)
    for i in range(0, pool, step):
        if len(chosen) >= count:
            break
        if i not in chosen:
            chosen.append(i)
    return chosen[:count]


def small_scene(config: str, seed: int) -> bytes:
    """Reduced versions of the configurations, sized for quick parity runs."""
    s = BASE_SEED + 7919 * seed
    if config == "c0_small":
        return c0(s, 256, 256, 16)
    if config == "c1_small":
        return c1(s, 256, 256, 24)
    if config == "c2_small":
        return c2(s, 256, 256, 30)
    if config == "mixed_small":
        rng = _rng(s)
        return mixed_canvas(s, int(rng.integers(32, 300)), int(rng.integers(32, 300)),
                            int(rng.integers(8, 25)), clip=bool(seed % 2))
    raise ValueError(config)


CONFIGS = {"c0": c0, "c1": c1, "c2": c2}
