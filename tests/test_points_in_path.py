"""Batched is_point_in_path on the GPU (cy_points_in_path): the same
answers as the reference's is_point_in_path (src/canvas_ity.hpp:3101-3132)
called once per point, for paths of lines, cubics, quadratics and arcs,
several subpaths, transforms, both fill rules, and points on vertices and
edges."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import native
from canvas_ity_gb300 import trace as T


def _build(t, seed: int):
    """Random current path on writer t; returns the path's vertices."""
    rng = np.random.default_rng(900 + seed)
    if seed % 3 == 1:
        t.set_fill_rule(T.EVEN_ODD)
    if seed % 4 == 2:
        t.translate(30.0, 10.0)
        t.rotate(0.3)
        t.scale(1.25, 0.8)
    t.begin_path()
    verts = []
    for _ in range(int(rng.integers(1, 4))):
        p = rng.integers(0, 150, 2).astype(float)   # integer vertices: exact boundary queries
        t.move_to(*p)
        verts.append(p)
        for _ in range(int(rng.integers(2, 8))):
            r = rng.random()
            q = rng.integers(0, 150, 2).astype(float)
            if r < 0.5:
                t.line_to(*q)
            elif r < 0.75:
                c = rng.uniform(0, 150, 4)
                t.bezier_curve_to(c[0], c[1], c[2], c[3], q[0], q[1])
            elif r < 0.9:
                c = rng.uniform(0, 150, 2)
                t.quadratic_curve_to(c[0], c[1], q[0], q[1])
            else:
                t.arc(q[0], q[1], float(rng.uniform(5, 40)), 0.0, float(rng.uniform(1, 2 * math.pi)))
            verts.append(q)
        if rng.random() < 0.6:
            t.close_path()
    qrng = np.random.default_rng(50 + seed)
    v = np.array(verts)
    return np.concatenate([qrng.uniform(-10, 210, (600, 2)), v, v + np.array([0.5, 0.0])]).astype(np.float32)


def path_trace(seed: int):
    """(call list whose canvas ends with a random current path, the same
    list with is_point_in_path for every query appended, the queries)."""
    base = T.TraceWriter(200, 150)
    queries = _build(base, seed)
    probe = T.TraceWriter(200, 150)
    _build(probe, seed)
    for x, y in queries:
        probe.is_point_in_path(float(x), float(y))
    return base.finish(read_back=False), probe.finish(read_back=False), queries


def expected(probe):
    return np.array(oracle.replay(probe)[1], np.float32).astype(np.uint8)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(12))
def test_points_in_path_matches_reference(seed):
    base, probe, queries = path_trace(seed)
    got = native.points_in_path(base, queries)
    want = expected(probe)
    assert len(got) == len(want)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, f"{bad.size} of {len(queries)} points differ, first {queries[bad[0]].tolist()}"


@pytest.mark.gpu
def test_points_in_path_empty_path():
    t = T.TraceWriter(16, 16)
    t.begin_path()
    got = native.points_in_path(t.finish(read_back=False), np.array([[1.0, 1.0], [8.0, 8.0]], np.float32))
    assert got.tolist() == [0, 0]


def test_points_in_path_rejects_bad_arguments():
    lib = native.load()
    fn = lib.cy_points_in_path
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                   ctypes.c_void_p]
    pts = np.zeros(8, np.float32)
    cnt = np.array([3], np.int32)          # not 1 + 3k points
    q = np.zeros(2, np.float32)
    out = np.zeros(1, np.uint8)
    assert fn(pts.ctypes.data, cnt.ctypes.data, 1, q.ctypes.data, 1, 0, out.ctypes.data) == -1
    assert fn(None, None, 0, None, 0, 0, None) == 0        # no queries: nothing to do
    assert fn(None, None, -1, None, 0, 0, None) == -1
