"""The CPU oracle is pinned against the reference's own golden data.

* the 76 recorded reference tests: the oracle must reproduce the reference's
  get_image_data bytes, hit tests and text measurements exactly, and its final
  images must hash within 5 bits of the golden hashes in the reference's table
  (test/test.cpp:2185-2261, pass rule at 2614-2618);
* the get_image_data known-answer test (test/test.cpp:1800-1830), whose exact
  byte hash 0xf53f9792 pins dither and quantisation;
* where the reference sources are present, seeded scenes replayed through the
  reference itself.
"""
import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import scenes
from canvas_ity_gb300 import trace as T
import cy_hash
import golden_util as G

MANIFEST = G.manifest()


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_oracle_matches_reference_fixture(entry):
    tb = G.load_fixture(entry)
    t = T.parse(tb)
    raw, results = oracle.replay(tb)
    got = G.split_images(tb, raw)
    want = [img for _, _, img in t.expected_images()]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    assert results == t.expected_results()
    assert cy_hash.hamming(cy_hash.hash_image(got[-1]), entry["golden_hash"]) <= 5


DEMOS = G.demos()


@pytest.mark.parametrize("demo", DEMOS, ids=[d["name"] for d in DEMOS])
def test_oracle_matches_reference_demo(demo):
    """The reference's tiger demo (demos/tiger/tiger.cpp, 733 x 757, its
    headline drawing): the oracle reproduces the reference's bytes, and the
    binned restatement stays within the contract."""
    tb = G.load_fixture(demo)
    want = G.final_image(tb)
    assert want.shape == (demo["height"], demo["width"], 4)
    got = G.split_images(tb, oracle.replay(tb)[0])[-1]
    assert np.array_equal(got, want)
    binned = G.split_images(tb, oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0])[-1]
    G.assert_within_contract(binned, want, demo["name"])


def _image(raw, w=64, h=48):
    return np.frombuffer(raw, np.uint8).reshape(h, w, 4)


@pytest.mark.parametrize("bad", [float("nan"), float("inf"), -float("inf")], ids=["nan", "inf", "-inf"])
def test_binned_leaves_out_non_finite_points_like_the_polygon_clip(bad):
    """The reference's polygon clip drops a point whose comparisons fail and
    joins its neighbours; the binned clip, segment by segment, does the same
    (the segment leaving the point starts from the finite point before it),
    so no row is left open."""
    tb = G.far_point_scene(bad)
    exact = oracle.replay(tb)[0]
    binned = oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0]
    G.assert_within_contract(_image(binned), _image(exact), f"binned, vertex at {bad}")
    if oracle.reference_available():
        assert exact == oracle.reference_replay(tb)[0]


@pytest.mark.parametrize("far", [1e9, 1e12, 1e30])
def test_binned_crossings_hold_for_far_points(far):
    """From about 1e9 on, the reference's clip loses a far point's crossing
    with the canvas edge to cancellation (a + t (b - a) with b far away), and
    the exact oracle keeps that.  The binned clip takes crossings from the
    nearer end: it draws what a moderately far point (1e6) on nearly the same
    line draws."""
    want = _image(oracle.replay(G.far_point_scene(1e6))[0])
    got = _image(oracle.replay(G.far_point_scene(far), ties="sign", trig="cr", coverage="binned")[0])
    G.assert_within_contract(got, want, f"binned, vertex at {far}")
    assert not np.array_equal(_image(oracle.replay(G.far_point_scene(far))[0]), want)


@pytest.mark.parametrize("span", [300.0, 1e4, 1e5])
def test_binned_projection_of_far_polygons_is_exact(span):
    """A rotated square whose corners lie `span` away around the canvas
    covers every pixel.  Its edges left of the canvas project onto x = 0,
    and clamping such a piece to [0, height] clips it exactly, so every
    pixel's binned coverage is exactly 1; the others add nothing."""
    w, h = 160, 128
    t = T.TraceWriter(w, h)
    t.set_color(T.FILL_STYLE, 1.0, 1.0, 1.0, 1.0)
    t.begin_path()
    for k in range(4):
        a = 0.3 + k * np.pi / 2
        p = (w / 2 + span * np.cos(a), h / 2 + span * np.sin(a))
        (t.move_to if k == 0 else t.line_to)(*p)
    t.close_path()
    t.fill()
    tb = t.finish()
    cov = oracle.replay_linear(tb, w, h, coverage="binned")[..., 3]
    assert (cov == 1.0).all()


def test_binned_wholly_left_subpath_cancels_exactly():
    """A subpath wholly left of the canvas projects onto x = 0 as a closed
    chain of vertical pieces.  Where its y values are 2 or more they are
    multiples of 2^-22 (a float's step there), so every piece's fixed-point
    sum is exact and the chain cancels to nothing: the float canvas is the
    same bit for bit as without the subpath."""
    def scene(extra):
        t = T.TraceWriter(96, 80)
        t.set_color(T.FILL_STYLE, 0.3, 0.6, 0.9, 1.0)
        t.begin_path()
        t.move_to(10.3, 12.7)
        t.line_to(80.1, 20.2)
        t.line_to(60.4, 70.9)
        t.close_path()
        if extra:
            t.move_to(-50.25, 5.5)
            t.line_to(-10.75, 60.125)
            t.line_to(-30.5, 79.0)
            t.close_path()
        t.fill()
        return t.finish()
    a = oracle.replay_linear(scene(False), 96, 80, coverage="binned")
    b = oracle.replay_linear(scene(True), 96, 80, coverage="binned")
    assert np.array_equal(a, b)


def test_get_image_data_known_answer():
    """test/test.cpp:1800-1826: strided, offset read of a 10x10 checker."""
    entry = next(e for e in MANIFEST if e["name"] == "get_image_data")
    tb = G.load_fixture(entry)
    raw, _ = oracle.replay(tb)
    first = G.split_images(tb, raw)[0]  # the 35x35 read at (-10, -10)
    data = np.zeros(4939, np.uint8)
    data[0] = 150
    for i in range(1, 4939):
        data[i] = (int(data[i - 1]) * 137 + 53) & 255
    for row in range(35):
        data[2 + row * 141: 2 + row * 141 + 140] = first[row].reshape(-1)
    h = 0
    for v in data:
        h = ((((h & 0x1FFFF) << 15) | (h >> 17)) ^ int(v)) & 0xFFFFFFFF
    assert h == 0xF53F9792


@pytest.mark.reference
@pytest.mark.parametrize("config", ["c0_small", "c1_small", "c2_small", "mixed_small"])
def test_oracle_matches_reference_on_seeded_scenes(config):
    if not oracle.reference_available():
        pytest.skip("reference sources are not present here")
    for seed in range(3):
        tb = scenes.small_scene(config, seed)
        a = oracle.replay(tb)
        r = oracle.reference_replay(tb)
        assert a[0] == r[0]
        assert a[1] == r[1]


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_sign_ordered_ties_match_reference_fixture(entry):
    """The oracle variant that orders equal-magnitude, opposite-sign runs of
    one cell negative first (the order the GPU path uses, where std::sort
    leaves them unordered) still reproduces every recorded reference image."""
    tb = G.load_fixture(entry)
    t = T.parse(tb)
    got = G.split_images(tb, oracle.replay(tb, ties="sign")[0])
    want = [img for _, _, img in t.expected_images()]
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("index", range(8))
def test_sign_ordered_ties_bounded_on_workload(index):
    """On canvases of the many-canvas workload the two tie orders differ by
    float rounding only.  What holds at every pixel:
      * the alpha byte is within 1 LSB;
      * the colour bytes are within 1 LSB wherever alpha is above 2/255;
      * where alpha is 2/255 or less, get_image_data divides the colour by
        alpha (hpp:3348-3381), which magnifies the last bit of the float by
        up to 255x at alpha 1/255: the colour bytes there are bounded by
        2 LSB, the largest difference seen on 256 workload canvases, and
        such pixels are at most 2/255 opaque.
    And at least 99.5% of the pixels are identical."""
    tb = scenes.c3_canvas(index * 37)
    a = np.frombuffer(oracle.replay(tb, ties="sign")[0], np.uint8).reshape(-1, 4).astype(np.int16)
    b = np.frombuffer(oracle.replay(tb)[0], np.uint8).reshape(-1, 4).astype(np.int16)
    d = np.abs(a - b)
    assert d[:, 3].max(initial=0) <= 1
    opaque = np.minimum(a[:, 3], b[:, 3]) > 2
    assert d[opaque].max(initial=0) <= 1
    assert d[~opaque].max(initial=0) <= 2
    assert (d.max(axis=1) != 0).mean() <= 0.005


# ------------------------------------------- the binned coverage restatement
# The GPU's default coverage (fixed-point areas accumulated per strip, no
# sorted runs) is restated in the oracle (coverage="binned"); the GPU tests
# hold the GPU to it bit for bit.  Here, on the CPU and at scale, that
# restatement is held to the reference's own outputs and to the oracle.

@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_binned_coverage_within_contract_on_reference_suite(entry):
    tb = G.load_fixture(entry)
    got = G.split_images(tb, oracle.replay(tb, coverage="binned")[0])
    want = [img for _, _, img in T.parse(tb).expected_images()]
    for i, (g, w) in enumerate(zip(got, want)):
        G.assert_within_contract(g, w, f"{entry['name']} read {i}")
    assert cy_hash.hamming(cy_hash.hash_image(got[-1]), entry["golden_hash"]) <= 5


@pytest.mark.parametrize("index", range(16))
def test_binned_coverage_within_contract_on_workload(index):
    tb = scenes.c3_canvas(index * 17 + 5)
    got = G.split_images(tb, oracle.replay(tb, coverage="binned")[0])
    want = G.split_images(tb, oracle.replay(tb)[0])
    for g, w in zip(got, want):
        G.assert_within_contract(g, w, f"c3 canvas {index * 17 + 5}")


@pytest.mark.parametrize("seed", range(24))
def test_binned_coverage_within_tolerance(seed):
    """One opaque white fill on a blank canvas (its float alpha is its
    coverage): within 1e-5 of the sorted-run coverage wherever both paint;
    where only one side paints, its coverage is within 1e-5 of the
    1/8160 painting threshold (hpp:2571)."""
    rng = np.random.default_rng(1000 + seed)
    w, h = 160, 128
    t = T.TraceWriter(w, h)
    t.set_color(T.FILL_STYLE, 1.0, 1.0, 1.0, 1.0)
    if seed % 3 == 2:
        t.set_fill_rule(T.EVEN_ODD)
    t.begin_path()
    n = int(rng.integers(3, 40))
    pts = rng.uniform((-30, -30), (w + 30, h + 30), size=(n, 2))
    t.move_to(*pts[0])
    for i in range(1, n):
        if i % 3 == 0:
            c = rng.uniform((-30, -30), (w + 30, h + 30), size=(2, 2))
            t.bezier_curve_to(c[0, 0], c[0, 1], c[1, 0], c[1, 1], *pts[i])
        else:
            t.line_to(*pts[i])
    t.close_path()
    t.fill()
    tb = t.finish()
    a = oracle.replay_linear(tb, w, h, coverage="binned")[..., 3]
    b = oracle.replay_linear(tb, w, h)[..., 3]
    both = (a > 0) & (b > 0)
    assert np.abs(a - b)[both].max(initial=0.0) <= 1e-5
    one = (a > 0) != (b > 0)
    assert (np.maximum(a, b)[one] <= 1.0 / 8160.0 + 1e-5).all()


@pytest.mark.reference
def test_port_runs_at_the_reference_speed():
    """The CPU baseline on the GPU host is this restatement (the reference's
    sources do not travel there): on the same canvases, one thread, it must
    run at the speed of the reference header compiled here, so that a
    baseline measured with it stands for the reference's own."""
    import time
    if not oracle.reference_available():
        pytest.skip("reference sources are not present here")
    traces = [scenes.c3_canvas(i) for i in range(24)]
    oracle.replay(traces[0])
    oracle.reference_replay(traces[0])
    best = {}
    for name, fn in (("port", oracle.replay), ("reference", oracle.reference_replay)) * 2:
        t0 = time.perf_counter()
        for tb in traces:
            fn(tb)
        best[name] = min(best.get(name, 1e9), time.perf_counter() - t0)
    ratio = best["reference"] / best["port"]
    print(f"port {best['port']:.3f} s, reference {best['reference']:.3f} s, port speed / reference speed {ratio:.3f}")
    assert 0.67 <= ratio <= 1.5
