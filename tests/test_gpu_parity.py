"""GPU parity: the GB300 canvas against the reference's own outputs and the oracle.

Every test runs in each render mode (golden_util.MODES): the tile engine
with binned coverage (the default), the tile engine with exact sorted-run
coverage, and the plain per-draw engine.

Tolerances (the contract for this rasteriser, golden_util.assert_within_contract):
  * RGBA8 against the reference: at least MIN_IDENTICAL of the pixels
    identical, the alpha byte within MAX_LSB everywhere, the colour bytes
    within MAX_LSB wherever alpha is above 2/255 -- and, for the exact modes,
    every byte within MAX_LSB;
  * float coverage: within COVERAGE_TOL absolute;
  * the reference test suite's own LSH hash within 5 bits of its golden value.
Beyond the tolerance, each mode's float canvas equals, bit for bit, the
oracle variant that computes what it computes (the binned restatement for
the binned mode).
"""
import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import native, scenes
from canvas_ity_gb300 import trace as T
import cy_hash
import golden_util as G

pytestmark = pytest.mark.gpu

COVERAGE_TOL = 1e-5
MANIFEST = G.manifest()
_oracle_cache = {}


def oracle_images(tb, **kw):
    """The oracle's get_image_data images of a call list (cached: the large
    scenes are shared by the modes)."""
    key = (tb, tuple(sorted(kw.items())))
    if key not in _oracle_cache:
        _oracle_cache[key] = G.split_images(tb, oracle.replay(tb, **kw)[0])
    return _oracle_cache[key]


def assert_images_close(got, want, what, mode="tile"):
    G.assert_within_contract(got, want, what, strict=mode != "tile")


@pytest.fixture(params=sorted(G.MODES))
def engine(request):
    G.use_mode(request.param)
    yield request.param
    G.use_mode("tile")


@pytest.fixture(params=["device", "host"])
def stroke(request):
    """Where strokes are expanded: on the GPU (the default) or on the host."""
    native.set_device_stroke(request.param == "device")
    yield request.param
    native.set_device_stroke(True)


def trig():
    """The oracle variant whose round joins compute what the library's stroke
    expansion computes: acos/tan rounded from double on the GPU, libm's
    acosf/tanf on the host."""
    return "cr" if native.device_stroke() else "libm"


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_reference_suite(engine, entry):
    tb = G.load_fixture(entry)
    t = T.parse(tb)
    raw, results = native.replay(tb)
    got = G.split_images(tb, raw)
    want = [img for _, _, img in t.expected_images()]
    assert len(got) == len(want)
    for i, (g, w) in enumerate(zip(got, want)):
        assert_images_close(g, w, f"{entry['name']} read {i}", engine)
    assert results == t.expected_results()
    assert cy_hash.hamming(cy_hash.hash_image(got[-1]), entry["golden_hash"]) <= 5


@pytest.mark.parametrize("config", ["c0_small", "c1_small", "c2_small", "mixed_small"])
@pytest.mark.parametrize("seed", range(4))
def test_seeded_scene_vs_oracle(engine, config, seed):
    tb = scenes.small_scene(config, seed)
    got = G.split_images(tb, native.replay(tb)[0])
    want = G.split_images(tb, oracle.replay(tb)[0])
    for g, w in zip(got, want):
        assert_images_close(g, w, f"{config}/{seed}", engine)


@pytest.mark.parametrize("config", ["c0", "c1"])
def test_full_size_config_vs_oracle(engine, config):
    tb = scenes.CONFIGS[config]()
    got = G.split_images(tb, native.replay(tb)[0])[-1]
    want = oracle_images(tb)[-1]
    assert_images_close(got, want, config, engine)
    if engine == "tile":
        assert np.array_equal(got, oracle_images(tb, coverage="binned")[-1])


def test_c2_full_size_vs_oracle(engine):
    """The paint and composite scene at its stated size: 2048x2048, 500
    paths with gradients and patterns, all 11 operations, one 16-vertex
    clip, shadows on 20% of paths (about half a minute per oracle replay,
    shared by the modes)."""
    tb = scenes.c2()
    got = G.split_images(tb, native.replay(tb)[0])[-1]
    want = oracle_images(tb)[-1]
    assert_images_close(got, want, "c2", engine)
    if engine == "tile":
        assert np.array_equal(got, oracle_images(tb, coverage="binned")[-1])


_c4_cache = {}


def c4_sample():
    """16 serving requests of config 4 (sides log-uniform 32-2048, 1-512
    paths) covering its extremes, with the oracle's reads of each under the
    reference restatement and under the binned one (computed once, in
    parallel, for all modes)."""
    if not _c4_cache:
        from concurrent.futures import ThreadPoolExecutor
        ids = scenes.c4_parity_sample(16)
        tbs = [scenes.c4_request(i) for i in ids]
        oracle.replay(tbs[0])
        oracle.replay(tbs[0], ties="sign", trig="cr", coverage="binned")
        with ThreadPoolExecutor(16) as ex:
            ref = list(ex.map(lambda t: oracle.replay(t)[0], tbs))
            binned = list(ex.map(lambda t: oracle.replay(t, ties="sign", trig="cr", coverage="binned")[0], tbs))
        _c4_cache.update(ids=ids, traces=tbs, ref=ref, binned=binned)
    return _c4_cache


def test_c4_request_sample_vs_oracle(engine):
    """Config 4's requests, including its largest canvases (up to 2048 x
    2048) and path counts (up to 512), rendered together in one frame as the
    server renders them."""
    c4 = c4_sample()
    outs = native.render_batch(c4["traces"], G.MODES[engine][0])
    for i, (tb, raw) in enumerate(zip(c4["traces"], outs)):
        what = f"c4 request {c4['ids'][i]}"
        for g, w in zip(G.split_images(tb, raw), G.split_images(tb, c4["ref"][i])):
            assert_images_close(g, w, what, engine)
        if engine == "tile":
            assert raw == c4["binned"][i], what


def assert_float_canvas_exact(tb, what, mode):
    """The GPU's final premultiplied linear canvas equals, bit for bit, the
    oracle built with the GPU's order for runs of one cell that the
    reference's sort leaves unordered (equal magnitude, opposite sign), and
    with the mode's coverage."""
    w, h = T.canvas_size(tb)
    got = native.replay_linear(tb, w, h)
    want = oracle.replay_linear(tb, w, h, ties="sign", trig=trig(), coverage=G.oracle_coverage(mode))
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{what}: {len(bad)} float values differ, first at (y, x, c) = {bad[0].tolist()}"


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_reference_suite_bytes_identical(engine, entry):
    """Beyond the tolerance: every get_image_data byte of the reference's own
    suite equals the recorded reference output (exact modes), or the
    binned oracle's (binned mode)."""
    tb = G.load_fixture(entry)
    got = G.split_images(tb, native.replay(tb)[0])
    if engine == "tile":
        want = G.split_images(tb, oracle.replay(tb, coverage="binned")[0])
    else:
        want = [img for _, _, img in T.parse(tb).expected_images()]
    for i, (g, w) in enumerate(zip(got, want)):
        assert np.array_equal(g, w), f"{entry['name']} read {i}: {int((g != w).any(axis=-1).sum())} pixels differ"


DEMOS = G.demos()


@pytest.mark.parametrize("bad", [float("nan"), float("inf"), 1e9, 1e30], ids=["nan", "inf", "1e9", "1e30"])
def test_non_finite_and_far_points(engine, bad):
    """Vertices at NaN, infinity or far off the canvas: every mode equals
    its oracle byte for byte.  The exact modes reproduce the reference's
    polygon clip, which leaves non-finite points out and whose crossings
    with far points cancel (the draw's bounds are then unknown, so no row
    is skipped); the binned mode joins the neighbours of a non-finite point
    the same way and takes far crossings from the nearer end."""
    tb = G.far_point_scene(bad)
    got = native.replay(tb)[0]
    assert got == oracle.replay(tb, ties="sign", trig=trig(), coverage=G.oracle_coverage(engine))[0]


@pytest.mark.parametrize("demo", DEMOS, ids=[d["name"] for d in DEMOS])
def test_reference_demo(engine, stroke, demo):
    """The reference's tiger demo (demos/tiger/tiger.cpp, 733 x 757): the
    RGBA8 canvas within the contract of the reference's own bytes (equal to
    them in the exact modes), byte-identical to the mode's oracle, and the
    float canvas bit for bit the oracle's."""
    tb = G.load_fixture(demo)
    got = G.split_images(tb, native.replay(tb)[0])[-1]
    want = G.final_image(tb)
    assert_images_close(got, want, demo["name"], engine)
    if engine != "tile":
        assert np.array_equal(got, want)
    mine = oracle_images(tb, ties="sign", trig=trig(), coverage=G.oracle_coverage(engine))[-1]
    assert np.array_equal(got, mine)
    assert_float_canvas_exact(tb, demo["name"], engine)


@pytest.mark.parametrize("seed", range(8))
def test_rgba8_identical_to_oracle_on_workload(engine, stroke, seed):
    """RGBA8 bytes of many-canvas workload canvases equal the oracle's with
    the GPU's order for runs std::sort leaves unordered; with strokes
    expanded on the GPU they also equal the oracle with libm's round joins."""
    tb = scenes.c3_canvas(100 + seed)
    got = native.replay(tb)[0]
    cov = G.oracle_coverage(engine)
    assert got == oracle.replay(tb, ties="sign", trig=trig(), coverage=cov)[0]
    assert got == oracle.replay(tb, ties="sign", coverage=cov)[0]


@pytest.mark.parametrize("entry", MANIFEST, ids=[e["name"] for e in MANIFEST])
def test_float_canvas_bit_exact_reference_suite(engine, stroke, entry):
    assert_float_canvas_exact(G.load_fixture(entry), entry["name"], engine)


@pytest.mark.parametrize("config", ["c0_small", "c1_small", "c2_small", "mixed_small"])
@pytest.mark.parametrize("seed", range(3))
def test_float_canvas_bit_exact_seeded(engine, stroke, config, seed):
    assert_float_canvas_exact(scenes.small_scene(config, seed), f"{config}/{seed}", engine)


@pytest.mark.parametrize("seed", range(6))
def test_float_canvas_bit_exact_batched_workload(engine, stroke, seed):
    """Canvases of the many-canvas workload (random size, 8-128 paths of the
    c0/c1/c2 mixture, global transform)."""
    assert_float_canvas_exact(scenes.c3_canvas(seed), f"c3 canvas {seed}", engine)


def _even_odd(tb):
    """The same call list with the even-odd fill rule set right after the
    canvas record (header 8 bytes + canvas record 12 bytes)."""
    import struct
    return tb[:20] + struct.pack("<ii", T.SET_FILL_RULE, T.EVEN_ODD) + tb[20:]


@pytest.mark.parametrize("config", ["c0_small", "c1_small", "c2_small", "mixed_small"])
@pytest.mark.parametrize("seed", range(2))
def test_even_odd_float_canvas_bit_exact(engine, config, seed):
    """Even-odd fills, clips and shadows (an extension: pinned to the oracle's
    restatement of the rule, no reference output exists)."""
    assert_float_canvas_exact(_even_odd(scenes.small_scene(config, seed)), f"even-odd {config}/{seed}", engine)


@pytest.mark.parametrize("seed", range(6))
def test_float_coverage(engine, seed):
    """One opaque white nonzero fill on a blank canvas: the linear alpha is the
    coverage itself, compared as floats."""
    rng = np.random.default_rng(seed)
    w, h = 192, 160
    t = T.TraceWriter(w, h)
    t.set_color(T.FILL_STYLE, 1.0, 1.0, 1.0, 1.0)
    t.begin_path()
    n = int(rng.integers(3, 24))
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
    got = native.replay_linear(tb, w, h)[..., 3]
    want = oracle.replay_linear(tb, w, h)[..., 3]
    assert_coverage_close(got, want)
    if engine == "tile":
        assert np.array_equal(got, oracle.replay_linear(tb, w, h, coverage="binned")[..., 3])


def assert_coverage_close(got, want):
    """Coverage within COVERAGE_TOL.  A pixel is painted only when its
    coverage reaches 1/8160 (hpp:2571), so where one side painted and the
    other did not, the painted coverage must lie within COVERAGE_TOL of that
    threshold (the unpainted one was just below it)."""
    both = (got > 0) & (want > 0)
    assert np.abs(got - want)[both].max(initial=0.0) <= COVERAGE_TOL
    one = (got > 0) != (want > 0)
    assert (np.maximum(got, want)[one] <= 1.0 / 8160.0 + COVERAGE_TOL).all()


def test_empty_and_degenerate_inputs(engine):
    t = T.TraceWriter(33, 17)
    t.fill()                                   # empty path
    t.begin_path(); t.move_to(5, 5); t.fill()  # single point
    t.set_global_composite_operation(T.SOURCE_COPY)
    t.fill_rectangle(2, 2, 0, 5)               # zero width: ignored
    t.set_global_composite_operation(T.SOURCE_OVER)
    t.set_color(T.FILL_STYLE, 1, 0, 0, 1)
    t.fill_rectangle(-10, -10, 20, 20)         # partly off canvas
    t.scale(0, 1)
    t.fill_rectangle(0, 0, 10, 10)             # singular transform: nothing drawn
    t.set_transform(1, 0, 0, 1, 0, 0)
    t.get_image_data(50, 40, -8, -8)           # read outside the canvas
    t.put_image_data(None, 4, 4, 0, 0)         # null image: ignored
    tb = t.finish()
    got = G.split_images(tb, native.replay(tb)[0])
    want = G.split_images(tb, oracle.replay(tb, coverage=G.oracle_coverage(engine))[0])
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_one_by_one_and_large_canvas(engine):
    for w, h in ((1, 1), (4096, 3)):
        t = T.TraceWriter(w, h)
        t.set_color(T.FILL_STYLE, 0.2, 0.6, 0.9, 0.7)
        t.begin_path()
        t.move_to(0.3, 0.1)
        t.line_to(w - 0.2, h * 0.8)
        t.line_to(0.1, h - 0.1)
        t.fill()
        tb = t.finish()
        got = G.split_images(tb, native.replay(tb)[0])[-1]
        want = G.split_images(tb, oracle.replay(tb)[0])[-1]
        assert_images_close(got, want, f"{w}x{h}", engine)


@pytest.mark.parametrize("mode", sorted(G.MODES))
def test_batched_frame_matches_oracle(mode):
    """Many canvases of mixed sizes rendered in one frame: each result equals
    the oracle's, i.e. the same as when rendered alone."""
    traces = [scenes.small_scene(cfg, s) for s in range(3)
              for cfg in ("c0_small", "c1_small", "c2_small", "mixed_small")]
    traces += [G.load_fixture(e) for e in MANIFEST[::7]]
    G.use_mode(mode)
    try:
        outs = native.render_batch(traces, G.MODES[mode][0])
    finally:
        G.use_mode("tile")
    for tb, raw in zip(traces, outs):
        got = G.split_images(tb, raw)
        want = G.split_images(tb, oracle.replay(tb)[0])
        for g, w in zip(got, want):
            assert_images_close(g, w, "batched", mode)
        if mode == "tile":
            assert raw == oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0]


@pytest.mark.parametrize("mode", sorted(G.MODES))
def test_graph_captured_frame_matches_oracle(mode):
    """A frame run replayed from its captured CUDA graph gives the same
    reads as the oracle (and as the run that sized it)."""
    traces = [scenes.small_scene(cfg, 5) for cfg in ("c0_small", "c1_small", "c2_small", "mixed_small")]
    G.use_mode(mode)
    try:
        with native.Frame(traces, G.MODES[mode][0]) as f:
            f.capture()
            for _ in range(2):
                f.run()
            f.sync()
            outs = f.finish()
    finally:
        G.use_mode("tile")
    for tb, raw in zip(traces, outs):
        got = G.split_images(tb, raw)
        want = G.split_images(tb, oracle.replay(tb)[0])
        for g, w in zip(got, want):
            assert_images_close(g, w, "graph", mode)
        if mode == "tile":
            assert raw == oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0]


def test_autotuned_frame_matches_oracle():
    """The autotuner times the paint stage over strip configurations, keeps
    the fastest, and the frame then renders with it unchanged."""
    traces = [scenes.small_scene(cfg, 7) for cfg in ("c0_small", "c1_small", "c2_small", "mixed_small")]
    try:
        with native.Frame(traces, 0) as f:
            tuned = f.autotune()
            assert tuned["strip_pixels"] in (2048, 4096, 8192)
            assert tuned["threads"] in (128, 256, 512) and tuned["paint_ms"] > 0
            f.capture()
            f.run()
            f.sync()
            outs = f.finish()
        for tb, raw in zip(traces, outs):
            got = G.split_images(tb, raw)
            want = G.split_images(tb, oracle.replay(tb)[0])
            for g, w in zip(got, want):
                assert_images_close(g, w, f"autotuned {tuned}")
            assert raw == oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0]
    finally:
        native.set_strip_config(4096, 256)


@pytest.mark.parametrize("threads", [128, 256, 512])
@pytest.mark.parametrize("strip_pixels", [1024, 4096, 8192])
def test_tile_engine_strip_sizes(strip_pixels, threads):
    """Every strip configuration renders the same bytes: the binned sums
    are integers, so neither the strip height nor how rows are dealt to
    warps changes a pixel (several canvas widths give strips of 1 to 128
    rows, with rows split across warps or whole)."""
    native.set_strip_config(strip_pixels, threads)
    try:
        traces = [scenes.small_scene("mixed_small", s) for s in range(4)] + [scenes.c3_canvas(s) for s in (3, 11, 29)]
        outs = native.render_batch(traces, 0)
        for tb, raw in zip(traces, outs):
            assert raw == oracle.replay(tb, ties="sign", trig="cr", coverage="binned")[0], f"strip {strip_pixels}"
            got = G.split_images(tb, raw)[-1]
            want = G.split_images(tb, oracle.replay(tb)[0])[-1]
            assert_images_close(got, want, f"strip {strip_pixels}")
    finally:
        native.set_strip_config(4096, 256)


def test_frame_views_match_copies():
    """cy_frame_finish_views hands out the pinned read-back buffer itself;
    its per-canvas ranges hold the same bytes as the copying collection."""
    traces = [scenes.small_scene(cfg, 9) for cfg in ("c0_small", "c1_small", "c2_small", "mixed_small")]
    traces += [scenes.c3_canvas(70 + s) for s in range(3)]
    want = native.render_batch(traces, 0)
    with native.Frame(traces, 0) as f:
        views = f.finish(copy=False)
        got = [bytes(v) for v in views]
    assert got == want


@pytest.mark.parametrize("frame_pixels", [0, 60000])
def test_render_traces_pipelined_matches_frames(frame_pixels):
    """cy_render_traces (frames pipelined: host replay of one under the
    device work of the previous) writes every canvas's reads where the
    caller's offsets say, equal to the single-frame path; small frames
    force many frames in flight."""
    traces = [scenes.c3_canvas(80 + s) for s in range(6)]
    traces += [scenes.small_scene(cfg, 4) for cfg in ("c0_small", "c1_small", "c2_small", "mixed_small")]
    want = native.render_batch(traces, 0)
    views, stats = native.render_traces(traces, 0, frame_pixels)
    assert [bytes(v) for v in views] == want
    assert stats["read_bytes"] == sum(len(w) for w in want)
    if frame_pixels:
        assert stats["frames"] > 1


def test_render_traces_rejects_wrong_sizes():
    traces = [scenes.small_scene("c0_small", 1), scenes.small_scene("c1_small", 1)]
    sizes = [T.read_bytes(t) for t in traces]
    offsets = np.array([0, sizes[0] + 4, sizes[0] + sizes[1] + 4], np.uint64)
    with pytest.raises(RuntimeError, match="status -1"):
        native.render_traces(traces, 0, 0, np.zeros(int(offsets[-1]), np.uint8), offsets)


def test_render_traces_wide_canvas_falls_back():
    """A canvas wider than a tile-engine strip renders on the per-draw engine
    inside cy_render_traces, with the same reads as alone."""
    t = T.TraceWriter(4500, 12)
    t.set_color(T.FILL_STYLE, 0.3, 0.6, 0.9, 0.8)
    t.begin_path(); t.move_to(3.5, 1.25); t.line_to(4490.0, 6.0); t.line_to(10.0, 11.0); t.fill()
    t.get_image_data(4500, 12, 0, 0)
    wide = t.finish(read_back=False)
    traces = [scenes.small_scene("c0_small", 2), wide]
    views, _ = native.render_traces(traces, 0)
    assert bytes(views[1]) == native.replay(wide)[0]
    assert bytes(views[0]) == native.replay(traces[0])[0]
