"""Text and images drawn across many canvases, through the caches.

The same image drawn on many canvases of a frame (or by many requests) is
kept on the device after its second sighting (cy_image_cache_stats), and
glyph outlines are decoded once per font and glyph for the whole process;
text is flattened on the device.  Every canvas must still equal the oracle:
bit for bit against the oracle variant computing the library's default
coverage, and within the contract against the reference restatement.
"""
import ctypes

import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import native
from canvas_ity_gb300 import trace as T
import golden_util as G

pytestmark = pytest.mark.gpu


def font_bytes():
    entry = next(e for e in G.manifest() if e["name"] == "fill_text")
    rec = next(r for r in T.parse(G.load_fixture(entry)).records if r.op == T.SET_FONT)
    return bytes(rec.data)


def image(seed, w=48, h=40):
    return np.random.default_rng(seed).integers(0, 256, size=(h, w, 4), dtype=np.uint8)


def text_and_images(index, font, img):
    """A canvas drawing the shared image three times and the shared font's
    glyphs, filled and stroked, under a per-canvas transform."""
    rng = np.random.default_rng(500 + index)
    w, h = int(rng.integers(120, 260)), int(rng.integers(90, 200))
    t = T.TraceWriter(w, h)
    t.set_color(T.FILL_STYLE, 0.9, 0.9, 0.85, 1.0)
    t.fill_rectangle(0, 0, w, h)
    t.rotate(float(rng.uniform(-0.2, 0.2)))
    for k in range(3):
        t.draw_image(img, img.shape[1], img.shape[0], float(rng.uniform(0, w - 40)), float(rng.uniform(0, h - 30)),
                     float(rng.uniform(20, 80)), float(rng.uniform(20, 60)))
    t.set_pattern(T.FILL_STYLE, img, img.shape[1], img.shape[0], T.REPEAT)
    t.fill_rectangle(5.0, 5.0, w * 0.3, h * 0.25)
    t.set_font(font, float(rng.uniform(12, 28)))
    t.set_color(T.FILL_STYLE, 0.1, 0.2, 0.5, 0.9)
    t.fill_text("Shared glyphs, every canvas", 4.0, h * 0.6)
    t.set_line_width(float(rng.uniform(0.6, 2.0)))
    t.set_color(T.STROKE_STYLE, 0.7, 0.1, 0.1, 0.8)
    t.stroke_text("Stroked text 0123", 6.0, h * 0.9)
    return t.finish()


def cache_stats():
    lib = native.load()
    lib.cy_image_cache_stats.restype = ctypes.c_int
    lib.cy_image_cache_stats.argtypes = [ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]
    v = (ctypes.c_longlong * 5)()
    assert lib.cy_image_cache_stats(v, 5) == 5
    return {"hits": v[0], "inserts": v[1], "entries": v[2], "texel_bytes": v[3], "pool_bytes": v[4]}


@pytest.mark.parametrize("mode", sorted(G.MODES))
def test_text_and_images_through_the_caches(mode):
    font, img = font_bytes(), image(7 + len(mode))
    traces = [text_and_images(i, font, img) for i in range(24)]
    before = cache_stats()
    G.use_mode(mode)
    try:
        outs = native.render_batch(traces, G.MODES[mode][0])
    finally:
        G.use_mode("tile")
    after = cache_stats()
    # 24 canvases x 4 draws of one image: all but the first two are hits
    assert after["hits"] - before["hits"] >= 24 * 4 - 2
    assert after["inserts"] - before["inserts"] == 1
    cov = G.oracle_coverage(mode)
    for i, (tb, raw) in enumerate(zip(traces, outs)):
        assert raw == oracle.replay(tb, ties="sign", trig="cr", coverage=cov)[0], f"canvas {i}"
        for g, w in zip(G.split_images(tb, raw), G.split_images(tb, oracle.replay(tb)[0])):
            G.assert_within_contract(g, w, f"canvas {i}", strict=mode != "tile")
