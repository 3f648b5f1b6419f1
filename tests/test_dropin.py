"""The drop-in boundary, checked with a compiled application.

tests/dropin/app.cpp is application code written against the reference's
public class (src/canvas_ity.hpp:177-1148): it includes include/canvas_ity.hpp,
uses the public data members, the enums, text, draw_image, save/restore and
get_image_data, and links -lcanvas_ity_gb300 with the command INTEGRATION.md
gives.  On the CPU it must compile and link, with every class symbol it needs
defined by the library; on the GPU its output must equal the oracle's for the
same calls (bit for bit against the oracle variant that computes what the
library computes, and within the parity contract against the oracle itself).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from canvas_ity_gb300 import build, scenes
from canvas_ity_gb300 import trace as T
import golden_util as G

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
APP_SRC = os.path.join(HERE, "dropin", "app.cpp")


@pytest.fixture(scope="module")
def app(tmp_path_factory):
    """The application, compiled and linked as an application would be."""
    lib = build.build()
    out = str(tmp_path_factory.mktemp("dropin") / "app")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", APP_SRC,
                    "-I", os.path.join(REPO, "include"), "-L", libdir, "-lcanvas_ity_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", out], check=True)
    return out


def test_application_compiles_and_links(app):
    """Every canvas_ity symbol the application needs is defined by the library."""
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm is not available")
    need = subprocess.run([nm, "-D", "--undefined-only", app], check=True, capture_output=True,
                          text=True).stdout.split()
    need = {s for s in need if "canvas_ity" in s}
    have = subprocess.run([nm, "-D", "--defined-only", build.LIB], check=True, capture_output=True,
                          text=True).stdout.split()
    assert need, "the application uses no class symbols"
    assert need <= set(have), sorted(need - set(have))


def font_bytes():
    entry = next(e for e in G.manifest() if e["name"] == "fill_text")
    rec = next(r for r in T.parse(G.load_fixture(entry)).records if r.op == T.SET_FONT)
    return bytes(rec.data)


def checker():
    img = np.zeros((4, 4, 4), np.uint8)
    for i in range(16):
        on = ((i & 3) + (i >> 2)) & 1
        img[i >> 2, i & 3] = (230, 120, 30, 255) if on else (20, 60, 200, 255)
    return img


STAR = [(80.0, 14.0), (91.75, 45.8), (125.65, 47.15), (99.0, 68.2), (108.2, 100.85), (80.0, 82.0),
        (51.8, 100.85), (61.0, 68.2), (34.35, 47.15), (68.25, 45.8)]


def demo_trace(font):
    """The calls of app.cpp's `demo`, as a call list for the oracle."""
    w, h = 160, 120
    t = T.TraceWriter(w, h)
    img = checker()
    t.set_pattern(T.FILL_STYLE, img, 4, 4, T.REPEAT)
    t.fill_rectangle(4.0, 4.0, 70.0, 50.0)
    t.save()
    t.begin_path()
    t.arc(80.0, 60.0, 50.0, 0.0, 6.2831853)
    t.clip()
    t.set_shadow_offset_x(4.0)
    t.set_shadow_offset_y(3.0)
    t.set_shadow_color(0.1, 0.0, 0.2, 0.6)
    t.set_shadow_blur(3.0)
    t.set_linear_gradient(T.FILL_STYLE, 30.0, 10.0, 130.0, 110.0)
    t.add_color_stop(T.FILL_STYLE, 0.0, 1.0, 0.8, 0.1, 1.0)
    t.add_color_stop(T.FILL_STYLE, 1.0, 0.1, 0.3, 0.9, 0.8)
    t.begin_path()
    t.move_to(*STAR[0])
    for p in STAR[1:]:
        t.line_to(*p)
    t.close_path()
    t.fill()
    t.restore()
    t.set_line_cap(T.CIRCLE)
    t.set_line_join(T.ROUNDED)
    t.set_line_dash([9.0, 5.0])
    t.set_line_dash_offset(3.0)
    t.set_line_width(3.0)
    t.set_color(T.STROKE_STYLE, 0.9, 0.2, 0.3, 0.9)
    t.begin_path()
    t.move_to(10.0, 100.0)
    t.bezier_curve_to(50.0, 60.0, 110.0, 140.0, 150.0, 90.0)
    t.stroke()
    t.set_line_dash(None, 0)
    t.set_font(font, 18.0)
    t.set_color(T.FILL_STYLE, 0.05, 0.05, 0.1, 1.0)
    t.set_text_align(2)       # center
    t.set_text_baseline(2)    # middle
    t.fill_text("Drop-in", 80.0, 20.0)
    t.set_text_align(1)       # rightward
    t.set_text_baseline(0)    # alphabetic
    t.set_line_width(1.0)
    t.set_color(T.STROKE_STYLE, 0.0, 0.5, 0.2, 1.0)
    t.stroke_text("GB300", 156.0, 116.0)
    t.save()
    t.set_global_composite_operation(T.LIGHTER)
    t.set_global_alpha(0.7)
    t.draw_image(img, 4, 4, 120.0, 40.0, 24.0, 20.0)
    t.restore()
    t.set_global_composite_operation(T.DESTINATION_OVER)
    t.set_color(T.FILL_STYLE, 0.95, 0.95, 0.9, 1.0)
    t.fill_rectangle(0.0, 0.0, float(w), float(h))
    t.get_image_data(w, h, 0, 0)
    t.get_image_data(30, 20, 140, 110)
    return t.finish(read_back=False)


def run_app(app, tmp_path, mode, data):
    src, out = tmp_path / "in.bin", tmp_path / "out.bin"
    src.write_bytes(data)
    subprocess.run([app, mode, str(src), str(out)], check=True, timeout=300)
    return out.read_bytes()


def check(trace, raw):
    """Bit for bit against the oracle computing the library's default (binned
    coverage, GPU stroke joins); within the contract against the oracle."""
    assert raw == oracle.replay(trace, ties="sign", trig="cr", coverage="binned")[0]
    got = G.split_images(trace, raw)
    want = G.split_images(trace, oracle.replay(trace)[0])
    for i, (g, w) in enumerate(zip(got, want)):
        G.assert_within_contract(g, w, f"read {i}")


@pytest.mark.gpu
def test_application_demo_matches_oracle(app, tmp_path):
    font = font_bytes()
    check(demo_trace(font), run_app(app, tmp_path, "demo", font))


@pytest.mark.gpu
@pytest.mark.parametrize("scene", ["c0", "c2_small"])
def test_application_replays_scene_like_oracle(app, tmp_path, scene):
    tb = scenes.CONFIGS["c0"]() if scene == "c0" else scenes.small_scene("c2_small", 0)
    check(tb, run_app(app, tmp_path, "replay", tb))
