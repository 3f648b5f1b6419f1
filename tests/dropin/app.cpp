// app.cpp -- an application written against the reference's public API
// (src/canvas_ity.hpp:142-1148), compiled against include/canvas_ity.hpp
// and linked with -lcanvas_ity_gb300 exactly as INTEGRATION.md tells an
// application to.  It is the drop-in check: nothing here knows about the GPU.
//
//   app replay <trace> <out>   replay a recorded call list through the class
//                              (every public method, via include/cy_replay.hpp)
//                              and write the get_image_data bytes to <out>
//   app demo <font> <out>      draw the scene below, which uses the public data
//                              members, the enums, text, draw_image, save and
//                              restore directly, and write its reads to <out>
//
// tests/test_dropin.py builds it, runs it and compares <out> with the oracle
// replaying the same calls (its mirror of `demo` is `demo_trace` there).

#include "canvas_ity.hpp"
#include "cy_replay.hpp"

#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace {

struct app_traits {
    typedef canvas_ity::canvas canvas_type;
    typedef canvas_ity::brush_type brush_type;
    typedef canvas_ity::composite_operation composite_operation;
    typedef canvas_ity::cap_style cap_style;
    typedef canvas_ity::join_style join_style;
    typedef canvas_ity::repetition_style repetition_style;
    typedef canvas_ity::align_style align_style;
    typedef canvas_ity::baseline_style baseline_style;
    static std::unique_ptr<canvas_type> make(int w, int h) {
        return std::unique_ptr<canvas_type>(new canvas_type(w, h));
    }
    static bool set_fill_rule(canvas_type &c, int rule) {
        if (rule != 0 && rule != 1) return false;
        c.set_fill_rule(rule ? canvas_ity::even_odd : canvas_ity::nonzero);
        return true;
    }
};

bool read_file(const char *path, std::vector<unsigned char> &out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    unsigned char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
    std::fclose(f);
    return true;
}

bool write_file(const char *path, const std::vector<unsigned char> &data) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return false;
    bool ok = data.empty() || std::fwrite(data.data(), 1, data.size(), f) == data.size();
    return std::fclose(f) == 0 && ok;
}

// 160 x 120: a clipped, shadowed gradient star over a pattern-filled
// rectangle, a dashed round-joined stroke, text in two alignments, a drawn
// image under save/restore and two composite operations.
int demo(const std::vector<unsigned char> &font, std::vector<unsigned char> &reads) {
    using namespace canvas_ity;
    const int w = 160, h = 120;
    canvas c(w, h);
    unsigned char checker[4 * 4 * 4];
    for (int i = 0; i < 16; ++i) {
        bool on = ((i & 3) + (i >> 2)) & 1;
        checker[4 * i + 0] = on ? 230 : 20;
        checker[4 * i + 1] = on ? 120 : 60;
        checker[4 * i + 2] = on ? 30 : 200;
        checker[4 * i + 3] = 255;
    }
    c.set_pattern(fill_style, checker, 4, 4, 16, repeat);
    c.fill_rectangle(4.0f, 4.0f, 70.0f, 50.0f);
    c.save();
    c.begin_path();
    c.arc(80.0f, 60.0f, 50.0f, 0.0f, 6.2831853f);
    c.clip();
    c.shadow_offset_x = 4.0f;
    c.shadow_offset_y = 3.0f;
    c.set_shadow_color(0.1f, 0.0f, 0.2f, 0.6f);
    c.set_shadow_blur(3.0f);
    c.set_linear_gradient(fill_style, 30.0f, 10.0f, 130.0f, 110.0f);
    c.add_color_stop(fill_style, 0.0f, 1.0f, 0.8f, 0.1f, 1.0f);
    c.add_color_stop(fill_style, 1.0f, 0.1f, 0.3f, 0.9f, 0.8f);
    static const float star[10][2] = {{80.0f, 14.0f},  {91.75f, 45.8f}, {125.65f, 47.15f}, {99.0f, 68.2f},
                                      {108.2f, 100.85f}, {80.0f, 82.0f}, {51.8f, 100.85f}, {61.0f, 68.2f},
                                      {34.35f, 47.15f}, {68.25f, 45.8f}};
    c.begin_path();
    c.move_to(star[0][0], star[0][1]);
    for (int i = 1; i < 10; ++i) c.line_to(star[i][0], star[i][1]);
    c.close_path();
    c.fill();
    c.restore();
    c.line_cap = circle;
    c.line_join = rounded;
    float dash[2] = {9.0f, 5.0f};
    c.set_line_dash(dash, 2);
    c.line_dash_offset = 3.0f;
    c.set_line_width(3.0f);
    c.set_color(stroke_style, 0.9f, 0.2f, 0.3f, 0.9f);
    c.begin_path();
    c.move_to(10.0f, 100.0f);
    c.bezier_curve_to(50.0f, 60.0f, 110.0f, 140.0f, 150.0f, 90.0f);
    c.stroke();
    c.set_line_dash(nullptr, 0);
    if (!c.set_font(font.data(), static_cast<int>(font.size()), 18.0f)) return 2;
    c.set_color(fill_style, 0.05f, 0.05f, 0.1f, 1.0f);
    c.text_align = center;
    c.text_baseline = middle;
    c.fill_text("Drop-in", 80.0f, 20.0f);
    c.text_align = rightward;
    c.text_baseline = alphabetic;
    c.set_line_width(1.0f);
    c.set_color(stroke_style, 0.0f, 0.5f, 0.2f, 1.0f);
    c.stroke_text("GB300", 156.0f, 116.0f);
    c.save();
    c.global_composite_operation = lighter;
    c.set_global_alpha(0.7f);
    c.draw_image(checker, 4, 4, 16, 120.0f, 40.0f, 24.0f, 20.0f);
    c.restore();
    c.global_composite_operation = destination_over;
    c.set_color(fill_style, 0.95f, 0.95f, 0.9f, 1.0f);
    c.fill_rectangle(0.0f, 0.0f, static_cast<float>(w), static_cast<float>(h));
    reads.resize(static_cast<size_t>(w) * h * 4 + 30 * 20 * 4);
    c.get_image_data(reads.data(), w, h, w * 4, 0, 0);
    c.get_image_data(reads.data() + static_cast<size_t>(w) * h * 4, 30, 20, 30 * 4, 140, 110);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s replay <trace> <out> | demo <font> <out>\n", argv[0]);
        return 1;
    }
    std::vector<unsigned char> in, out;
    if (!read_file(argv[2], in)) return 1;
    const std::string mode = argv[1];
    if (mode == "replay") {
        cy_trace::output o;
        if (cy_trace::replay<app_traits>(in.data(), in.size(), o) != 0) return 2;
        out = o.images;
    } else if (mode == "demo") {
        int rc = demo(in, out);
        if (rc) return rc;
    } else {
        return 1;
    }
    return write_file(argv[3], out) ? 0 : 1;
}
