// recorder.cpp -- records the reference test suite's calls into call lists.
//
// TEST INFRASTRUCTURE ONLY (golden-fixture generation, runs only where the
// reference sources are present).  The reference header is compiled here
// under the namespace `canvas_ity_ref`; every call on the recording canvas
// (recorder.hpp) is appended to a call list and forwarded to a reference
// canvas, so get_image_data / is_point_in_path / measure_text inside a test
// see the reference's real answers, which are stored in the call list as the
// expected values.  Each canvas writes its call list to
// $CY_RECORD_DIR/trace_NNN.bin when it is destroyed.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#define canvas_ity canvas_ity_ref
#define CANVAS_ITY_IMPLEMENTATION
#include CY_REFERENCE_HEADER
#undef CANVAS_ITY_IMPLEMENTATION
#undef canvas_ity

#include "recorder.hpp"
#include "../../include/cy_trace.h"

namespace canvas_ity {

static int g_serial = 0;

struct canvas::impl {
    canvas_ity_ref::canvas ref;
    std::vector<uint8_t> out;
    int serial;
    composite_operation op;
    float sox, soy, dash_off;
    cap_style cap;
    join_style join;
    align_style align;
    baseline_style baseline;
    impl(int w, int h) : ref(w, h), serial(g_serial++) {}
    void i32(int32_t v) { uint8_t b[4]; std::memcpy(b, &v, 4); out.insert(out.end(), b, b + 4); }
    void f32(float v) { uint8_t b[4]; std::memcpy(b, &v, 4); out.insert(out.end(), b, b + 4); }
    void raw(const uint8_t *p, size_t n) { out.insert(out.end(), p, p + n); }
    void rows(const unsigned char *img, int w, int h, int stride) {
        for (int y = 0; y < h; ++y) raw(img + static_cast<ptrdiff_t>(y) * stride, static_cast<size_t>(w) * 4u);
    }
};

canvas::canvas(int width, int height)
    : global_composite_operation(source_over), shadow_offset_x(0.0f), shadow_offset_y(0.0f),
      line_cap(butt), line_join(miter), line_dash_offset(0.0f), text_align(start),
      text_baseline(alphabetic), self(new impl(width, height)) {
    self->i32(static_cast<int32_t>(CY_TRACE_MAGIC));
    self->i32(CY_TRACE_VERSION);
    self->i32(CYT_CANVAS);
    self->i32(width);
    self->i32(height);
    self->op = global_composite_operation;
    self->sox = shadow_offset_x;
    self->soy = shadow_offset_y;
    self->cap = line_cap;
    self->join = line_join;
    self->dash_off = line_dash_offset;
    self->align = text_align;
    self->baseline = text_baseline;
}

canvas::~canvas() {
    self->i32(CYT_END);
    const char *dir = std::getenv("CY_RECORD_DIR");
    if (dir) {
        char name[64];
        std::snprintf(name, sizeof(name), "/trace_%03d.bin", self->serial);
        std::string path = std::string(dir) + name;
        FILE *f = std::fopen(path.c_str(), "wb");
        if (f) {
            std::fwrite(self->out.data(), 1, self->out.size(), f);
            std::fclose(f);
        }
    }
    delete self;
}

// Record changes of the public data members and push them to the reference.
void canvas::sync() {
    impl &s = *self;
    if (global_composite_operation != s.op) {
        s.i32(CYT_SET_COMPOSITE_OP); s.i32(global_composite_operation); s.op = global_composite_operation;
    }
    if (std::memcmp(&shadow_offset_x, &s.sox, 4)) {
        s.i32(CYT_SET_SHADOW_OFFSET_X); s.f32(shadow_offset_x); s.sox = shadow_offset_x;
    }
    if (std::memcmp(&shadow_offset_y, &s.soy, 4)) {
        s.i32(CYT_SET_SHADOW_OFFSET_Y); s.f32(shadow_offset_y); s.soy = shadow_offset_y;
    }
    if (line_cap != s.cap) { s.i32(CYT_SET_LINE_CAP); s.i32(line_cap); s.cap = line_cap; }
    if (line_join != s.join) { s.i32(CYT_SET_LINE_JOIN); s.i32(line_join); s.join = line_join; }
    if (std::memcmp(&line_dash_offset, &s.dash_off, 4)) {
        s.i32(CYT_SET_LINE_DASH_OFFSET); s.f32(line_dash_offset); s.dash_off = line_dash_offset;
    }
    if (text_align != s.align) { s.i32(CYT_SET_TEXT_ALIGN); s.i32(text_align); s.align = text_align; }
    if (text_baseline != s.baseline) {
        s.i32(CYT_SET_TEXT_BASELINE); s.i32(text_baseline); s.baseline = text_baseline;
    }
    s.ref.global_composite_operation = static_cast<canvas_ity_ref::composite_operation>(global_composite_operation);
    s.ref.shadow_offset_x = shadow_offset_x;
    s.ref.shadow_offset_y = shadow_offset_y;
    s.ref.line_cap = static_cast<canvas_ity_ref::cap_style>(line_cap);
    s.ref.line_join = static_cast<canvas_ity_ref::join_style>(line_join);
    s.ref.line_dash_offset = line_dash_offset;
    s.ref.text_align = static_cast<canvas_ity_ref::align_style>(text_align);
    s.ref.text_baseline = static_cast<canvas_ity_ref::baseline_style>(text_baseline);
}

#define REC0(OP) sync(); self->i32(OP)
#define BT(t) static_cast<canvas_ity_ref::brush_type>(t)

void canvas::scale(float x, float y) { REC0(CYT_SCALE); self->f32(x); self->f32(y); self->ref.scale(x, y); }
void canvas::rotate(float a) { REC0(CYT_ROTATE); self->f32(a); self->ref.rotate(a); }
void canvas::translate(float x, float y) {
    REC0(CYT_TRANSLATE); self->f32(x); self->f32(y); self->ref.translate(x, y);
}
void canvas::transform(float a, float b, float c, float d, float e, float f) {
    REC0(CYT_TRANSFORM);
    self->f32(a); self->f32(b); self->f32(c); self->f32(d); self->f32(e); self->f32(f);
    self->ref.transform(a, b, c, d, e, f);
}
void canvas::set_transform(float a, float b, float c, float d, float e, float f) {
    REC0(CYT_SET_TRANSFORM);
    self->f32(a); self->f32(b); self->f32(c); self->f32(d); self->f32(e); self->f32(f);
    self->ref.set_transform(a, b, c, d, e, f);
}
void canvas::set_global_alpha(float a) { REC0(CYT_SET_GLOBAL_ALPHA); self->f32(a); self->ref.set_global_alpha(a); }
void canvas::set_shadow_color(float r, float g, float b, float a) {
    REC0(CYT_SET_SHADOW_COLOR); self->f32(r); self->f32(g); self->f32(b); self->f32(a);
    self->ref.set_shadow_color(r, g, b, a);
}
void canvas::set_shadow_blur(float v) { REC0(CYT_SET_SHADOW_BLUR); self->f32(v); self->ref.set_shadow_blur(v); }
void canvas::set_line_width(float v) { REC0(CYT_SET_LINE_WIDTH); self->f32(v); self->ref.set_line_width(v); }
void canvas::set_miter_limit(float v) { REC0(CYT_SET_MITER_LIMIT); self->f32(v); self->ref.set_miter_limit(v); }
void canvas::set_line_dash(float const *segments, int count) {
    REC0(CYT_SET_LINE_DASH);
    self->i32(count);
    self->i32(segments ? 1 : 0);
    if (segments && count > 0)
        for (int i = 0; i < count; ++i) self->f32(segments[i]);
    self->ref.set_line_dash(segments, count);
}
void canvas::set_color(brush_type t, float r, float g, float b, float a) {
    REC0(CYT_SET_COLOR); self->i32(t); self->f32(r); self->f32(g); self->f32(b); self->f32(a);
    self->ref.set_color(BT(t), r, g, b, a);
}
void canvas::set_linear_gradient(brush_type t, float x0, float y0, float x1, float y1) {
    REC0(CYT_SET_LINEAR_GRADIENT); self->i32(t);
    self->f32(x0); self->f32(y0); self->f32(x1); self->f32(y1);
    self->ref.set_linear_gradient(BT(t), x0, y0, x1, y1);
}
void canvas::set_radial_gradient(brush_type t, float x0, float y0, float r0, float x1, float y1, float r1) {
    REC0(CYT_SET_RADIAL_GRADIENT); self->i32(t);
    self->f32(x0); self->f32(y0); self->f32(r0); self->f32(x1); self->f32(y1); self->f32(r1);
    self->ref.set_radial_gradient(BT(t), x0, y0, r0, x1, y1, r1);
}
void canvas::add_color_stop(brush_type t, float o, float r, float g, float b, float a) {
    REC0(CYT_ADD_COLOR_STOP); self->i32(t);
    self->f32(o); self->f32(r); self->f32(g); self->f32(b); self->f32(a);
    self->ref.add_color_stop(BT(t), o, r, g, b, a);
}
void canvas::set_pattern(brush_type t, unsigned char const *img, int w, int h, int stride, repetition_style rep) {
    REC0(CYT_SET_PATTERN); self->i32(t); self->i32(w); self->i32(h); self->i32(rep); self->i32(img ? 1 : 0);
    if (img && w > 0 && h > 0) self->rows(img, w, h, stride);
    self->ref.set_pattern(BT(t), img, w, h, stride, static_cast<canvas_ity_ref::repetition_style>(rep));
}
void canvas::begin_path() { REC0(CYT_BEGIN_PATH); self->ref.begin_path(); }
void canvas::move_to(float x, float y) { REC0(CYT_MOVE_TO); self->f32(x); self->f32(y); self->ref.move_to(x, y); }
void canvas::close_path() { REC0(CYT_CLOSE_PATH); self->ref.close_path(); }
void canvas::line_to(float x, float y) { REC0(CYT_LINE_TO); self->f32(x); self->f32(y); self->ref.line_to(x, y); }
void canvas::quadratic_curve_to(float cx, float cy, float x, float y) {
    REC0(CYT_QUADRATIC_CURVE_TO); self->f32(cx); self->f32(cy); self->f32(x); self->f32(y);
    self->ref.quadratic_curve_to(cx, cy, x, y);
}
void canvas::bezier_curve_to(float a, float b, float c, float d, float x, float y) {
    REC0(CYT_BEZIER_CURVE_TO);
    self->f32(a); self->f32(b); self->f32(c); self->f32(d); self->f32(x); self->f32(y);
    self->ref.bezier_curve_to(a, b, c, d, x, y);
}
void canvas::arc_to(float vx, float vy, float x, float y, float r) {
    REC0(CYT_ARC_TO); self->f32(vx); self->f32(vy); self->f32(x); self->f32(y); self->f32(r);
    self->ref.arc_to(vx, vy, x, y, r);
}
void canvas::arc(float x, float y, float r, float a0, float a1, bool ccw) {
    REC0(CYT_ARC); self->f32(x); self->f32(y); self->f32(r); self->f32(a0); self->f32(a1); self->i32(ccw ? 1 : 0);
    self->ref.arc(x, y, r, a0, a1, ccw);
}
void canvas::rectangle(float x, float y, float w, float h) {
    REC0(CYT_RECTANGLE); self->f32(x); self->f32(y); self->f32(w); self->f32(h);
    self->ref.rectangle(x, y, w, h);
}
void canvas::fill() { REC0(CYT_FILL); self->ref.fill(); }
void canvas::stroke() { REC0(CYT_STROKE); self->ref.stroke(); }
void canvas::clip() { REC0(CYT_CLIP); self->ref.clip(); }
bool canvas::is_point_in_path(float x, float y) {
    REC0(CYT_IS_POINT_IN_PATH); self->f32(x); self->f32(y);
    bool inside = self->ref.is_point_in_path(x, y);
    self->i32(inside ? 1 : 0);
    return inside;
}
void canvas::clear_rectangle(float x, float y, float w, float h) {
    REC0(CYT_CLEAR_RECTANGLE); self->f32(x); self->f32(y); self->f32(w); self->f32(h);
    self->ref.clear_rectangle(x, y, w, h);
}
void canvas::fill_rectangle(float x, float y, float w, float h) {
    REC0(CYT_FILL_RECTANGLE); self->f32(x); self->f32(y); self->f32(w); self->f32(h);
    self->ref.fill_rectangle(x, y, w, h);
}
void canvas::stroke_rectangle(float x, float y, float w, float h) {
    REC0(CYT_STROKE_RECTANGLE); self->f32(x); self->f32(y); self->f32(w); self->f32(h);
    self->ref.stroke_rectangle(x, y, w, h);
}
bool canvas::set_font(unsigned char const *font, int bytes, float size) {
    REC0(CYT_SET_FONT); self->i32(bytes); self->i32(font ? 1 : 0); self->f32(size);
    if (font && bytes > 0) self->raw(font, static_cast<size_t>(bytes));
    return self->ref.set_font(font, bytes, size);
}
static void record_text(std::vector<uint8_t> &out, const char *text) {
    int32_t n = text ? static_cast<int32_t>(std::strlen(text)) : 0;
    int32_t nonnull = text ? 1 : 0;
    uint8_t b[4];
    std::memcpy(b, &nonnull, 4); out.insert(out.end(), b, b + 4);
    std::memcpy(b, &n, 4); out.insert(out.end(), b, b + 4);
    if (n) out.insert(out.end(), reinterpret_cast<const uint8_t *>(text), reinterpret_cast<const uint8_t *>(text) + n);
}
void canvas::fill_text(char const *text, float x, float y, float maxw) {
    REC0(CYT_FILL_TEXT); self->f32(x); self->f32(y); self->f32(maxw); record_text(self->out, text);
    self->ref.fill_text(text, x, y, maxw);
}
void canvas::stroke_text(char const *text, float x, float y, float maxw) {
    REC0(CYT_STROKE_TEXT); self->f32(x); self->f32(y); self->f32(maxw); record_text(self->out, text);
    self->ref.stroke_text(text, x, y, maxw);
}
float canvas::measure_text(char const *text) {
    REC0(CYT_MEASURE_TEXT); record_text(self->out, text);
    float w = self->ref.measure_text(text);
    self->f32(w);
    return w;
}
void canvas::draw_image(unsigned char const *img, int w, int h, int stride, float x, float y, float tw, float th) {
    REC0(CYT_DRAW_IMAGE); self->i32(w); self->i32(h); self->i32(img ? 1 : 0);
    self->f32(x); self->f32(y); self->f32(tw); self->f32(th);
    if (img && w > 0 && h > 0) self->rows(img, w, h, stride);
    self->ref.draw_image(img, w, h, stride, x, y, tw, th);
}
void canvas::get_image_data(unsigned char *img, int w, int h, int stride, int x, int y) {
    REC0(CYT_GET_IMAGE_DATA); self->i32(w); self->i32(h); self->i32(x); self->i32(y); self->i32(img ? 1 : 0);
    self->ref.get_image_data(img, w, h, stride, x, y);
    bool has = img && w > 0 && h > 0;
    self->i32(has ? 1 : 0);
    if (has) self->rows(img, w, h, stride);
}
void canvas::put_image_data(unsigned char const *img, int w, int h, int stride, int x, int y) {
    REC0(CYT_PUT_IMAGE_DATA); self->i32(w); self->i32(h); self->i32(x); self->i32(y); self->i32(img ? 1 : 0);
    if (img && w > 0 && h > 0) self->rows(img, w, h, stride);
    self->ref.put_image_data(img, w, h, stride, x, y);
}
void canvas::save() { REC0(CYT_SAVE); self->ref.save(); }
void canvas::restore() {
    REC0(CYT_RESTORE);
    self->ref.restore();
    // The reference restores its public members; mirror them without recording.
    impl &s = *self;
    global_composite_operation = static_cast<composite_operation>(s.ref.global_composite_operation);
    shadow_offset_x = s.ref.shadow_offset_x;
    shadow_offset_y = s.ref.shadow_offset_y;
    line_cap = static_cast<cap_style>(s.ref.line_cap);
    line_join = static_cast<join_style>(s.ref.line_join);
    line_dash_offset = s.ref.line_dash_offset;
    text_align = static_cast<align_style>(s.ref.text_align);
    text_baseline = static_cast<baseline_style>(s.ref.text_baseline);
    s.op = global_composite_operation;
    s.sox = shadow_offset_x;
    s.soy = shadow_offset_y;
    s.cap = line_cap;
    s.join = line_join;
    s.dash_off = line_dash_offset;
    s.align = text_align;
    s.baseline = text_baseline;
}

}  // namespace canvas_ity

// The reference test program's main() is compiled renamed to cy_test_main.
int cy_test_main(int argc, char **argv);
int main(int argc, char **argv) { return cy_test_main(argc, argv); }
