// cy_replay.hpp -- replay driver for recorded canvas_ity call lists.
//
// Header-only.  `cy_trace::replay<Traits>()` walks a trace (format in
// cy_trace.h) and issues every recorded call on a canvas created through
// `Traits::make(width, height)`, so the same driver replays a trace through
// any class with the public canvas_ity::canvas API
// (reference: src/canvas_ity.hpp:194-1148).  Every non-null
// get_image_data call appends its compact RGBA8 rectangle to `images`;
// is_point_in_path and measure_text append their return value to `results`.
#ifndef CY_REPLAY_HPP
#define CY_REPLAY_HPP

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "cy_trace.h"

namespace cy_trace {

struct reader {
    const uint8_t *p;
    const uint8_t *end;
    bool ok;
    reader(const uint8_t *data, size_t size) : p(data), end(data + size), ok(true) {}
    bool need(size_t n) {
        if (!ok || static_cast<size_t>(end - p) < n) { ok = false; return false; }
        return true;
    }
    int32_t i32() {
        int32_t v = 0;
        if (need(4)) { std::memcpy(&v, p, 4); p += 4; }
        return v;
    }
    float f32() {
        float v = 0.0f;
        if (need(4)) { std::memcpy(&v, p, 4); p += 4; }
        return v;
    }
    const uint8_t *bytes(size_t n) {
        if (!need(n)) return nullptr;
        const uint8_t *at = p;
        p += n;
        return at;
    }
};

struct output {
    std::vector<uint8_t> images;
    std::vector<float> results;
};

// Returns 0 on success, -1 on a malformed or truncated trace.
template <class Traits>
int replay(const uint8_t *data, size_t size, output &out,
           std::unique_ptr<typename Traits::canvas_type> *keep = nullptr) {
    typedef typename Traits::canvas_type canvas_type;
    typedef typename Traits::brush_type brush_type;
    reader in(data, size);
    if (in.i32() != static_cast<int32_t>(CY_TRACE_MAGIC) || in.i32() != CY_TRACE_VERSION)
        return -1;
    std::unique_ptr<canvas_type> c;
    std::vector<uint8_t> scratch;
    std::vector<float> floats;
    std::vector<char> text;
    for (;;) {
        int32_t op = in.i32();
        if (!in.ok) return -1;
        if (op == CYT_END) break;
        if (op != CYT_CANVAS && !c) return -1;
        switch (op) {
        case CYT_CANVAS: {
            int32_t w = in.i32(), h = in.i32();
            if (!in.ok || w < 1 || h < 1 || w > 32768 || h > 32768) return -1;
            c.reset();
            c = Traits::make(w, h);
            break;
        }
        case CYT_SCALE: { float x = in.f32(), y = in.f32(); c->scale(x, y); break; }
        case CYT_ROTATE: { float a = in.f32(); c->rotate(a); break; }
        case CYT_TRANSLATE: { float x = in.f32(), y = in.f32(); c->translate(x, y); break; }
        case CYT_TRANSFORM:
        case CYT_SET_TRANSFORM: {
            float m[6];
            for (int i = 0; i < 6; ++i) m[i] = in.f32();
            if (op == CYT_TRANSFORM) c->transform(m[0], m[1], m[2], m[3], m[4], m[5]);
            else c->set_transform(m[0], m[1], m[2], m[3], m[4], m[5]);
            break;
        }
        case CYT_SET_GLOBAL_ALPHA: { float a = in.f32(); c->set_global_alpha(a); break; }
        case CYT_SET_COMPOSITE_OP:
            c->global_composite_operation =
                static_cast<typename Traits::composite_operation>(in.i32());
            break;
        case CYT_SET_SHADOW_COLOR: {
            float r = in.f32(), g = in.f32(), b = in.f32(), a = in.f32();
            c->set_shadow_color(r, g, b, a);
            break;
        }
        case CYT_SET_SHADOW_OFFSET_X: c->shadow_offset_x = in.f32(); break;
        case CYT_SET_SHADOW_OFFSET_Y: c->shadow_offset_y = in.f32(); break;
        case CYT_SET_SHADOW_BLUR: { float v = in.f32(); c->set_shadow_blur(v); break; }
        case CYT_SET_LINE_WIDTH: { float v = in.f32(); c->set_line_width(v); break; }
        case CYT_SET_LINE_CAP:
            c->line_cap = static_cast<typename Traits::cap_style>(in.i32());
            break;
        case CYT_SET_LINE_JOIN:
            c->line_join = static_cast<typename Traits::join_style>(in.i32());
            break;
        case CYT_SET_MITER_LIMIT: { float v = in.f32(); c->set_miter_limit(v); break; }
        case CYT_SET_LINE_DASH_OFFSET: c->line_dash_offset = in.f32(); break;
        case CYT_SET_LINE_DASH: {
            int32_t count = in.i32(), nonnull = in.i32();
            floats.clear();
            if (nonnull && count > 0)
                for (int32_t i = 0; i < count; ++i) floats.push_back(in.f32());
            if (!in.ok) return -1;
            // A null pointer with a positive count is legal and clears the dash.
            floats.push_back(0.0f);
            c->set_line_dash(nonnull ? floats.data() : nullptr, count);
            break;
        }
        case CYT_SET_COLOR: {
            brush_type t = static_cast<brush_type>(in.i32());
            float r = in.f32(), g = in.f32(), b = in.f32(), a = in.f32();
            c->set_color(t, r, g, b, a);
            break;
        }
        case CYT_SET_LINEAR_GRADIENT: {
            brush_type t = static_cast<brush_type>(in.i32());
            float v[4];
            for (int i = 0; i < 4; ++i) v[i] = in.f32();
            c->set_linear_gradient(t, v[0], v[1], v[2], v[3]);
            break;
        }
        case CYT_SET_RADIAL_GRADIENT: {
            brush_type t = static_cast<brush_type>(in.i32());
            float v[6];
            for (int i = 0; i < 6; ++i) v[i] = in.f32();
            c->set_radial_gradient(t, v[0], v[1], v[2], v[3], v[4], v[5]);
            break;
        }
        case CYT_ADD_COLOR_STOP: {
            brush_type t = static_cast<brush_type>(in.i32());
            float v[5];
            for (int i = 0; i < 5; ++i) v[i] = in.f32();
            c->add_color_stop(t, v[0], v[1], v[2], v[3], v[4]);
            break;
        }
        case CYT_SET_PATTERN: {
            brush_type t = static_cast<brush_type>(in.i32());
            int32_t w = in.i32(), h = in.i32(), rep = in.i32(), nonnull = in.i32();
            const uint8_t *px = nullptr;
            if (nonnull && w > 0 && h > 0) {
                px = in.bytes(static_cast<size_t>(w) * static_cast<size_t>(h) * 4u);
            } else if (nonnull) {
                scratch.assign(4, 0);
                px = scratch.data();
            }
            if (!in.ok) return -1;
            c->set_pattern(t, px, w, h, w * 4,
                           static_cast<typename Traits::repetition_style>(rep));
            break;
        }
        case CYT_BEGIN_PATH: c->begin_path(); break;
        case CYT_MOVE_TO: { float x = in.f32(), y = in.f32(); c->move_to(x, y); break; }
        case CYT_CLOSE_PATH: c->close_path(); break;
        case CYT_LINE_TO: { float x = in.f32(), y = in.f32(); c->line_to(x, y); break; }
        case CYT_QUADRATIC_CURVE_TO: {
            float v[4];
            for (int i = 0; i < 4; ++i) v[i] = in.f32();
            c->quadratic_curve_to(v[0], v[1], v[2], v[3]);
            break;
        }
        case CYT_BEZIER_CURVE_TO: {
            float v[6];
            for (int i = 0; i < 6; ++i) v[i] = in.f32();
            c->bezier_curve_to(v[0], v[1], v[2], v[3], v[4], v[5]);
            break;
        }
        case CYT_ARC_TO: {
            float v[5];
            for (int i = 0; i < 5; ++i) v[i] = in.f32();
            c->arc_to(v[0], v[1], v[2], v[3], v[4]);
            break;
        }
        case CYT_ARC: {
            float v[5];
            for (int i = 0; i < 5; ++i) v[i] = in.f32();
            int32_t ccw = in.i32();
            c->arc(v[0], v[1], v[2], v[3], v[4], ccw != 0);
            break;
        }
        case CYT_RECTANGLE:
        case CYT_CLEAR_RECTANGLE:
        case CYT_FILL_RECTANGLE:
        case CYT_STROKE_RECTANGLE: {
            float v[4];
            for (int i = 0; i < 4; ++i) v[i] = in.f32();
            if (op == CYT_RECTANGLE) c->rectangle(v[0], v[1], v[2], v[3]);
            else if (op == CYT_CLEAR_RECTANGLE) c->clear_rectangle(v[0], v[1], v[2], v[3]);
            else if (op == CYT_FILL_RECTANGLE) c->fill_rectangle(v[0], v[1], v[2], v[3]);
            else c->stroke_rectangle(v[0], v[1], v[2], v[3]);
            break;
        }
        case CYT_FILL: c->fill(); break;
        case CYT_STROKE: c->stroke(); break;
        case CYT_CLIP: c->clip(); break;
        case CYT_IS_POINT_IN_PATH: {
            float x = in.f32(), y = in.f32();
            in.i32();  // expected answer, compared by the caller
            out.results.push_back(c->is_point_in_path(x, y) ? 1.0f : 0.0f);
            break;
        }
        case CYT_SET_TEXT_ALIGN:
            c->text_align = static_cast<typename Traits::align_style>(in.i32());
            break;
        case CYT_SET_TEXT_BASELINE:
            c->text_baseline = static_cast<typename Traits::baseline_style>(in.i32());
            break;
        case CYT_SET_FONT: {
            int32_t bytes = in.i32(), nonnull = in.i32();
            float size_px = in.f32();
            const uint8_t *font = nullptr;
            if (nonnull && bytes > 0) font = in.bytes(static_cast<size_t>(bytes));
            else if (nonnull) { scratch.assign(4, 0); font = scratch.data(); }
            if (!in.ok) return -1;
            c->set_font(font, bytes, size_px);
            break;
        }
        case CYT_FILL_TEXT:
        case CYT_STROKE_TEXT: {
            float x = in.f32(), y = in.f32(), maxw = in.f32();
            int32_t nonnull = in.i32(), len = in.i32();
            if (len < 0) return -1;
            const uint8_t *s = in.bytes(static_cast<size_t>(len));
            if (!in.ok) return -1;
            text.assign(reinterpret_cast<const char *>(s), reinterpret_cast<const char *>(s) + len);
            text.push_back('\0');
            if (op == CYT_FILL_TEXT) c->fill_text(nonnull ? text.data() : nullptr, x, y, maxw);
            else c->stroke_text(nonnull ? text.data() : nullptr, x, y, maxw);
            break;
        }
        case CYT_MEASURE_TEXT: {
            int32_t nonnull = in.i32(), len = in.i32();
            if (len < 0) return -1;
            const uint8_t *s = in.bytes(static_cast<size_t>(len));
            in.f32();  // expected answer, compared by the caller
            if (!in.ok) return -1;
            text.assign(reinterpret_cast<const char *>(s), reinterpret_cast<const char *>(s) + len);
            text.push_back('\0');
            out.results.push_back(c->measure_text(nonnull ? text.data() : nullptr));
            break;
        }
        case CYT_DRAW_IMAGE: {
            int32_t w = in.i32(), h = in.i32(), nonnull = in.i32();
            float v[4];
            for (int i = 0; i < 4; ++i) v[i] = in.f32();
            const uint8_t *px = nullptr;
            if (nonnull && w > 0 && h > 0)
                px = in.bytes(static_cast<size_t>(w) * static_cast<size_t>(h) * 4u);
            else if (nonnull) { scratch.assign(4, 0); px = scratch.data(); }
            if (!in.ok) return -1;
            c->draw_image(px, w, h, w * 4, v[0], v[1], v[2], v[3]);
            break;
        }
        case CYT_GET_IMAGE_DATA: {
            int32_t w = in.i32(), h = in.i32(), x = in.i32(), y = in.i32();
            int32_t nonnull = in.i32(), has_expected = in.i32();
            if (has_expected && w > 0 && h > 0)
                in.bytes(static_cast<size_t>(w) * static_cast<size_t>(h) * 4u);
            if (!in.ok) return -1;
            if (!nonnull) {
                scratch.assign(4, 0);
                c->get_image_data(nullptr, w, h, w * 4, x, y);
            } else if (w > 0 && h > 0) {
                size_t at = out.images.size();
                out.images.resize(at + static_cast<size_t>(w) * static_cast<size_t>(h) * 4u);
                c->get_image_data(out.images.data() + at, w, h, w * 4, x, y);
            } else {
                scratch.assign(4, 0);
                c->get_image_data(scratch.data(), w, h, w * 4, x, y);
            }
            break;
        }
        case CYT_PUT_IMAGE_DATA: {
            int32_t w = in.i32(), h = in.i32(), x = in.i32(), y = in.i32();
            int32_t nonnull = in.i32();
            const uint8_t *px = nullptr;
            if (nonnull && w > 0 && h > 0)
                px = in.bytes(static_cast<size_t>(w) * static_cast<size_t>(h) * 4u);
            else if (nonnull) { scratch.assign(4, 0); px = scratch.data(); }
            if (!in.ok) return -1;
            c->put_image_data(px, w, h, w * 4, x, y);
            break;
        }
        case CYT_SET_FILL_RULE: {
            int32_t rule = in.i32();
            if (!in.ok || !Traits::set_fill_rule(*c, rule)) return -1;
            break;
        }
        case CYT_SAVE: c->save(); break;
        case CYT_RESTORE: c->restore(); break;
        default:
            return -1;
        }
        if (!in.ok) return -1;
    }
    if (keep) *keep = std::move(c);
    return 0;
}

// Shared body of the `<prefix>_replay` C entry points.  Copies the outputs
// into caller buffers; returns -2 (and the needed sizes) when they are short.
template <class Traits>
int replay_to_buffers(const void *trace, size_t trace_len, void *images, size_t images_cap,
                      size_t *images_len, float *results, int results_cap, int *results_len) {
    output out;
    int rc = replay<Traits>(static_cast<const uint8_t *>(trace), trace_len, out);
    if (images_len) *images_len = out.images.size();
    if (results_len) *results_len = static_cast<int>(out.results.size());
    if (rc != 0) return rc;
    if (out.images.size() > images_cap || static_cast<int>(out.results.size()) > results_cap)
        return -2;
    if (!out.images.empty()) std::memcpy(images, out.images.data(), out.images.size());
    if (!out.results.empty())
        std::memcpy(results, out.results.data(), out.results.size() * sizeof(float));
    return 0;
}

}  // namespace cy_trace

#endif  // CY_REPLAY_HPP
