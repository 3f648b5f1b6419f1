// canvas.cpp -- host side of the drop-in canvas_ity::canvas.
//
// Keeps the canvas state the reference keeps (src/canvas_ity.hpp:1150-1172),
// builds paths in device space exactly as the reference does, and performs
// the host-side geometry the reference performs before scan conversion for
// strokes and text: stroke-mode flattening, dashing, stroke expansion and
// TrueType outlines.  Every draw is then handed to the GPU engine
// (include/cy_gpu.h): fills and clips as Bezier paths (flattened on the
// GPU), everything else as polylines.
//
// The float arithmetic mirrors the reference operation for operation (this
// file is compiled with -ffp-contract=off) so that host-produced geometry is
// identical to the reference's.  Citations: hpp = src/canvas_ity.hpp.
//
// Derived from canvas_ity (src/canvas_ity.hpp), Copyright (c) 2022 Andrew
// Kensler, under the ISC license; its copyright and permission notice is
// reproduced in LICENSES/canvas_ity-ISC.txt and applies to this file.

#include "../../include/canvas_ity.hpp"
#include "../../include/cy_gpu.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <unordered_map>
#include <vector>

namespace canvas_ity {
namespace detail {

// std::min / std::max semantics, kept explicit (NaN ordering matters).
static inline float lo(float a, float b) { return b < a ? b : a; }
static inline float hi(float a, float b) { return a < b ? b : a; }

struct v2 { float x, y; };
static inline v2 mk(float x, float y) { v2 v; v.x = x; v.y = y; return v; }
static inline v2 add(v2 a, v2 b) { return mk(a.x + b.x, a.y + b.y); }
static inline v2 sub(v2 a, v2 b) { return mk(a.x - b.x, a.y - b.y); }
static inline v2 scl(float s, v2 a) { return mk(a.x * s, a.y * s); }
static inline float dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float norm(v2 a) { return sqrtf(dot(a, a)); }
static inline v2 unit(v2 a) { return scl(1.0f / hi(1.0e-6f, norm(a)), a); }
static inline v2 perp(v2 a) { return mk(-a.y, a.x); }
static inline v2 mix(v2 a, v2 b, float t) { return add(a, scl(t, sub(b, a))); }

struct affine { float a, b, c, d, e, f; };
static inline v2 apply(const affine &m, v2 p) {
    return mk(m.a * p.x + m.c * p.y + m.e, m.b * p.x + m.d * p.y + m.f);
}

struct rgba4 { float r, g, b, a; };

// Colour conversions of the reference (hpp:1273-1297).
static inline float linearized(float v) {
    return v < 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
}
static inline float clamp01(float v) { return lo(hi(v, 0.0f), 1.0f); }
static inline rgba4 clamped_linear(float r, float g, float b, float a) {
    rgba4 c = {linearized(clamp01(r)), linearized(clamp01(g)), linearized(clamp01(b)), clamp01(a)};
    return c;
}
static inline rgba4 premultiplied(rgba4 c) {
    rgba4 o = {c.r * c.a, c.g * c.a, c.b * c.a, c.a};
    return o;
}

struct subpath { size_t count; bool closed; };
struct polyline { std::vector<v2> pts; std::vector<subpath> subs; };

// paint_brush (hpp:165-168).  Pattern pixels are kept as the caller's sRGB
// bytes; the GPU linearises and premultiplies them.
struct brush {
    int kind;  // cy_paint_kind; CY_PAINT_NONE is never stored here
    std::vector<rgba4> colors;  // solid: premultiplied linear; gradient: straight linear stops
    std::vector<float> stops;
    v2 p0, p1;
    float r0, r1;
    std::vector<unsigned char> pixels;
    int w, h, rep;
    brush() : kind(CY_PAINT_SOLID), p0(mk(0, 0)), p1(mk(0, 0)), r0(0), r1(0), w(0), h(0), rep(0) {}
};

struct font_face {
    std::vector<unsigned char> data;
    int cmap, glyf, head, hhea, hmtx, loca, maxp, os_2;
    float scale;
    uint64_t hash;   // of the loaded tables (the glyph cache's key)
    font_face() : cmap(0), glyf(0), head(0), hhea(0), hmtx(0), loca(0), maxp(0), os_2(0), scale(0), hash(0) {}
};

struct saved_state {
    composite_operation op; float sox, soy; cap_style cap; join_style join; float dash_off;
    align_style align; baseline_style baseline; affine fwd, inv; float alpha; rgba4 shcol;
    float shblur, lw, miter_limit; std::vector<float> dash; brush fill, stroke; int mask; font_face face;
};

struct canvas_state {
    int W, H;
    cy_ctx *ctx;
    int status;
    affine fwd, inv;
    float alpha;
    rgba4 shadow_color;
    float shadow_blur;
    float lw, miter_limit;
    std::vector<float> dash;
    brush fill, stroke, image;
    polyline path, lines, scratch;
    int mask;  // current clip mask id (0 = whole canvas)
    bool even_odd = false;   // fill rule of fill(), clip(), is_point_in_path() (extension)
    font_face face;
    std::vector<saved_state> stack;
    // copies of the public members, refreshed before each draw
    composite_operation op;
    float sox, soy, dash_off;
    cap_style cap;
    join_style join;
    align_style align;
    baseline_style baseline;
    std::vector<int> counts;  // scratch for subpath counts
    std::vector<int> closed_flags;
    std::vector<float> stop_colors;

    void note(int rc) { if (rc < 0 && status == 0) status = rc; }
    void transform(float a, float b, float c, float d, float e, float f);
    void set_transform(float a, float b, float c, float d, float e, float f);
    void tessellate(v2 p1, v2 c1, v2 c2, v2 p2, float angular, int limit);
    void bezier(v2 p1, v2 c1, v2 c2, v2 p2, float angular);
    void flatten(bool stroking);
    void apply_dash();
    void half_stroke(size_t begin, size_t end, bool closed);
    void stroke_outline();
    void glyph_outline(int glyph, float angular);
    // Glyph outlines into `path` as cubic control points (lines as
    // degenerate cubics) instead of flattening them into `lines`: what the
    // device stroke expansion takes (set while stroke_text builds them).
    bool outline_cubics = false;
    int glyph_of(const char *text, int &index);
    void text_outline(const char *text, v2 at, float maxw, bool stroking);
    float measure(const char *text);
    bool singular() const { return fwd.a * fwd.d - fwd.b * fwd.c == 0.0f; }
    void make_paint(const brush &br, bool clamp_edges, bool force_solid, cy_paint &p);
    void make_state(cy_draw_state &s, bool with_shadow);
    void draw_lines(const brush &br, bool clamp_edges, bool force_solid, bool with_shadow);
    void draw_path(const brush &br, bool with_rule = true);
    void stroke_path(const brush &br);
    void line_to(float x, float y);
    void move_to(float x, float y);
};

void canvas_state::set_transform(float a, float b, float c, float d, float e, float f) {
    // hpp:2694-2711
    float det = a * d - b * c;
    float s = det != 0.0f ? 1.0f / det : 0.0f;
    affine nf = {a, b, c, d, e, f};
    affine ni = {s * d, s * -b, s * -c, s * a, s * (c * f - d * e), s * (b * e - a * f)};
    fwd = nf;
    inv = ni;
}
void canvas_state::transform(float a, float b, float c, float d, float e, float f) {
    // hpp:2680-2692
    set_transform(fwd.a * a + fwd.c * b, fwd.b * a + fwd.d * b, fwd.a * c + fwd.c * d,
                  fwd.b * c + fwd.d * d, fwd.a * e + fwd.c * f + fwd.e, fwd.b * e + fwd.d * f + fwd.f);
}

void canvas_state::move_to(float x, float y) {
    // hpp:2871-2882
    if (!path.subs.empty() && path.subs.back().count == 1) {
        path.pts.back() = apply(fwd, mk(x, y));
        return;
    }
    subpath s = {1, false};
    path.pts.push_back(apply(fwd, mk(x, y)));
    path.subs.push_back(s);
}
void canvas_state::line_to(float x, float y) {
    // hpp:2898-2916: lines are stored as degenerate cubics (p1, p2, p2)
    if (path.subs.empty()) { move_to(x, y); return; }
    v2 p1 = path.pts.back();
    v2 p2 = apply(fwd, mk(x, y));
    if (dot(sub(p2, p1), sub(p2, p1)) == 0.0f) return;
    path.pts.push_back(p1);
    path.pts.push_back(p2);
    path.pts.push_back(p2);
    path.subs.back().count += 3;
}

// ---- stroke-mode flattening on the host (hpp:1331-1524) ----
void canvas_state::tessellate(v2 p1, v2 c1, v2 c2, v2 p2, float angular, int limit) {
    const float tol = 0.125f;
    float flat = tol * tol;
    v2 e1 = sub(c1, p1), e2 = sub(c2, c1), e3 = sub(p2, c2), seg = sub(p2, p1);
    float q1 = dot(e1, e1), q2 = dot(e2, e2), q3 = dot(e3, e3);
    float lsq = hi(1.0e-4f, dot(seg, seg));
    float t1 = lo(hi(dot(e1, seg) / lsq, 0.0f), 1.0f);
    float t2 = lo(hi(dot(e3, seg) / lsq, 0.0f), 1.0f);
    v2 d1 = sub(add(p1, scl(t1, seg)), c1);
    v2 d2 = sub(sub(p2, scl(t2, seg)), c2);
    float cosine = 1.0f;
    if (angular > -1.0f) {
        if (q1 * q3 != 0.0f) cosine = dot(e1, e3) / sqrtf(q1 * q3);
        else if (q1 * q2 != 0.0f) cosine = dot(e1, e2) / sqrtf(q1 * q2);
        else if (q2 * q3 != 0.0f) cosine = dot(e2, e3) / sqrtf(q2 * q3);
    }
    if ((dot(d1, d1) <= flat && dot(d2, d2) <= flat && cosine >= angular) || !limit) {
        if (angular > -1.0f && q1 != 0.0f) lines.pts.push_back(c1);
        if (angular > -1.0f && q2 != 0.0f) lines.pts.push_back(c2);
        if (angular == -1.0f || q3 != 0.0f) lines.pts.push_back(p2);
        return;
    }
    v2 l1 = mix(p1, c1, 0.5f), m = mix(c1, c2, 0.5f), r2 = mix(c2, p2, 0.5f);
    v2 l2 = mix(l1, m, 0.5f), r1 = mix(m, r2, 0.5f), sp = mix(l2, r1, 0.5f);
    tessellate(p1, l1, l2, sp, angular, limit - 1);
    tessellate(sp, r1, r2, p2, angular, limit - 1);
}

static void extrema_of(float a, float b, float c, float *at, int &cuts) {
    // hpp:1420-1447: roots of one coordinate's derivative
    const float eps = 1.0e-4f;
    if (fabsf(a) > eps) {
        float disc = b * b - 4.0f * a * c;
        if (disc >= 0.0f) {
            float sign = b > 0.0f ? 1.0f : -1.0f;
            float term = -b - sign * sqrtf(disc);
            float r1 = term / (2.0f * a);
            at[cuts++] = r1;
            at[cuts++] = c / (a * r1);
        }
    } else if (fabsf(b) > eps) {
        at[cuts++] = -c / b;
    }
}

void canvas_state::bezier(v2 p1, v2 c1, v2 c2, v2 p2, float angular) {
    // hpp:1398-1487
    v2 e1 = sub(c1, p1), e2 = sub(c2, c1), e3 = sub(p2, c2);
    if (dot(e1, e1) == 0.0f && dot(e3, e3) == 0.0f) {
        lines.pts.push_back(p2);
        return;
    }
    float at[7] = {0.0f, 1.0f};
    int cuts = 2;
    v2 ea = add(scl(-9.0f, e2), scl(3.0f, sub(p2, p1)));
    v2 eb = sub(scl(6.0f, add(p1, c2)), scl(12.0f, c1));
    v2 ec = scl(3.0f, e1);
    extrema_of(ea.x, eb.x, ec.x, at, cuts);
    extrema_of(ea.y, eb.y, ec.y, at, cuts);
    float k1 = dot(perp(e1), e2), k2 = dot(perp(e1), e3), k3 = dot(perp(e2), e3);
    float ca = k1 - k2 + k3, cb = -2.0f * k1 + k2;
    if (fabsf(ca) > 1.0e-4f && fabsf(cb) > 1.0e-4f) at[cuts++] = -0.5f * cb / ca;
    for (int i = 1; i < cuts; ++i) {
        float v = at[i];
        int j = i - 1;
        for (; 0 <= j && v < at[j]; --j) at[j + 1] = at[j];
        at[j + 1] = v;
    }
    v2 s1 = p1;
    for (int i = 0; i < cuts - 1; ++i) {
        if (!(0.0f <= at[i] && at[i + 1] <= 1.0f && at[i] != at[i + 1])) continue;
        float t = at[i + 1], ratio = at[i] / t;
        v2 q1 = mix(p1, c1, t), q2 = mix(c1, c2, t), q3 = mix(c2, p2, t);
        v2 q4 = mix(q1, q2, t), q5 = mix(q2, q3, t), q6 = mix(q1, q4, ratio);
        v2 s2 = mix(q4, q5, t);
        v2 sc2 = mix(q4, s2, ratio);
        v2 sc1 = mix(q6, sc2, ratio);
        tessellate(s1, sc1, sc2, s2, angular, 20);
        s1 = s2;
    }
}

void canvas_state::flatten(bool stroking) {
    // hpp:1495-1524
    const float tol = 0.125f;
    float ratio = tol / hi(0.5f * lw, tol);
    float angular = stroking ? (ratio - 2.0f) * ratio * 2.0f + 1.0f : -1.0f;
    lines.pts.clear();
    lines.subs.clear();
    size_t i = 0, end = 0;
    for (size_t s = 0; s < path.subs.size(); ++s) {
        end += path.subs[s].count;
        size_t first = lines.pts.size();
        v2 p1 = path.pts[i++];
        lines.pts.push_back(p1);
        for (; i < end; i += 3) {
            v2 c1 = path.pts[i], c2 = path.pts[i + 1], p2 = path.pts[i + 2];
            bezier(p1, c1, c2, p2, angular);
            p1 = p2;
        }
        subpath e = {lines.pts.size() - first, path.subs[s].closed};
        lines.subs.push_back(e);
    }
}

// ---- dashing and stroke expansion (hpp:1858-2100) ----
void canvas_state::apply_dash() {
    if (dash.empty()) return;
    lines.pts.swap(scratch.pts);
    lines.pts.clear();
    lines.subs.swap(scratch.subs);
    lines.subs.clear();
    float total = 0.0f;
    for (size_t i = 0; i < dash.size(); ++i) total = total + dash[i];
    float offset = fmodf(dash_off, total);
    if (offset < 0.0f) offset += total;
    size_t start = 0;
    while (offset >= dash[start]) {
        offset -= dash[start];
        start = start + 1 < dash.size() ? start + 1 : 0;
    }
    size_t end = 0;
    for (size_t s = 0; s < scratch.subs.size(); ++s) {
        size_t i = end;
        end += scratch.subs[s].count;
        size_t first = lines.pts.size();
        size_t seg = start;
        bool emit = ~start & 1;
        size_t merge_pt = lines.pts.size(), merge_sub = lines.subs.size();
        bool merge_emit = emit;
        float next = dash[start] - offset;
        for (; i + 1 < end; ++i) {
            v2 from = scratch.pts[i], to = scratch.pts[i + 1];
            if (emit) lines.pts.push_back(from);
            float length = norm(sub(apply(inv, to), apply(inv, from)));
            while (next < length) {
                lines.pts.push_back(mix(from, to, next / length));
                if (emit) {
                    subpath e = {lines.pts.size() - first, false};
                    lines.subs.push_back(e);
                    first = lines.pts.size();
                }
                seg = seg + 1 < dash.size() ? seg + 1 : 0;
                emit = !emit;
                next += dash[seg];
            }
            next -= length;
        }
        if (emit) {
            lines.pts.push_back(scratch.pts[i]);
            subpath e = {lines.pts.size() - first, false};
            lines.subs.push_back(e);
            if (scratch.subs[s].closed && merge_emit) {
                if (lines.subs.size() == merge_sub + 1) {
                    lines.subs.back().closed = true;
                } else {
                    size_t count = lines.subs.back().count;
                    std::rotate(lines.pts.begin() + static_cast<ptrdiff_t>(merge_pt),
                                lines.pts.end() - static_cast<ptrdiff_t>(count), lines.pts.end());
                    lines.subs[merge_sub].count += count;
                    lines.subs.pop_back();
                }
            }
        }
    }
}

void canvas_state::half_stroke(size_t begin, size_t end, bool closed) {
    // hpp:1949-2058
    float half = lw * 0.5f;
    float ratio = miter_limit * miter_limit * half * half;
    v2 in_dir = mk(0.0f, 0.0f);
    float in_len = 0.0f;
    v2 point = apply(inv, scratch.pts[begin]);
    size_t finish = begin, i = begin;
    const float eps = 1.0e-4f;
    do {
        v2 next = apply(inv, scratch.pts[i]);
        v2 out_dir = unit(sub(next, point));
        float out_len = norm(sub(next, point));
        if (in_len != 0.0f && out_len >= eps) {
            if (closed && finish == begin) finish = i;
            v2 side_in = add(point, scl(half, perp(in_dir)));
            v2 side_out = add(point, scl(half, perp(out_dir)));
            float turn = dot(perp(in_dir), out_dir);
            if (fabsf(turn) < eps) turn = 0.0f;
            v2 off = turn == 0.0f ? mk(0.0f, 0.0f) : scl(half / turn, sub(out_dir, in_dir));
            bool tight = (dot(off, in_dir) < -in_len && dot(off, out_dir) > out_len);
            if (turn > 0.0f && tight) {
                std::swap(side_in, side_out);
                std::swap(in_dir, out_dir);
                lines.pts.push_back(apply(fwd, side_out));
                lines.pts.push_back(apply(fwd, point));
                lines.pts.push_back(apply(fwd, side_in));
            }
            if ((turn > 0.0f && !tight) || (turn != 0.0f && join == canvas_ity::miter && dot(off, off) <= ratio)) {
                lines.pts.push_back(apply(fwd, add(point, off)));
            } else if (join == canvas_ity::rounded) {
                float cosine = dot(in_dir, out_dir);
                float angle = acosf(lo(hi(cosine, -1.0f), 1.0f));
                float alpha_k = 4.0f / 3.0f * tanf(0.25f * angle);
                lines.pts.push_back(apply(fwd, side_in));
                bezier(apply(fwd, side_in), apply(fwd, add(side_in, scl(alpha_k * half, in_dir))),
                       apply(fwd, sub(side_out, scl(alpha_k * half, out_dir))), apply(fwd, side_out), -1.0f);
            } else {
                lines.pts.push_back(apply(fwd, side_in));
                lines.pts.push_back(apply(fwd, side_out));
            }
            if (turn > 0.0f && tight) {
                lines.pts.push_back(apply(fwd, side_out));
                lines.pts.push_back(apply(fwd, point));
                lines.pts.push_back(apply(fwd, side_in));
                std::swap(in_dir, out_dir);
            }
        }
        if (out_len >= eps) {
            in_dir = out_dir;
            in_len = out_len;
            point = next;
        }
        i = (i == end ? begin : end > begin ? i + 1 : i - 1);
    } while (i != finish);
    if (closed || in_len == 0.0f) return;
    v2 ahead = scl(half, in_dir);
    v2 side = perp(ahead);
    if (cap == butt) {
        lines.pts.push_back(apply(fwd, add(point, side)));
        lines.pts.push_back(apply(fwd, sub(point, side)));
    } else if (cap == square) {
        lines.pts.push_back(apply(fwd, add(add(point, ahead), side)));
        lines.pts.push_back(apply(fwd, sub(add(point, ahead), side)));
    } else if (cap == circle) {
        const float k = 0.55228475f;  // 4/3 tan(pi/8)
        lines.pts.push_back(apply(fwd, add(point, side)));
        bezier(apply(fwd, add(point, side)), apply(fwd, add(add(point, side), scl(k, ahead))),
               apply(fwd, add(add(point, ahead), scl(k, side))), apply(fwd, add(point, ahead)), -1.0f);
        bezier(apply(fwd, add(point, ahead)), apply(fwd, sub(add(point, ahead), scl(k, side))),
               apply(fwd, add(sub(point, side), scl(k, ahead))), apply(fwd, sub(point, side)), -1.0f);
    }
}

void canvas_state::stroke_outline() {
    // hpp:2070-2100
    if (singular()) return;
    apply_dash();
    lines.pts.swap(scratch.pts);
    lines.pts.clear();
    lines.subs.swap(scratch.subs);
    lines.subs.clear();
    size_t end = 0;
    for (size_t s = 0; s < scratch.subs.size(); ++s) {
        size_t begin = end;
        end += scratch.subs[s].count;
        if (end - begin < 2) continue;
        size_t first = lines.pts.size();
        half_stroke(begin, end - 1, scratch.subs[s].closed);
        if (scratch.subs[s].closed) {
            subpath e = {lines.pts.size() - first, true};
            lines.subs.push_back(e);
            first = lines.pts.size();
        }
        half_stroke(end - 1, begin, scratch.subs[s].closed);
        subpath e = {lines.pts.size() - first, true};
        lines.subs.push_back(e);
    }
}

// ---- TrueType text on the host (hpp:1299-1314, 1533-1846, 3205-3311) ----
typedef std::vector<unsigned char> bytes;
static int u8at(const bytes &d, int i) { return d[static_cast<size_t>(i)]; }
static int s8at(const bytes &d, int i) { return static_cast<signed char>(d[static_cast<size_t>(i)]); }
static int u16at(const bytes &d, int i) {
    size_t p = static_cast<size_t>(i);
    return d[p] << 8 | d[p + 1];
}
static int s16at(const bytes &d, int i) {
    size_t p = static_cast<size_t>(i);
    return static_cast<short>(d[p] << 8 | d[p + 1]);
}
static int s32at(const bytes &d, int i) {
    size_t p = static_cast<size_t>(i);
    return (d[p] << 24 | d[p + 1] << 16 | d[p + 2] << 8 | d[p + 3]);
}

// ---- glyph outlines (add_glyph, hpp:1533-1846) ----
// A glyph's TrueType record decoded once per font and glyph, for every
// canvas and request of the process: a composite glyph's components with
// their transforms, or a simple glyph's points in font units with their
// on-curve flags and contour ends.  Keyed by a hash of the font's loaded
// tables and the glyph index, and checked against the table bytes' size.
struct glyph_rec {
    bool empty = false;
    bool composite = false;
    struct component {
        int glyph;
        bool xy_args, more;
        float a, b, c, d, e, f;
    };
    std::vector<component> parts;
    std::vector<int> ends;              // last point index of each contour
    std::vector<float> x, y;            // font units
    std::vector<unsigned char> on;
};

static std::mutex g_glyph_lock;
static std::unordered_map<uint64_t, std::shared_ptr<const glyph_rec>> g_glyphs;
static size_t g_glyph_points = 0;       // points held (the cache stops growing at 64 M)

static std::shared_ptr<const glyph_rec> decode_glyph(const font_face &face, int glyph) {
    const bytes &d = face.data;
    auto rec = std::make_shared<glyph_rec>();
    int loc_format = u16at(d, face.head + 50);
    int offset = face.glyf + (loc_format ? s32at(d, face.loca + glyph * 4) : u16at(d, face.loca + glyph * 2) * 2);
    int next = face.glyf + (loc_format ? s32at(d, face.loca + glyph * 4 + 4) : u16at(d, face.loca + glyph * 2 + 2) * 2);
    if (offset == next) {
        rec->empty = true;
        return rec;
    }
    int contours = s16at(d, offset);
    if (contours < 0) {
        // composite glyph: each component under its own transform
        rec->composite = true;
        offset += 10;
        for (;;) {
            int flags = u16at(d, offset);
            glyph_rec::component cp;
            cp.glyph = u16at(d, offset + 2);
            cp.xy_args = (flags & 2) != 0;
            cp.more = (flags & 32) != 0;
            cp.a = cp.b = cp.c = cp.d = cp.e = cp.f = 0.0f;
            if (!cp.xy_args) {
                rec->parts.push_back(cp);
                break;
            }
            cp.e = static_cast<float>(flags & 1 ? s16at(d, offset + 4) : s8at(d, offset + 4));
            cp.f = static_cast<float>(flags & 1 ? s16at(d, offset + 6) : s8at(d, offset + 5));
            offset += flags & 1 ? 8 : 6;
            cp.a = flags & 200 ? static_cast<float>(s16at(d, offset)) / 16384.0f : 1.0f;
            cp.b = flags & 128 ? static_cast<float>(s16at(d, offset + 2)) / 16384.0f : 0.0f;
            cp.c = flags & 128 ? static_cast<float>(s16at(d, offset + 4)) / 16384.0f : 0.0f;
            cp.d = flags & 8 ? cp.a
                 : flags & 64 ? static_cast<float>(s16at(d, offset + 2)) / 16384.0f
                 : flags & 128 ? static_cast<float>(s16at(d, offset + 6)) / 16384.0f
                 : 1.0f;
            offset += flags & 8 ? 2 : flags & 64 ? 4 : flags & 128 ? 8 : 0;
            rec->parts.push_back(cp);
            if (!cp.more) break;
        }
        return rec;
    }
    int hmetrics = u16at(d, face.hhea + 34);
    int lsb = glyph < hmetrics ? s16at(d, face.hmtx + glyph * 4 + 2)
                               : s16at(d, face.hmtx + hmetrics * 2 + glyph * 2);
    int x_min = s16at(d, offset + 2);
    int points = u16at(d, offset + 8 + contours * 2) + 1;
    int instructions = u16at(d, offset + 10 + contours * 2);
    int flags_at = offset + 12 + contours * 2 + instructions;
    int flags_size = 0, x_size = 0;
    for (int i = 0; i < points;) {
        int fl = u8at(d, flags_at + flags_size++);
        int rep = fl & 8 ? u8at(d, flags_at + flags_size++) + 1 : 1;
        x_size += rep * (fl & 2 ? 1 : fl & 16 ? 0 : 2);
        i += rep;
    }
    int xs = flags_at + flags_size, ys = xs + x_size;
    int x = lsb - x_min, y = 0, fl = 0, rep = 0, idx = 0;
    for (int ct = 0; ct < contours; ++ct) {
        int end = u16at(d, offset + 10 + ct * 2);
        for (; idx <= end; ++idx) {
            if (rep) --rep;
            else {
                fl = u8at(d, flags_at++);
                if (fl & 8) rep = u8at(d, flags_at++);
            }
            if (fl & 2) x += (u8at(d, xs) * (fl & 16 ? 1 : -1));
            else if (!(fl & 16)) x += s16at(d, xs);
            if (fl & 4) y += (u8at(d, ys) * (fl & 32 ? 1 : -1));
            else if (!(fl & 32)) y += s16at(d, ys);
            xs += fl & 2 ? 1 : fl & 16 ? 0 : 2;
            ys += fl & 4 ? 1 : fl & 32 ? 0 : 2;
            rec->x.push_back(static_cast<float>(x));
            rec->y.push_back(static_cast<float>(y));
            rec->on.push_back(static_cast<unsigned char>(fl & 1));
        }
        rec->ends.push_back(end);
    }
    return rec;
}

static std::shared_ptr<const glyph_rec> cached_glyph(const font_face &face, int glyph) {
    const uint64_t key = (face.hash ^ (static_cast<uint64_t>(glyph) * 0x9e3779b97f4a7c15ull)) ^ face.data.size();
    {
        std::lock_guard<std::mutex> hold(g_glyph_lock);
        auto it = g_glyphs.find(key);
        if (it != g_glyphs.end()) return it->second;
    }
    std::shared_ptr<const glyph_rec> rec = decode_glyph(face, glyph);
    std::lock_guard<std::mutex> hold(g_glyph_lock);
    if (g_glyph_points + rec->x.size() <= (size_t(64) << 20)) {
        g_glyph_points += rec->x.size();
        g_glyphs.emplace(key, rec);
    }
    return rec;
}

void canvas_state::glyph_outline(int glyph, float angular) {
    std::shared_ptr<const glyph_rec> rec = cached_glyph(face, glyph);
    if (rec->empty) return;
    if (rec->composite) {
        for (const glyph_rec::component &cp : rec->parts) {
            if (!cp.xy_args) return;
            affine sf = fwd, si = inv;
            transform(cp.a, cp.b, cp.c, cp.d, cp.e, cp.f);
            glyph_outline(cp.glyph, angular);
            fwd = sf;
            inv = si;
            if (!cp.more) return;
        }
        return;
    }
    int idx = 0;
    for (size_t ct = 0; ct < rec->ends.size(); ++ct) {
        int begin = idx;
        int end = rec->ends[ct];
        v2 bp = mk(0, 0), ep = mk(0, 0);
        bool bon = false, eon = false;
        // Each contour is emitted as points and cubics: flattened into
        // `lines` (add_glyph, hpp:1533-1846), or kept as cubic control points
        // in `path` (outline_cubics), where the device flattens them alike.
        polyline &out = outline_cubics ? path : lines;
        size_t first = out.pts.size();
        auto put_point = [&](v2 p) {
            if (!outline_cubics) {
                lines.pts.push_back(p);
            } else if (out.pts.size() == first) {
                path.pts.push_back(p);
            } else {
                v2 p1 = path.pts.back();
                path.pts.push_back(p1);
                path.pts.push_back(p);
                path.pts.push_back(p);
            }
        };
        auto put_curve = [&](v2 p1, v2 c1, v2 c2, v2 p2) {
            if (!outline_cubics) {
                bezier(p1, c1, c2, p2, angular);
            } else {
                path.pts.push_back(c1);
                path.pts.push_back(c2);
                path.pts.push_back(p2);
            }
        };
        for (; idx <= end; ++idx) {
            v2 pt = apply(fwd, mk(rec->x[static_cast<size_t>(idx)], rec->y[static_cast<size_t>(idx)]));
            int on = rec->on[static_cast<size_t>(idx)];
            if (idx == begin) {
                bp = pt;
                bon = on;
                if (on) put_point(pt);
            } else {
                v2 p2 = on ? pt : mix(ep, pt, 0.5f);
                if (out.pts.size() == first || (eon && on)) {
                    put_point(p2);
                } else if (!eon || on) {
                    v2 p1 = out.pts.back();
                    put_curve(p1, mix(p1, ep, 2.0f / 3.0f), mix(p2, ep, 2.0f / 3.0f), p2);
                }
            }
            ep = pt;
            eon = on;
        }
        // a contour of one off-curve point has nothing to close (the host
        // walk below follows the reference even there)
        if (outline_cubics && out.pts.size() == first) continue;
        if (bon ^ eon) {
            v2 p1 = out.pts.back(), p2 = out.pts[first];
            v2 ctl = eon ? bp : ep;
            put_curve(p1, mix(p1, ctl, 2.0f / 3.0f), mix(p2, ctl, 2.0f / 3.0f), p2);
        } else if (!bon && !eon) {
            v2 p1 = out.pts.back();
            v2 split = mix(bp, ep, 0.5f);
            v2 p2 = out.pts[first];
            put_curve(p1, mix(p1, ep, 2.0f / 3.0f), mix(split, ep, 2.0f / 3.0f), split);
            put_curve(split, mix(split, bp, 2.0f / 3.0f), mix(p2, bp, 2.0f / 3.0f), p2);
        }
        put_point(out.pts[first]);
        subpath e = {out.pts.size() - first, true};
        out.subs.push_back(e);
    }
}

int canvas_state::glyph_of(const char *text, int &index) {
    // hpp:1749-1820: UTF-8 decode, then cmap format 12, 4 or 0 lookup
    const bytes &d = face.data;
    int nb = ((text[index] & 0x80) == 0x00 ? 1 : (text[index] & 0xe0) == 0xc0 ? 2
              : (text[index] & 0xf0) == 0xe0 ? 3 : (text[index] & 0xf8) == 0xf0 ? 4 : 0);
    const int masks[] = {0x0, 0x7f, 0x1f, 0x0f, 0x07};
    int cp = nb ? text[index] & masks[nb] : 0xfffd;
    ++index;
    while (--nb > 0) {
        if ((text[index] & 0xc0) == 0x80) cp = cp << 6 | (text[index++] & 0x3f);
        else { cp = 0xfffd; break; }
    }
    if (cp == '\t' || cp == '\v' || cp == '\f' || cp == '\r' || cp == '\n') cp = ' ';
    int tables = u16at(d, face.cmap + 2);
    int f12 = 0, f4 = 0, f0 = 0;
    for (int t = 0; t < tables; ++t) {
        int platform = u16at(d, face.cmap + t * 8 + 4);
        int encoding = u16at(d, face.cmap + t * 8 + 6);
        int off = s32at(d, face.cmap + t * 8 + 8);
        int format = u16at(d, face.cmap + off);
        if (platform == 3 && encoding == 10 && format == 12) f12 = face.cmap + off;
        else if (platform == 3 && encoding == 1 && format == 4) f4 = face.cmap + off;
        else if (format == 0) f0 = face.cmap + off;
    }
    if (f12) {
        int groups = s32at(d, f12 + 12);
        for (int g = 0; g < groups; ++g) {
            int s = s32at(d, f12 + 16 + g * 12), e = s32at(d, f12 + 20 + g * 12), gl = s32at(d, f12 + 24 + g * 12);
            if (s <= cp && cp <= e) return cp - s + gl;
        }
    } else if (f4) {
        int segs = u16at(d, f4 + 6);
        int ends = f4 + 14, starts = ends + 2 + segs, deltas = starts + segs, ranges = deltas + segs;
        for (int s = 0; s < segs; s += 2) {
            int st = u16at(d, starts + s), en = u16at(d, ends + s), de = s16at(d, deltas + s), ra = u16at(d, ranges + s);
            if (st <= cp && cp <= en) return ra ? u16at(d, ranges + s + (cp - st) * 2 + ra) : (cp + de) & 0xffff;
        }
    } else if (f0 && 0 <= cp && cp < 256) {
        return u8at(d, f0 + 6 + cp);
    }
    return 0;
}

float canvas_state::measure(const char *text) {
    // hpp:3296-3311
    if (face.data.empty() || !text) return 0.0f;
    int hmetrics = u16at(face.data, face.hhea + 34);
    int width = 0;
    for (int i = 0; text[i];) {
        int g = glyph_of(text, i);
        int entry = g < hmetrics - 1 ? g : hmetrics - 1;
        width += u16at(face.data, face.hmtx + entry * 4);
    }
    return static_cast<float>(width) * face.scale;
}

void canvas_state::text_outline(const char *text, v2 at, float maxw, bool stroking) {
    // hpp:1830-1846 (text_to_lines)
    const float tol = 0.125f;
    float ratio = tol / hi(0.5f * lw, tol);
    float angular = stroking ? (ratio - 2.0f) * ratio * 2.0f + 1.0f : -1.0f;
    lines.pts.clear();
    lines.subs.clear();
    if (face.data.empty() || !text || maxw <= 0.0f) return;
    const bytes &d = face.data;
    float width = maxw == 1.0e30f && align == leftward ? 0.0f : measure(text);
    float reduction = maxw / hi(maxw, width);
    if (align == rightward) at.x -= width * reduction;
    else if (align == center) at.x -= 0.5f * width * reduction;
    v2 scaling = scl(face.scale, mk(reduction, 1.0f));
    float upem = static_cast<float>(u16at(d, face.head + 18));
    float ascender = static_cast<float>(s16at(d, face.os_2 + 68));
    float descender = static_cast<float>(s16at(d, face.os_2 + 70));
    float normalize = face.scale * upem / (ascender - descender);
    if (baseline == top) at.y += ascender * normalize;
    else if (baseline == middle) at.y += (ascender + descender) * 0.5f * normalize;
    else if (baseline == bottom) at.y += descender * normalize;
    else if (baseline == hanging) at.y += 0.6f * face.scale * upem;
    affine sf = fwd, si = inv;
    int hmetrics = u16at(d, face.hhea + 34);
    int place = 0;
    for (int i = 0; text[i];) {
        int g = glyph_of(text, i);
        fwd = sf;
        transform(scaling.x, 0.0f, 0.0f, -scaling.y, at.x + static_cast<float>(place) * scaling.x, at.y);
        glyph_outline(g, angular);
        int entry = g < hmetrics - 1 ? g : hmetrics - 1;
        place += u16at(d, face.hmtx + entry * 4);
    }
    fwd = sf;
    inv = si;
}

// ---- handing draws to the GPU engine ----
void canvas_state::make_paint(const brush &br, bool clamp_edges, bool force_solid, cy_paint &p) {
    std::memset(&p, 0, sizeof(p));
    p.clamp_edges = clamp_edges ? 1 : 0;
    p.inverse[0] = inv.a; p.inverse[1] = inv.b; p.inverse[2] = inv.c;
    p.inverse[3] = inv.d; p.inverse[4] = inv.e; p.inverse[5] = inv.f;
    int kind = force_solid ? CY_PAINT_SOLID : br.kind;
    bool empty = kind == CY_PAINT_PATTERN ? br.pixels.empty() : br.colors.empty();
    if (kind == CY_PAINT_SOLID && force_solid && br.kind == CY_PAINT_PATTERN) {
        // clear_rectangle forces the fill brush to a solid colour and paints
        // its first stored colour (hpp:3134-3153, 2271-2272); for a pattern
        // that is the first texel, linearised and premultiplied.
        empty = br.pixels.empty();
        if (!empty) {
            rgba4 c = {linearized(br.pixels[0] / 255.0f), linearized(br.pixels[1] / 255.0f),
                       linearized(br.pixels[2] / 255.0f), br.pixels[3] / 255.0f};
            c = premultiplied(c);
            p.kind = CY_PAINT_SOLID;
            p.color[0] = c.r; p.color[1] = c.g; p.color[2] = c.b; p.color[3] = c.a;
        }
        if (empty) p.kind = CY_PAINT_NONE;
        return;
    }
    if (empty) { p.kind = CY_PAINT_NONE; return; }
    p.kind = kind;
    if (kind == CY_PAINT_SOLID) {
        const rgba4 &c = br.colors.front();
        p.color[0] = c.r; p.color[1] = c.g; p.color[2] = c.b; p.color[3] = c.a;
    } else if (kind == CY_PAINT_LINEAR || kind == CY_PAINT_RADIAL) {
        p.start[0] = br.p0.x; p.start[1] = br.p0.y; p.end[0] = br.p1.x; p.end[1] = br.p1.y;
        p.start_radius = br.r0;
        p.end_radius = br.r1;
        stop_colors.resize(br.colors.size() * 4);
        for (size_t i = 0; i < br.colors.size(); ++i) {
            stop_colors[i * 4 + 0] = br.colors[i].r;
            stop_colors[i * 4 + 1] = br.colors[i].g;
            stop_colors[i * 4 + 2] = br.colors[i].b;
            stop_colors[i * 4 + 3] = br.colors[i].a;
        }
        p.stop_offsets = br.stops.data();
        p.stop_colors = stop_colors.data();
        p.n_stops = static_cast<int>(br.stops.size());
    } else {
        p.pattern = br.pixels.data();
        p.pattern_width = br.w;
        p.pattern_height = br.h;
        p.repetition = br.rep;
    }
}

void canvas_state::make_state(cy_draw_state &s, bool with_shadow) {
    s.operation = op;
    s.global_alpha = alpha;
    s.mask = mask;
    s.shadow_color[0] = shadow_color.r;
    s.shadow_color[1] = shadow_color.g;
    s.shadow_color[2] = shadow_color.b;
    s.shadow_color[3] = with_shadow ? shadow_color.a : 0.0f;
    s.shadow_blur = shadow_blur;
    s.shadow_offset_x = sox;
    s.shadow_offset_y = soy;
    s.fill_rule = 0;
}

void canvas_state::draw_lines(const brush &br, bool clamp_edges, bool force_solid, bool with_shadow) {
    // render_main (hpp:2551-2605): nothing is drawn under a singular transform
    if (singular()) return;
    cy_paint p;
    cy_draw_state s;
    make_paint(br, clamp_edges, force_solid, p);
    make_state(s, with_shadow);
    counts.resize(lines.subs.size());
    for (size_t i = 0; i < lines.subs.size(); ++i) counts[i] = static_cast<int>(lines.subs[i].count);
    note(cy_fill_lines(ctx, reinterpret_cast<const float *>(lines.pts.data()), counts.data(),
                       static_cast<int>(counts.size()), &p, &s));
}

// A filled path flattened on the device; with_rule false fills nonzero
// whatever the fill rule (text, as with strokes and rectangles).
void canvas_state::draw_path(const brush &br, bool with_rule) {
    if (singular()) return;
    cy_paint p;
    cy_draw_state s;
    make_paint(br, false, false, p);
    make_state(s, true);
    s.fill_rule = with_rule && even_odd ? 1 : 0;
    counts.resize(path.subs.size());
    for (size_t i = 0; i < path.subs.size(); ++i) counts[i] = static_cast<int>(path.subs[i].count);
    note(cy_fill_path(ctx, reinterpret_cast<const float *>(path.pts.data()), counts.data(),
                      static_cast<int>(counts.size()), &p, &s));
}

// stroke() with the expansion on the device: the path's cubics and the
// line style go to cy_stroke_path, which flattens, dashes and expands them
// as path_to_lines(true), dash_lines and stroke_lines do (hpp:1495-1524,
// 1858-2100) before render_main.
void canvas_state::stroke_path(const brush &br) {
    if (singular()) return;
    cy_paint p;
    cy_draw_state s;
    make_paint(br, false, false, p);
    make_state(s, true);
    counts.resize(path.subs.size());
    closed_flags.resize(path.subs.size());
    for (size_t i = 0; i < path.subs.size(); ++i) {
        counts[i] = static_cast<int>(path.subs[i].count);
        closed_flags[i] = path.subs[i].closed ? 1 : 0;
    }
    cy_stroke_style st;
    st.line_width = lw;
    st.miter_limit = miter_limit;
    st.line_join = static_cast<int>(join);
    st.line_cap = static_cast<int>(cap);
    st.dash = dash.empty() ? nullptr : dash.data();
    st.n_dash = static_cast<int>(dash.size());
    st.dash_offset = dash_off;
    const float f[6] = {fwd.a, fwd.b, fwd.c, fwd.d, fwd.e, fwd.f};
    const float v[6] = {inv.a, inv.b, inv.c, inv.d, inv.e, inv.f};
    for (int i = 0; i < 6; ++i) {
        st.forward[i] = f[i];
        st.inverse[i] = v[i];
    }
    note(cy_stroke_path(ctx, reinterpret_cast<const float *>(path.pts.data()), counts.data(), closed_flags.data(),
                        static_cast<int>(counts.size()), &st, &p, &s));
}

}  // namespace detail

using detail::mk;
using detail::v2;
using detail::apply;

canvas::canvas(int width, int height)
    : global_composite_operation(source_over), shadow_offset_x(0.0f), shadow_offset_y(0.0f),
      line_cap(butt), line_join(miter), line_dash_offset(0.0f), text_align(start),
      text_baseline(alphabetic), self(new detail::canvas_state()) {
    detail::canvas_state &s = *self;
    s.W = width;
    s.H = height;
    s.ctx = nullptr;
    s.status = cy_ctx_create(width, height, &s.ctx);
    detail::affine identity = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f};
    s.fwd = identity;
    s.inv = identity;
    s.alpha = 1.0f;
    s.shadow_color.r = s.shadow_color.g = s.shadow_color.b = s.shadow_color.a = 0.0f;
    s.shadow_blur = 0.0f;
    s.lw = 1.0f;
    s.miter_limit = 10.0f;
    s.mask = 0;
    set_color(fill_style, 0.0f, 0.0f, 0.0f, 1.0f);
    set_color(stroke_style, 0.0f, 0.0f, 0.0f, 1.0f);
    sync_public_state();
}

canvas::~canvas() {
    if (self->ctx) cy_ctx_destroy(self->ctx);
    delete self;
}

int canvas::gpu_status() const {
    if (self->status) return self->status;
    return self->ctx ? cy_ctx_status(self->ctx) : CY_ENODEV;
}

void *canvas::gpu_context() const { return self->ctx; }

int canvas::read_linear(float *rgba) {
    if (!self->ctx) return CY_ENODEV;
    return cy_read_linear(self->ctx, rgba);
}

void canvas::sync_public_state() {
    self->op = global_composite_operation;
    self->sox = shadow_offset_x;
    self->soy = shadow_offset_y;
    self->cap = line_cap;
    self->join = line_join;
    self->dash_off = line_dash_offset;
    self->align = text_align;
    self->baseline = text_baseline;
}

void canvas::scale(float x, float y) { self->transform(x, 0.0f, 0.0f, y, 0.0f, 0.0f); }
void canvas::rotate(float angle) {
    float c = cosf(angle), s = sinf(angle);
    self->transform(c, s, -s, c, 0.0f, 0.0f);
}
void canvas::translate(float x, float y) { self->transform(1.0f, 0.0f, 0.0f, 1.0f, x, y); }
void canvas::transform(float a, float b, float c, float d, float e, float f) { self->transform(a, b, c, d, e, f); }
void canvas::set_transform(float a, float b, float c, float d, float e, float f) {
    self->set_transform(a, b, c, d, e, f);
}
void canvas::set_global_alpha(float a) { if (0.0f <= a && a <= 1.0f) self->alpha = a; }
void canvas::set_shadow_color(float r, float g, float b, float a) {
    self->shadow_color = detail::premultiplied(detail::clamped_linear(r, g, b, a));
}
void canvas::set_shadow_blur(float level) { if (0.0f <= level) self->shadow_blur = level; }
void canvas::set_line_width(float w) { if (0.0f < w) self->lw = w; }
void canvas::set_miter_limit(float m) { if (0.0f < m) self->miter_limit = m; }
void canvas::set_line_dash(float const *segments, int count) {
    // hpp:2748-2763
    for (int i = 0; i < count; ++i)
        if (segments && segments[i] < 0.0f) return;
    self->dash.clear();
    if (!segments) return;
    for (int i = 0; i < count; ++i) self->dash.push_back(segments[i]);
    if (count & 1)
        for (int i = 0; i < count; ++i) self->dash.push_back(segments[i]);
}

void canvas::set_color(brush_type type, float r, float g, float b, float a) {
    detail::brush &br = type == fill_style ? self->fill : self->stroke;
    br.kind = CY_PAINT_SOLID;
    br.colors.clear();
    br.colors.push_back(detail::premultiplied(detail::clamped_linear(r, g, b, a)));
    br.pixels.clear();
}
void canvas::set_linear_gradient(brush_type type, float x0, float y0, float x1, float y1) {
    detail::brush &br = type == fill_style ? self->fill : self->stroke;
    br.kind = CY_PAINT_LINEAR;
    br.colors.clear();
    br.stops.clear();
    br.pixels.clear();
    br.p0 = mk(x0, y0);
    br.p1 = mk(x1, y1);
}
void canvas::set_radial_gradient(brush_type type, float x0, float y0, float r0, float x1, float y1, float r1) {
    if (r0 < 0.0f || r1 < 0.0f) return;
    detail::brush &br = type == fill_style ? self->fill : self->stroke;
    br.kind = CY_PAINT_RADIAL;
    br.colors.clear();
    br.stops.clear();
    br.pixels.clear();
    br.p0 = mk(x0, y0);
    br.p1 = mk(x1, y1);
    br.r0 = r0;
    br.r1 = r1;
}
void canvas::add_color_stop(brush_type type, float offset, float r, float g, float b, float a) {
    // hpp:2822-2839: sorted insert (after equal offsets), straight alpha
    detail::brush &br = type == fill_style ? self->fill : self->stroke;
    if ((br.kind != CY_PAINT_LINEAR && br.kind != CY_PAINT_RADIAL) || offset < 0.0f || 1.0f < offset) return;
    size_t at = 0;
    while (at < br.stops.size() && !(offset < br.stops[at])) ++at;
    br.colors.insert(br.colors.begin() + static_cast<ptrdiff_t>(at), detail::clamped_linear(r, g, b, a));
    br.stops.insert(br.stops.begin() + static_cast<ptrdiff_t>(at), offset);
}
void canvas::set_pattern(brush_type type, unsigned char const *image, int width, int height, int stride,
                         repetition_style repetition) {
    if (!image || width <= 0 || height <= 0) return;
    detail::brush &br = type == fill_style ? self->fill : self->stroke;
    br.kind = CY_PAINT_PATTERN;
    br.colors.clear();
    br.stops.clear();
    br.pixels.resize(static_cast<size_t>(width) * static_cast<size_t>(height) * 4u);
    for (int y = 0; y < height; ++y)
        std::memcpy(&br.pixels[static_cast<size_t>(y) * static_cast<size_t>(width) * 4u],
                    image + static_cast<ptrdiff_t>(y) * stride, static_cast<size_t>(width) * 4u);
    br.w = width;
    br.h = height;
    br.rep = repetition;
}

void canvas::begin_path() {
    self->path.pts.clear();
    self->path.subs.clear();
}
void canvas::move_to(float x, float y) { self->move_to(x, y); }
void canvas::close_path() {
    // hpp:2884-2896
    detail::canvas_state &s = *self;
    if (s.path.subs.empty()) return;
    v2 first = s.path.pts[s.path.pts.size() - s.path.subs.back().count];
    detail::affine saved = s.fwd;
    detail::affine identity = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f};
    s.fwd = identity;
    s.line_to(first.x, first.y);
    s.path.subs.back().closed = true;
    s.move_to(first.x, first.y);
    s.fwd = saved;
}
void canvas::line_to(float x, float y) { self->line_to(x, y); }
void canvas::quadratic_curve_to(float cx, float cy, float x, float y) {
    // hpp:2918-2934: raised to a cubic
    detail::canvas_state &s = *self;
    if (s.path.subs.empty()) s.move_to(cx, cy);
    v2 p1 = s.path.pts.back();
    v2 c = apply(s.fwd, mk(cx, cy));
    v2 p2 = apply(s.fwd, mk(x, y));
    s.path.pts.push_back(detail::mix(p1, c, 2.0f / 3.0f));
    s.path.pts.push_back(detail::mix(p2, c, 2.0f / 3.0f));
    s.path.pts.push_back(p2);
    s.path.subs.back().count += 3;
}
void canvas::bezier_curve_to(float c1x, float c1y, float c2x, float c2y, float x, float y) {
    detail::canvas_state &s = *self;
    if (s.path.subs.empty()) s.move_to(c1x, c1y);
    v2 c1 = apply(s.fwd, mk(c1x, c1y));
    v2 c2 = apply(s.fwd, mk(c2x, c2y));
    v2 p2 = apply(s.fwd, mk(x, y));
    s.path.pts.push_back(c1);
    s.path.pts.push_back(c2);
    s.path.pts.push_back(p2);
    s.path.subs.back().count += 3;
}
void canvas::arc_to(float vx, float vy, float x, float y, float radius) {
    // hpp:2955-2988
    detail::canvas_state &s = *self;
    if (radius < 0.0f || s.singular()) return;
    if (s.path.subs.empty()) s.move_to(vx, vy);
    v2 p1 = apply(s.inv, s.path.pts.back());
    v2 v = mk(vx, vy), p2 = mk(x, y);
    v2 e1 = detail::unit(detail::sub(p1, v));
    v2 e2 = detail::unit(detail::sub(p2, v));
    float sine = fabsf(detail::dot(detail::perp(e1), e2));
    if (sine < 1.0e-4f) { s.line_to(vx, vy); return; }
    v2 off = detail::scl(radius / sine, detail::add(e1, e2));
    v2 center = detail::add(v, off);
    v2 t1 = detail::sub(detail::scl(detail::dot(off, e1), e1), off);
    v2 t2 = detail::sub(detail::scl(detail::dot(off, e2), e2), off);
    float a1 = atan2f(t1.y, t1.x);
    float a2 = atan2f(t2.y, t2.x);
    bool reverse = static_cast<int>(floorf((a2 - a1) / 3.14159265f)) & 1;
    arc(center.x, center.y, radius, a1, a2, reverse);
}
void canvas::arc(float x, float y, float radius, float a0, float a1, bool ccw) {
    // hpp:2990-3028: at most 16 cubic segments per full turn
    if (radius < 0.0f) return;
    const float tau = 6.28318531f;
    float winding = ccw ? -1.0f : 1.0f;
    float from = fmodf(a0, tau);
    float span = fmodf(a1, tau) - from;
    if ((a1 - a0) * winding >= tau) span = tau * winding;
    else if (span * winding < 0.0f) span += tau * winding;
    v2 c1 = detail::scl(radius, mk(cosf(from), sinf(from)));
    line_to(x + c1.x, y + c1.y);
    if (span == 0.0f) return;
    int steps = static_cast<int>(detail::hi(1.0f, roundf(16.0f / tau * span * winding)));
    float segment = span / static_cast<float>(steps);
    float k = 4.0f / 3.0f * tanf(0.25f * segment);
    for (int st = 0; st < steps; ++st) {
        float angle = from + static_cast<float>(st + 1) * segment;
        v2 c2 = detail::scl(radius, mk(cosf(angle), sinf(angle)));
        v2 q1 = detail::add(mk(x, y), c1), q2 = detail::add(mk(x, y), c2);
        v2 k1 = detail::add(q1, detail::scl(k, detail::perp(c1)));
        v2 k2 = detail::sub(q2, detail::scl(k, detail::perp(c2)));
        bezier_curve_to(k1.x, k1.y, k2.x, k2.y, q2.x, q2.y);
        c1 = c2;
    }
}
void canvas::rectangle(float x, float y, float w, float h) {
    move_to(x, y);
    line_to(x + w, y);
    line_to(x + w, y + h);
    line_to(x, y + h);
    close_path();
}

void canvas::fill() {
    sync_public_state();
    self->draw_path(self->fill);
}
void canvas::stroke() {
    // hpp:3050-3055
    sync_public_state();
    if (cy_device_stroke()) {
        self->stroke_path(self->stroke);
        return;
    }
    self->flatten(true);
    self->stroke_outline();
    self->draw_lines(self->stroke, false, false, true);
}
void canvas::clip() {
    // hpp:3057-3099: the new mask is the old one times the path coverage
    detail::canvas_state &s = *self;
    s.counts.resize(s.path.subs.size());
    for (size_t i = 0; i < s.path.subs.size(); ++i) s.counts[i] = static_cast<int>(s.path.subs[i].count);
    int out = s.mask;
    int rc = cy_clip_path(s.ctx, reinterpret_cast<const float *>(s.path.pts.data()), s.counts.data(),
                          static_cast<int>(s.counts.size()), s.mask, s.even_odd ? 1 : 0, &out);
    s.note(rc);
    if (rc == 0) {
        if (s.mask) s.note(cy_mask_release(s.ctx, s.mask));
        s.mask = out;
    }
}
bool canvas::is_point_in_path(float x, float y) {
    // hpp:3101-3132: nonzero winding over the fill-mode polyline
    detail::canvas_state &s = *self;
    s.flatten(false);
    int winding = 0;
    size_t sp = 0, begin = 0, end = 0;
    for (size_t i = 0; i < s.lines.pts.size(); ++i) {
        while (i >= end) {
            begin = end;
            end += s.lines.subs[sp++].count;
        }
        v2 from = s.lines.pts[i];
        v2 to = s.lines.pts[i + 1 < end ? i + 1 : begin];
        if ((from.y < y && y <= to.y) || (to.y < y && y <= from.y)) {
            float side = detail::dot(detail::perp(detail::sub(to, from)), detail::sub(mk(x, y), from));
            if (side == 0.0f) return true;
            winding += side > 0.0f ? 1 : -1;
        } else if (from.y == y && y == to.y && ((from.x <= x && x <= to.x) || (to.x <= x && x <= from.x))) {
            return true;
        }
    }
    return s.even_odd ? (winding & 2) != 0 : winding != 0;   // each crossing edge counts +-1 on each side: twice the winding number
}
void canvas::set_fill_rule(fill_rule_style rule) { self->even_odd = rule == even_odd; }
int canvas::points_in_path(float const *xy, int n, unsigned char *inside) {
    // is_point_in_path (hpp:3101-3132) for many points: the path's
    // device-space cubics go to the GPU, flattened there as for a fill
    detail::canvas_state &s = *self;
    s.counts.resize(s.path.subs.size());
    for (size_t i = 0; i < s.path.subs.size(); ++i) s.counts[i] = static_cast<int>(s.path.subs[i].count);
    return cy_points_in_path(reinterpret_cast<const float *>(s.path.pts.data()), s.counts.data(),
                             static_cast<int>(s.counts.size()), xy, n, s.even_odd ? 1 : 0, inside);
}

static void rect_lines(detail::canvas_state &s, float x, float y, float w, float h, bool closing_point) {
    s.lines.pts.clear();
    s.lines.subs.clear();
    s.lines.pts.push_back(apply(s.fwd, mk(x, y)));
    s.lines.pts.push_back(apply(s.fwd, mk(x + w, y)));
    s.lines.pts.push_back(apply(s.fwd, mk(x + w, y + h)));
    s.lines.pts.push_back(apply(s.fwd, mk(x, y + h)));
    if (closing_point) s.lines.pts.push_back(apply(s.fwd, mk(x, y)));
    detail::subpath e = {s.lines.pts.size(), true};
    s.lines.subs.push_back(e);
}

void canvas::clear_rectangle(float x, float y, float w, float h) {
    // hpp:3134-3153: destination_out at full alpha with the fill brush forced
    // to a solid colour and no shadow
    sync_public_state();
    detail::canvas_state &s = *self;
    if (w == 0.0f || h == 0.0f) return;
    rect_lines(s, x, y, w, h, false);
    composite_operation saved_op = s.op;
    float saved_alpha = s.alpha;
    s.op = destination_out;
    s.alpha = 1.0f;
    s.draw_lines(s.fill, false, true, false);
    s.op = saved_op;
    s.alpha = saved_alpha;
}
void canvas::fill_rectangle(float x, float y, float w, float h) {
    sync_public_state();
    if (w == 0.0f || h == 0.0f) return;
    rect_lines(*self, x, y, w, h, false);
    self->draw_lines(self->fill, false, false, true);
}
void canvas::stroke_rectangle(float x, float y, float w, float h) {
    // hpp:3174-3203
    sync_public_state();
    detail::canvas_state &s = *self;
    if (w == 0.0f && h == 0.0f) return;
    if (cy_device_stroke()) {
        // The rectangle's lines as a path of degenerate cubics, which the
        // device flattens to the same points, stroked on the device; the
        // current path is left as it was.
        detail::polyline saved;
        saved.pts.swap(s.path.pts);
        saved.subs.swap(s.path.subs);
        v2 a = apply(s.fwd, mk(x, y));
        s.path.pts.push_back(a);
        auto line = [&](v2 p) {
            v2 p1 = s.path.pts.back();
            s.path.pts.push_back(p1);
            s.path.pts.push_back(p);
            s.path.pts.push_back(p);
        };
        bool flat = w == 0.0f || h == 0.0f;
        if (flat) {
            line(apply(s.fwd, mk(x + w, y + h)));
        } else {
            line(apply(s.fwd, mk(x + w, y)));
            line(apply(s.fwd, mk(x + w, y + h)));
            line(apply(s.fwd, mk(x, y + h)));
            line(a);
        }
        detail::subpath e = {s.path.pts.size(), !flat};
        s.path.subs.push_back(e);
        s.stroke_path(s.stroke);
        s.path.pts.swap(saved.pts);
        s.path.subs.swap(saved.subs);
        return;
    }
    if (w == 0.0f || h == 0.0f) {
        s.lines.pts.clear();
        s.lines.subs.clear();
        s.lines.pts.push_back(apply(s.fwd, mk(x, y)));
        s.lines.pts.push_back(apply(s.fwd, mk(x + w, y + h)));
        detail::subpath e = {2, false};
        s.lines.subs.push_back(e);
    } else {
        rect_lines(s, x, y, w, h, true);
    }
    s.stroke_outline();
    s.draw_lines(s.stroke, false, false, true);
}

bool canvas::set_font(unsigned char const *font, int nbytes, float size) {
    // hpp:3205-3275
    detail::font_face &face = self->face;
    if (font && nbytes) {
        face.data.clear();
        face.cmap = face.glyf = face.head = face.hhea = face.hmtx = face.loca = face.maxp = face.os_2 = 0;
        if (nbytes < 6) return false;
        int version = (font[0] << 24 | font[1] << 16 | font[2] << 8 | font[3] << 0);
        int tables = font[4] << 8 | font[5];
        if ((version != 0x00010000 && version != 0x74727565) || nbytes < tables * 16 + 12) return false;
        face.data.insert(face.data.end(), font, font + tables * 16 + 12);
        for (int t = 0; t < tables; ++t) {
            int tag = detail::s32at(face.data, t * 16 + 12);
            int off = detail::s32at(face.data, t * 16 + 20);
            int span = detail::s32at(face.data, t * 16 + 24);
            if (nbytes < off + span) { face.data.clear(); return false; }
            int place = static_cast<int>(face.data.size());
            if (tag == 0x636d6170) face.cmap = place;
            else if (tag == 0x676c7966) face.glyf = place;
            else if (tag == 0x68656164) face.head = place;
            else if (tag == 0x68686561) face.hhea = place;
            else if (tag == 0x686d7478) face.hmtx = place;
            else if (tag == 0x6c6f6361) face.loca = place;
            else if (tag == 0x6d617870) face.maxp = place;
            else if (tag == 0x4f532f32) face.os_2 = place;
            else continue;
            face.data.insert(face.data.end(), font + off, font + off + span);
        }
        if (!face.cmap || !face.glyf || !face.head || !face.hhea || !face.hmtx || !face.loca ||
            !face.maxp || !face.os_2) {
            face.data.clear();
            return false;
        }
    }
    if (face.data.empty()) return false;
    if (font && nbytes) {
        // FNV-1a of the loaded tables: the key of their glyph outlines
        uint64_t hsh = 1469598103934665603ull;
        for (unsigned char ch : face.data) hsh = (hsh ^ ch) * 1099511628211ull;
        face.hash = hsh;
    }
    int upem = detail::u16at(face.data, face.head + 18);
    face.scale = size / static_cast<float>(upem);
    return true;
}
void canvas::fill_text(char const *text, float x, float y, float maxw) {
    // hpp:3277-3284: the glyph outlines go to the device as cubics and are
    // flattened there like any filled path; the current path is left as it was.
    sync_public_state();
    detail::canvas_state &s = *self;
    detail::polyline saved;
    saved.pts.swap(s.path.pts);
    saved.subs.swap(s.path.subs);
    s.outline_cubics = true;
    s.text_outline(text, mk(x, y), maxw, false);
    s.outline_cubics = false;
    if (!s.path.subs.empty()) s.draw_path(s.fill, false);
    s.path.pts.swap(saved.pts);
    s.path.subs.swap(saved.subs);
}
void canvas::stroke_text(char const *text, float x, float y, float maxw) {
    sync_public_state();
    detail::canvas_state &s = *self;
    if (cy_device_stroke()) {
        // The glyph outlines as cubics, flattened and stroked on the device;
        // the current path is left as it was.
        detail::polyline saved;
        saved.pts.swap(s.path.pts);
        saved.subs.swap(s.path.subs);
        s.outline_cubics = true;
        s.text_outline(text, mk(x, y), maxw, true);
        s.outline_cubics = false;
        if (!s.path.subs.empty()) s.stroke_path(s.stroke);
        s.path.pts.swap(saved.pts);
        s.path.subs.swap(saved.subs);
        return;
    }
    self->text_outline(text, mk(x, y), maxw, true);
    self->stroke_outline();
    self->draw_lines(self->stroke, false, false, true);
}
float canvas::measure_text(char const *text) { return self->measure(text); }

void canvas::draw_image(unsigned char const *image, int width, int height, int stride, float x, float y,
                        float to_width, float to_height) {
    // hpp:3313-3346: clamp-edged bicubic image brush under a temporary transform
    sync_public_state();
    detail::canvas_state &s = *self;
    if (!image || width <= 0 || height <= 0 || to_width == 0.0f || to_height == 0.0f) return;
    detail::brush &br = s.image;
    br.kind = CY_PAINT_PATTERN;
    br.colors.clear();
    br.pixels.resize(static_cast<size_t>(width) * static_cast<size_t>(height) * 4u);
    for (int row = 0; row < height; ++row)
        std::memcpy(&br.pixels[static_cast<size_t>(row) * static_cast<size_t>(width) * 4u],
                    image + static_cast<ptrdiff_t>(row) * stride, static_cast<size_t>(width) * 4u);
    br.w = width;
    br.h = height;
    br.rep = repeat;
    rect_lines(s, x, y, to_width, to_height, false);
    detail::affine sf = s.fwd, si = s.inv;
    s.transform(1.0f, 0.0f, 0.0f, 1.0f, x + detail::lo(0.0f, to_width), y + detail::lo(0.0f, to_height));
    s.transform(fabsf(to_width) / static_cast<float>(width), 0.0f, 0.0f,
                fabsf(to_height) / static_cast<float>(height), 0.0f, 0.0f);
    s.draw_lines(br, true, false, true);
    s.fwd = sf;
    s.inv = si;
}

void canvas::get_image_data(unsigned char *image, int width, int height, int stride, int x, int y) {
    if (!image) return;
    self->note(cy_get_image(self->ctx, image, width, height, stride, x, y));
}
void canvas::put_image_data(unsigned char const *image, int width, int height, int stride, int x, int y) {
    if (!image) return;
    self->note(cy_put_image(self->ctx, image, width, height, stride, x, y));
}

void canvas::save() {
    // hpp:3410-3437
    sync_public_state();
    detail::canvas_state &s = *self;
    detail::saved_state st;
    st.op = s.op; st.sox = s.sox; st.soy = s.soy; st.cap = s.cap; st.join = s.join;
    st.dash_off = s.dash_off; st.align = s.align; st.baseline = s.baseline;
    st.fwd = s.fwd; st.inv = s.inv; st.alpha = s.alpha; st.shcol = s.shadow_color;
    st.shblur = s.shadow_blur; st.lw = s.lw; st.miter_limit = s.miter_limit; st.dash = s.dash;
    st.fill = s.fill; st.stroke = s.stroke; st.mask = s.mask; st.face = s.face;
    if (s.mask) s.note(cy_mask_retain(s.ctx, s.mask));
    s.stack.push_back(st);
}
void canvas::restore() {
    // hpp:3439-3465
    detail::canvas_state &s = *self;
    if (s.stack.empty()) return;
    detail::saved_state &st = s.stack.back();
    global_composite_operation = st.op;
    shadow_offset_x = st.sox;
    shadow_offset_y = st.soy;
    line_cap = st.cap;
    line_join = st.join;
    line_dash_offset = st.dash_off;
    text_align = st.align;
    text_baseline = st.baseline;
    s.fwd = st.fwd; s.inv = st.inv; s.alpha = st.alpha; s.shadow_color = st.shcol;
    s.shadow_blur = st.shblur; s.lw = st.lw; s.miter_limit = st.miter_limit; s.dash.swap(st.dash);
    s.fill = st.fill; s.stroke = st.stroke; s.face = st.face;
    if (s.mask) s.note(cy_mask_release(s.ctx, s.mask));
    s.mask = st.mask;
    s.stack.pop_back();
    sync_public_state();
}

}  // namespace canvas_ity
