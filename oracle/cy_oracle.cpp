// cy_oracle.cpp -- CPU oracle for the canvas_ity render path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, step by step and with the
// same floating-point operation order, the CPU algorithm of the reference
// single-header library (src/canvas_ity.hpp).  It is the checker that the
// GB300 canvas is compared against: only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load it.  The product library never links,
// loads or calls it.
//
// Pinning: the restatement is checked byte-for-byte against the reference
// itself (built from its own sources by oracle/ref/build_ref.sh) and against
// the reference's 76 golden image hashes (test/test.cpp:2185-2261) through
// the recorded call lists in tests/golden/.
//
// Build with -ffp-contract=off so that no multiply-add is fused: the
// reference's published behaviour is that of x86-64 SSE code, which has no
// fused multiply-add.
//
// Every function cites the reference lines it restates (hpp = src/canvas_ity.hpp).
//
// Derived from canvas_ity (src/canvas_ity.hpp), Copyright (c) 2022 Andrew
// Kensler, under the ISC license; its copyright and permission notice is
// reproduced in LICENSES/canvas_ity-ISC.txt and applies to this file.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "../include/cy_replay.hpp"

namespace cyo {

// Public enums, same values as hpp:146-156.
enum composite_operation {
    source_in = 1, source_copy, source_out, destination_in,
    destination_atop = 7, lighter = 10, destination_over, destination_out,
    source_atop, source_over, exclusive_or };
enum cap_style { butt, square, circle };
enum join_style { miter, bevel, rounded };
enum brush_type { fill_style, stroke_style };
enum repetition_style { repeat, repeat_x, repeat_y, no_repeat };
enum align_style { leftward, rightward, center, start = 0, ending };
enum baseline_style { alphabetic, top, middle, bottom, hanging, ideographic = 3 };

// std::min / std::max semantics (hpp uses them with NaN-sensitive order).
static inline float lo(float a, float b) { return b < a ? b : a; }
static inline float hi(float a, float b) { return a < b ? b : a; }
static inline int loi(int a, int b) { return b < a ? b : a; }
static inline int hii(int a, int b) { return a < b ? b : a; }

// ---- 2D vectors (hpp:1223-1257) ----
struct vec2 { float x, y; };
static inline vec2 mk(float x, float y) { vec2 v; v.x = x; v.y = y; return v; }
static inline vec2 add(vec2 a, vec2 b) { return mk(a.x + b.x, a.y + b.y); }
static inline vec2 sub(vec2 a, vec2 b) { return mk(a.x - b.x, a.y - b.y); }
static inline vec2 scl(float s, vec2 a) { return mk(a.x * s, a.y * s); }
static inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
static inline float norm(vec2 a) { return sqrtf(dot(a, a)); }
static inline float angle_of(vec2 a) { return atan2f(a.y, a.x); }
static inline vec2 unit(vec2 a) { return scl(1.0f / hi(1.0e-6f, norm(a)), a); }
static inline vec2 perp(vec2 a) { return mk(-a.y, a.x); }
static inline vec2 mix(vec2 a, vec2 b, float t) { return add(a, scl(t, sub(b, a))); }

struct mat { float a, b, c, d, e, f; };
static inline vec2 apply(const mat &m, vec2 p) {
    return mk(m.a * p.x + m.c * p.y + m.e, m.b * p.x + m.d * p.y + m.f);
}

// ---- colours (hpp:1259-1297) ----
struct col { float r, g, b, a; };
static inline col mkc(float r, float g, float b, float a) { col c; c.r = r; c.g = g; c.b = b; c.a = a; return c; }
static inline col cadd(col x, col y) { return mkc(x.r + y.r, x.g + y.g, x.b + y.b, x.a + y.a); }
static inline col csub(col x, col y) { return mkc(x.r - y.r, x.g - y.g, x.b - y.b, x.a - y.a); }
static inline col cscl(float s, col x) { return mkc(x.r * s, x.g * s, x.b * s, x.a * s); }
static inline float to_linear(float v) {
    return v < 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
}
static inline col to_linear(col c) { return mkc(to_linear(c.r), to_linear(c.g), to_linear(c.b), c.a); }
static inline col premul(col c) { return mkc(c.r * c.a, c.g * c.a, c.b * c.a, c.a); }
static inline float to_srgb(float v) {
    return v < 0.0031308f ? 12.92f * v : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
}
static inline col to_srgb(col c) { return mkc(to_srgb(c.r), to_srgb(c.g), to_srgb(c.b), c.a); }
static const float kVisible = 1.0f / 8160.0f;
static inline col unpremul(col c) {
    if (c.a < kVisible) return mkc(0.0f, 0.0f, 0.0f, 0.0f);
    return mkc(1.0f / c.a * c.r, 1.0f / c.a * c.g, 1.0f / c.a * c.b, c.a);
}
static inline float clamp01(float v) { return lo(hi(v, 0.0f), 1.0f); }
static inline col clamp01(col c) { return mkc(clamp01(c.r), clamp01(c.g), clamp01(c.b), clamp01(c.a)); }

// ---- big-endian font readers (hpp:1299-1314) ----
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

struct subpath { size_t count; bool closed; };
struct polyline { std::vector<vec2> pts; std::vector<subpath> subs; };
struct run { unsigned short x, y; float delta; };

// Sort order of runs (hpp:2172-2181).  Runs of one cell with equal
// magnitude and opposite sign are equivalent under it, so std::sort leaves
// their order to its own partitioning.  Built with CYO_TIES_BY_SIGN the
// oracle orders them negative first instead, which is the order the GPU
// path uses; that build pins the GPU's float canvas bit for bit.
static bool run_before(const run &l, const run &r) {
    if (l.y != r.y) return l.y < r.y;
    if (l.x != r.x) return l.x < r.x;
#ifdef CYO_TIES_BY_SIGN
    if (fabsf(l.delta) == fabsf(r.delta)) return l.delta < r.delta;
#endif
    return fabsf(l.delta) < fabsf(r.delta);
}

// The round join's angle (hpp:2006-2008): libm's acosf and tanf, as the
// reference calls them; built with CYO_CR_TRIG, acos and tan in double
// precision rounded to float, which is what the GPU's stroke expansion
// computes (the two differ by one ulp on a small fraction of inputs).
#ifdef CYO_CR_TRIG
static float join_acos(float x) { return static_cast<float>(std::acos(static_cast<double>(x))); }
static float join_tan(float x) { return static_cast<float>(std::tan(static_cast<double>(x))); }
#else
static float join_acos(float x) { return acosf(x); }
static float join_tan(float x) { return tanf(x); }
#endif

struct brush {
    enum kind_t { solid, linear, radial, image } kind;
    std::vector<col> colors;
    std::vector<float> stops;
    vec2 p0, p1;
    float r0, r1;
    int w, h;
    repetition_style rep;
    brush() : kind(solid), p0(mk(0, 0)), p1(mk(0, 0)), r0(0), r1(0), w(0), h(0), rep(repeat) {}
};

struct font {
    bytes data;
    int cmap, glyf, head, hhea, hmtx, loca, maxp, os_2;
    float scale;
    font() : cmap(0), glyf(0), head(0), hhea(0), hmtx(0), loca(0), maxp(0), os_2(0), scale(0) {}
};

class canvas {
public:
    canvas(int width, int height);
    ~canvas() {}

    void scale(float x, float y) { transform(x, 0.0f, 0.0f, y, 0.0f, 0.0f); }
    void rotate(float angle) {
        float c = cosf(angle), s = sinf(angle);
        transform(c, s, -s, c, 0.0f, 0.0f);
    }
    void translate(float x, float y) { transform(1.0f, 0.0f, 0.0f, 1.0f, x, y); }
    void transform(float a, float b, float c, float d, float e, float f);
    void set_transform(float a, float b, float c, float d, float e, float f);
    void set_global_alpha(float alpha) { if (0.0f <= alpha && alpha <= 1.0f) g_alpha = alpha; }
    composite_operation global_composite_operation;
    void set_shadow_color(float r, float g, float b, float a) {
        sh_color = premul(to_linear(clamp01(mkc(r, g, b, a))));
    }
    float shadow_offset_x;
    float shadow_offset_y;
    void set_shadow_blur(float level) { if (0.0f <= level) sh_blur = level; }
    void set_line_width(float w) { if (0.0f < w) lw = w; }
    cap_style line_cap;
    join_style line_join;
    void set_miter_limit(float m) { if (0.0f < m) miter_lim = m; }
    float line_dash_offset;
    void set_line_dash(const float *segments, int count);
    void set_color(brush_type t, float r, float g, float b, float a);
    void set_linear_gradient(brush_type t, float x0, float y0, float x1, float y1);
    void set_radial_gradient(brush_type t, float x0, float y0, float r0, float x1, float y1, float r1);
    void add_color_stop(brush_type t, float off, float r, float g, float b, float a);
    void set_pattern(brush_type t, const unsigned char *img, int w, int h, int stride, repetition_style rep);
    void begin_path() { path.pts.clear(); path.subs.clear(); }
    void move_to(float x, float y);
    void close_path();
    void line_to(float x, float y);
    void quadratic_curve_to(float cx, float cy, float x, float y);
    void bezier_curve_to(float c1x, float c1y, float c2x, float c2y, float x, float y);
    void arc_to(float vx, float vy, float x, float y, float radius);
    void arc(float x, float y, float radius, float a0, float a1, bool ccw = false);
    void rectangle(float x, float y, float w, float h);
    void fill() {
        flatten(false);
        cur_rule = fill_rule;
        render(fill_br, false);
        cur_rule = 0;
    }
    // Extension (no reference counterpart): the fill rule of fill(), clip()
    // and is_point_in_path(); 0 nonzero (the reference's only rule), 1
    // even-odd.  Strokes, text and rectangles always fill nonzero.
    int fill_rule = 0;
    void stroke() { flatten(true); stroke_outline(); render(stroke_br, false); }
    void clip();
    bool is_point_in_path(float x, float y);
    void clear_rectangle(float x, float y, float w, float h);
    void fill_rectangle(float x, float y, float w, float h);
    void stroke_rectangle(float x, float y, float w, float h);
    align_style text_align;
    baseline_style text_baseline;
    bool set_font(const unsigned char *data, int nbytes, float size);
    void fill_text(const char *text, float x, float y, float maxw = 1.0e30f) {
        text_outline(text, mk(x, y), maxw, false);
        render(fill_br, false);
    }
    void stroke_text(const char *text, float x, float y, float maxw = 1.0e30f) {
        text_outline(text, mk(x, y), maxw, true);
        stroke_outline();
        render(stroke_br, false);
    }
    float measure_text(const char *text);
    void draw_image(const unsigned char *img, int w, int h, int stride, float x, float y, float tw, float th);
    void get_image_data(unsigned char *img, int w, int h, int stride, int x, int y);
    void put_image_data(const unsigned char *img, int w, int h, int stride, int x, int y);
    void save();
    void restore();
    const std::vector<col> &pixels() const { return bitmap; }

private:
    struct state {
        composite_operation op; float sox, soy; cap_style cap; join_style join; float dash_off;
        align_style align; baseline_style baseline; mat fwd, inv; float alpha; col shcol;
        float shblur; float lw, miter; std::vector<float> dash; brush fill, stroke;
        std::vector<run> mask; font face;
    };
    int W, H;
    int cur_rule = 0;   // rule of the draw being rendered
    // Coverage of an accumulated signed area s: min(|s|, 1) for nonzero;
    // for even-odd the distance from s to the nearest even integer, so each
    // further winding toggles coverage.
    float cover(float s) const {
        return cur_rule ? lo(fabsf(s - 2.0f * rintf(0.5f * s)), 1.0f) : lo(fabsf(s), 1.0f);
    }
    mat fwd, inv;
    float g_alpha;
    col sh_color;
    float sh_blur;
    std::vector<float> shadow;
    float lw, miter_lim;
    std::vector<float> dash;
    brush fill_br, stroke_br, image_br;
    polyline path, lines, scratch;
    std::vector<run> runs, mask;
    font face;
    std::vector<col> bitmap;
    std::vector<state> stack;

    brush &pick(brush_type t) { return t == fill_style ? fill_br : stroke_br; }
    void tessellate(vec2 p1, vec2 c1, vec2 c2, vec2 p2, float angular, int limit);
    void bezier(vec2 p1, vec2 c1, vec2 c2, vec2 p2, float angular);
    void flatten(bool stroking);
    void glyph_outline(int glyph, float angular);
    int glyph_of(const char *text, int &index);
    void text_outline(const char *text, vec2 at, float maxw, bool stroking);
    void apply_dash();
    void half_stroke(size_t begin, size_t end, bool closed);
    void stroke_outline();
    void scan_segment(vec2 from, vec2 to);
    void scan(vec2 offset, int padding);
    // Binned coverage (built with CYO_BINNED): the library's sort-free
    // coverage of a draw, restated -- fixed-point cell areas summed per
    // pixel row instead of sorted runs.
    std::vector<int32_t> acc;
    void scan_segment_binned(vec2 from, vec2 to);
    void scan_binned();
    col paint(vec2 p, const brush &br, bool clamp_edges);
    void render_shadow(const brush &br, bool clamp_edges);
    void render(const brush &br, bool clamp_edges);
};

canvas::canvas(int width, int height)
    : global_composite_operation(source_over), shadow_offset_x(0.0f), shadow_offset_y(0.0f),
      line_cap(butt), line_join(miter), line_dash_offset(0.0f), text_align(start),
      text_baseline(alphabetic), W(width), H(height), g_alpha(1.0f), sh_blur(0.0f),
      lw(1.0f), miter_lim(10.0f) {
    // hpp:2607-2644
    mat identity = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f};
    fwd = identity;
    inv = identity;
    sh_color = mkc(0, 0, 0, 0);
    bitmap.assign(static_cast<size_t>(width) * static_cast<size_t>(height), mkc(0, 0, 0, 0));
    set_color(fill_style, 0.0f, 0.0f, 0.0f, 1.0f);
    set_color(stroke_style, 0.0f, 0.0f, 0.0f, 1.0f);
    for (unsigned short y = 0; y < H; ++y) {
        run a = {0, y, 1.0f};
        run b = {static_cast<unsigned short>(W), y, -1.0f};
        mask.push_back(a);
        mask.push_back(b);
    }
}

// hpp:2680-2711
void canvas::transform(float a, float b, float c, float d, float e, float f) {
    set_transform(fwd.a * a + fwd.c * b, fwd.b * a + fwd.d * b,
                  fwd.a * c + fwd.c * d, fwd.b * c + fwd.d * d,
                  fwd.a * e + fwd.c * f + fwd.e, fwd.b * e + fwd.d * f + fwd.f);
}
void canvas::set_transform(float a, float b, float c, float d, float e, float f) {
    float det = a * d - b * c;
    float s = det != 0.0f ? 1.0f / det : 0.0f;
    mat nf = {a, b, c, d, e, f};
    mat ni = {s * d, s * -b, s * -c, s * a, s * (c * f - d * e), s * (b * e - a * f)};
    fwd = nf;
    inv = ni;
}

// hpp:2748-2763
void canvas::set_line_dash(const float *segments, int count) {
    for (int i = 0; i < count; ++i)
        if (segments && segments[i] < 0.0f) return;
    dash.clear();
    if (!segments) return;
    for (int i = 0; i < count; ++i) dash.push_back(segments[i]);
    if (count & 1)
        for (int i = 0; i < count; ++i) dash.push_back(segments[i]);
}

// hpp:2765-2864
void canvas::set_color(brush_type t, float r, float g, float b, float a) {
    brush &br = pick(t);
    br.kind = brush::solid;
    br.colors.clear();
    br.colors.push_back(premul(to_linear(clamp01(mkc(r, g, b, a)))));
}
void canvas::set_linear_gradient(brush_type t, float x0, float y0, float x1, float y1) {
    brush &br = pick(t);
    br.kind = brush::linear;
    br.colors.clear();
    br.stops.clear();
    br.p0 = mk(x0, y0);
    br.p1 = mk(x1, y1);
}
void canvas::set_radial_gradient(brush_type t, float x0, float y0, float r0, float x1, float y1, float r1) {
    if (r0 < 0.0f || r1 < 0.0f) return;
    brush &br = pick(t);
    br.kind = brush::radial;
    br.colors.clear();
    br.stops.clear();
    br.p0 = mk(x0, y0);
    br.p1 = mk(x1, y1);
    br.r0 = r0;
    br.r1 = r1;
}
void canvas::add_color_stop(brush_type t, float off, float r, float g, float b, float a) {
    brush &br = pick(t);
    if ((br.kind != brush::linear && br.kind != brush::radial) || off < 0.0f || 1.0f < off) return;
    ptrdiff_t at = std::upper_bound(br.stops.begin(), br.stops.end(), off) - br.stops.begin();
    col c = to_linear(clamp01(mkc(r, g, b, a)));
    br.colors.insert(br.colors.begin() + at, c);
    br.stops.insert(br.stops.begin() + at, off);
}
void canvas::set_pattern(brush_type t, const unsigned char *img, int w, int h, int stride,
                         repetition_style rep) {
    if (!img || w <= 0 || h <= 0) return;
    brush &br = pick(t);
    br.kind = brush::image;
    br.colors.clear();
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int i = y * stride + x * 4;
            col c = mkc(img[i + 0] / 255.0f, img[i + 1] / 255.0f, img[i + 2] / 255.0f, img[i + 3] / 255.0f);
            br.colors.push_back(premul(to_linear(c)));
        }
    br.w = w;
    br.h = h;
    br.rep = rep;
}

// ---- path building (hpp:2866-3042) ----
void canvas::move_to(float x, float y) {
    if (!path.subs.empty() && path.subs.back().count == 1) {
        path.pts.back() = apply(fwd, mk(x, y));
        return;
    }
    subpath s = {1, false};
    path.pts.push_back(apply(fwd, mk(x, y)));
    path.subs.push_back(s);
}
void canvas::close_path() {
    if (path.subs.empty()) return;
    vec2 first = path.pts[path.pts.size() - path.subs.back().count];
    mat saved = fwd;
    mat identity = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f};
    fwd = identity;
    line_to(first.x, first.y);
    path.subs.back().closed = true;
    move_to(first.x, first.y);
    fwd = saved;
}
void canvas::line_to(float x, float y) {
    if (path.subs.empty()) { move_to(x, y); return; }
    vec2 p1 = path.pts.back();
    vec2 p2 = apply(fwd, mk(x, y));
    if (dot(sub(p2, p1), sub(p2, p1)) == 0.0f) return;
    path.pts.push_back(p1);
    path.pts.push_back(p2);
    path.pts.push_back(p2);
    path.subs.back().count += 3;
}
void canvas::quadratic_curve_to(float cx, float cy, float x, float y) {
    if (path.subs.empty()) move_to(cx, cy);
    vec2 p1 = path.pts.back();
    vec2 c = apply(fwd, mk(cx, cy));
    vec2 p2 = apply(fwd, mk(x, y));
    path.pts.push_back(mix(p1, c, 2.0f / 3.0f));
    path.pts.push_back(mix(p2, c, 2.0f / 3.0f));
    path.pts.push_back(p2);
    path.subs.back().count += 3;
}
void canvas::bezier_curve_to(float c1x, float c1y, float c2x, float c2y, float x, float y) {
    if (path.subs.empty()) move_to(c1x, c1y);
    vec2 c1 = apply(fwd, mk(c1x, c1y));
    vec2 c2 = apply(fwd, mk(c2x, c2y));
    vec2 p2 = apply(fwd, mk(x, y));
    path.pts.push_back(c1);
    path.pts.push_back(c2);
    path.pts.push_back(p2);
    path.subs.back().count += 3;
}
void canvas::arc_to(float vx, float vy, float x, float y, float radius) {
    if (radius < 0.0f || fwd.a * fwd.d - fwd.b * fwd.c == 0.0f) return;
    if (path.subs.empty()) move_to(vx, vy);
    vec2 p1 = apply(inv, path.pts.back());
    vec2 v = mk(vx, vy);
    vec2 p2 = mk(x, y);
    vec2 e1 = unit(sub(p1, v));
    vec2 e2 = unit(sub(p2, v));
    float sine = fabsf(dot(perp(e1), e2));
    if (sine < 1.0e-4f) { line_to(vx, vy); return; }
    vec2 off = scl(radius / sine, add(e1, e2));
    vec2 center = add(v, off);
    float a1 = angle_of(sub(scl(dot(off, e1), e1), off));
    float a2 = angle_of(sub(scl(dot(off, e2), e2), off));
    bool reverse = static_cast<int>(floorf((a2 - a1) / 3.14159265f)) & 1;
    arc(center.x, center.y, radius, a1, a2, reverse);
}
void canvas::arc(float x, float y, float radius, float a0, float a1, bool ccw) {
    if (radius < 0.0f) return;
    const float tau = 6.28318531f;
    float winding = ccw ? -1.0f : 1.0f;
    float from = fmodf(a0, tau);
    float span = fmodf(a1, tau) - from;
    if ((a1 - a0) * winding >= tau) span = tau * winding;
    else if (span * winding < 0.0f) span += tau * winding;
    vec2 c1 = scl(radius, mk(cosf(from), sinf(from)));
    line_to(x + c1.x, y + c1.y);
    if (span == 0.0f) return;
    int steps = static_cast<int>(hi(1.0f, roundf(16.0f / tau * span * winding)));
    float segment = span / static_cast<float>(steps);
    float alpha = 4.0f / 3.0f * tanf(0.25f * segment);
    for (int s = 0; s < steps; ++s) {
        float angle = from + static_cast<float>(s + 1) * segment;
        vec2 c2 = scl(radius, mk(cosf(angle), sinf(angle)));
        vec2 q1 = add(mk(x, y), c1);
        vec2 q2 = add(mk(x, y), c2);
        vec2 k1 = add(q1, scl(alpha, perp(c1)));
        vec2 k2 = sub(q2, scl(alpha, perp(c2)));
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

// ---- flattening (hpp:1331-1524) ----
void canvas::tessellate(vec2 p1, vec2 c1, vec2 c2, vec2 p2, float angular, int limit) {
    const float tol = 0.125f;
    float flat = tol * tol;
    vec2 e1 = sub(c1, p1), e2 = sub(c2, c1), e3 = sub(p2, c2), seg = sub(p2, p1);
    float q1 = dot(e1, e1), q2 = dot(e2, e2), q3 = dot(e3, e3);
    float lsq = hi(1.0e-4f, dot(seg, seg));
    float t1 = lo(hi(dot(e1, seg) / lsq, 0.0f), 1.0f);
    float t2 = lo(hi(dot(e3, seg) / lsq, 0.0f), 1.0f);
    vec2 d1 = sub(add(p1, scl(t1, seg)), c1);
    vec2 d2 = sub(sub(p2, scl(t2, seg)), c2);
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
    vec2 l1 = mix(p1, c1, 0.5f), m = mix(c1, c2, 0.5f), r2 = mix(c2, p2, 0.5f);
    vec2 l2 = mix(l1, m, 0.5f), r1 = mix(m, r2, 0.5f), sp = mix(l2, r1, 0.5f);
    tessellate(p1, l1, l2, sp, angular, limit - 1);
    tessellate(sp, r1, r2, p2, angular, limit - 1);
}

// Roots of one coordinate's derivative, appended to `at` (hpp:1420-1447).
static void axis_extrema(float a, float b, float c, float *at, int &cuts) {
    const float eps = 1.0e-4f;
    if (fabsf(a) > eps) {
        float disc = b * b - 4.0f * a * c;
        if (disc >= 0.0f) {
            float sign = b > 0.0f ? 1.0f : -1.0f;
            float term = -b - sign * sqrtf(disc);
            float x1 = term / (2.0f * a);
            at[cuts++] = x1;
            at[cuts++] = c / (a * x1);
        }
    } else if (fabsf(b) > eps) {
        at[cuts++] = -c / b;
    }
}

void canvas::bezier(vec2 p1, vec2 c1, vec2 c2, vec2 p2, float angular) {
    vec2 e1 = sub(c1, p1), e2 = sub(c2, c1), e3 = sub(p2, c2);
    if (dot(e1, e1) == 0.0f && dot(e3, e3) == 0.0f) {
        lines.pts.push_back(p2);
        return;
    }
    float at[7] = {0.0f, 1.0f};
    int cuts = 2;
    vec2 ea = add(scl(-9.0f, e2), scl(3.0f, sub(p2, p1)));
    vec2 eb = sub(scl(6.0f, add(p1, c2)), scl(12.0f, c1));
    vec2 ec = scl(3.0f, e1);
    axis_extrema(ea.x, eb.x, ec.x, at, cuts);
    axis_extrema(ea.y, eb.y, ec.y, at, cuts);
    float k1 = dot(perp(e1), e2), k2 = dot(perp(e1), e3), k3 = dot(perp(e2), e3);
    float ca = k1 - k2 + k3;
    float cb = -2.0f * k1 + k2;
    if (fabsf(ca) > 1.0e-4f && fabsf(cb) > 1.0e-4f) at[cuts++] = -0.5f * cb / ca;
    for (int i = 1; i < cuts; ++i) {
        float v = at[i];
        int j = i - 1;
        for (; 0 <= j && v < at[j]; --j) at[j + 1] = at[j];
        at[j + 1] = v;
    }
    vec2 s1 = p1;
    for (int i = 0; i < cuts - 1; ++i) {
        if (!(0.0f <= at[i] && at[i + 1] <= 1.0f && at[i] != at[i + 1])) continue;
        float t = at[i + 1];
        float ratio = at[i] / t;
        vec2 q1 = mix(p1, c1, t), q2 = mix(c1, c2, t), q3 = mix(c2, p2, t);
        vec2 q4 = mix(q1, q2, t), q5 = mix(q2, q3, t);
        vec2 q6 = mix(q1, q4, ratio);
        vec2 s2 = mix(q4, q5, t);
        vec2 sc2 = mix(q4, s2, ratio);
        vec2 sc1 = mix(q6, sc2, ratio);
        tessellate(s1, sc1, sc2, s2, angular, 20);
        s1 = s2;
    }
}

void canvas::flatten(bool stroking) {
    const float tol = 0.125f;
    float ratio = tol / hi(0.5f * lw, tol);
    float angular = stroking ? (ratio - 2.0f) * ratio * 2.0f + 1.0f : -1.0f;
    lines.pts.clear();
    lines.subs.clear();
    size_t i = 0, end = 0;
    for (size_t s = 0; s < path.subs.size(); ++s) {
        end += path.subs[s].count;
        size_t first = lines.pts.size();
        vec2 p1 = path.pts[i++];
        lines.pts.push_back(p1);
        for (; i < end; i += 3) {
            vec2 c1 = path.pts[i], c2 = path.pts[i + 1], p2 = path.pts[i + 2];
            bezier(p1, c1, c2, p2, angular);
            p1 = p2;
        }
        subpath e = {lines.pts.size() - first, path.subs[s].closed};
        lines.subs.push_back(e);
    }
}

// ---- text (hpp:1533-1846, 3205-3311) ----
void canvas::glyph_outline(int glyph, float angular) {
    const bytes &d = face.data;
    int loc_format = u16at(d, face.head + 50);
    int offset = face.glyf + (loc_format ? s32at(d, face.loca + glyph * 4) : u16at(d, face.loca + glyph * 2) * 2);
    int next = face.glyf + (loc_format ? s32at(d, face.loca + glyph * 4 + 4) : u16at(d, face.loca + glyph * 2 + 2) * 2);
    if (offset == next) return;
    int contours = s16at(d, offset);
    if (contours < 0) {
        offset += 10;
        for (;;) {
            int flags = u16at(d, offset);
            int component = u16at(d, offset + 2);
            if (!(flags & 2)) return;
            float e = static_cast<float>(flags & 1 ? s16at(d, offset + 4) : s8at(d, offset + 4));
            float f = static_cast<float>(flags & 1 ? s16at(d, offset + 6) : s8at(d, offset + 5));
            offset += flags & 1 ? 8 : 6;
            float a = flags & 200 ? static_cast<float>(s16at(d, offset)) / 16384.0f : 1.0f;
            float b = flags & 128 ? static_cast<float>(s16at(d, offset + 2)) / 16384.0f : 0.0f;
            float c = flags & 128 ? static_cast<float>(s16at(d, offset + 4)) / 16384.0f : 0.0f;
            float dd = flags & 8 ? a
                     : flags & 64 ? static_cast<float>(s16at(d, offset + 2)) / 16384.0f
                     : flags & 128 ? static_cast<float>(s16at(d, offset + 6)) / 16384.0f
                     : 1.0f;
            offset += flags & 8 ? 2 : flags & 64 ? 4 : flags & 128 ? 8 : 0;
            mat sf = fwd, si = inv;
            transform(a, b, c, dd, e, f);
            glyph_outline(component, angular);
            fwd = sf;
            inv = si;
            if (!(flags & 32)) return;
        }
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
    int xs = flags_at + flags_size;
    int ys = xs + x_size;
    int x = lsb - x_min, y = 0, fl = 0, rep = 0, idx = 0;
    for (int ct = 0; ct < contours; ++ct) {
        int begin = idx;
        int end = u16at(d, offset + 10 + ct * 2);
        vec2 bp = mk(0, 0), ep = mk(0, 0);
        bool bon = false, eon = false;
        size_t first = lines.pts.size();
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
            vec2 pt = apply(fwd, mk(static_cast<float>(x), static_cast<float>(y)));
            int on = fl & 1;
            if (idx == begin) {
                bp = pt;
                bon = on;
                if (on) lines.pts.push_back(pt);
            } else {
                vec2 p2 = on ? pt : mix(ep, pt, 0.5f);
                if (lines.pts.size() == first || (eon && on)) lines.pts.push_back(p2);
                else if (!eon || on) {
                    vec2 p1 = lines.pts.back();
                    bezier(p1, mix(p1, ep, 2.0f / 3.0f), mix(p2, ep, 2.0f / 3.0f), p2, angular);
                }
            }
            ep = pt;
            eon = on;
        }
        if (bon ^ eon) {
            vec2 p1 = lines.pts.back();
            vec2 p2 = lines.pts[first];
            vec2 ctl = eon ? bp : ep;
            bezier(p1, mix(p1, ctl, 2.0f / 3.0f), mix(p2, ctl, 2.0f / 3.0f), p2, angular);
        } else if (!bon && !eon) {
            vec2 p1 = lines.pts.back();
            vec2 split = mix(bp, ep, 0.5f);
            vec2 p2 = lines.pts[first];
            bezier(p1, mix(p1, ep, 2.0f / 3.0f), mix(split, ep, 2.0f / 3.0f), split, angular);
            bezier(split, mix(split, bp, 2.0f / 3.0f), mix(p2, bp, 2.0f / 3.0f), p2, angular);
        }
        lines.pts.push_back(lines.pts[first]);
        subpath e = {lines.pts.size() - first, true};
        lines.subs.push_back(e);
    }
}

int canvas::glyph_of(const char *text, int &index) {
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
            if (st <= cp && cp <= en)
                return ra ? u16at(d, ranges + s + (cp - st) * 2 + ra) : (cp + de) & 0xffff;
        }
    } else if (f0 && 0 <= cp && cp < 256) {
        return u8at(d, f0 + 6 + cp);
    }
    return 0;
}

void canvas::text_outline(const char *text, vec2 at, float maxw, bool stroking) {
    const float tol = 0.125f;
    float ratio = tol / hi(0.5f * lw, tol);
    float angular = stroking ? (ratio - 2.0f) * ratio * 2.0f + 1.0f : -1.0f;
    lines.pts.clear();
    lines.subs.clear();
    if (face.data.empty() || !text || maxw <= 0.0f) return;
    const bytes &d = face.data;
    float width = maxw == 1.0e30f && text_align == leftward ? 0.0f : measure_text(text);
    float reduction = maxw / hi(maxw, width);
    if (text_align == rightward) at.x -= width * reduction;
    else if (text_align == center) at.x -= 0.5f * width * reduction;
    vec2 scaling = scl(face.scale, mk(reduction, 1.0f));
    float upem = static_cast<float>(u16at(d, face.head + 18));
    float ascender = static_cast<float>(s16at(d, face.os_2 + 68));
    float descender = static_cast<float>(s16at(d, face.os_2 + 70));
    float normalize = face.scale * upem / (ascender - descender);
    if (text_baseline == top) at.y += ascender * normalize;
    else if (text_baseline == middle) at.y += (ascender + descender) * 0.5f * normalize;
    else if (text_baseline == bottom) at.y += descender * normalize;
    else if (text_baseline == hanging) at.y += 0.6f * face.scale * upem;
    mat sf = fwd, si = inv;
    int hmetrics = u16at(d, face.hhea + 34);
    int place = 0;
    for (int i = 0; text[i];) {
        int g = glyph_of(text, i);
        fwd = sf;
        transform(scaling.x, 0.0f, 0.0f, -scaling.y, at.x + static_cast<float>(place) * scaling.x, at.y);
        glyph_outline(g, angular);
        int entry = loi(g, hmetrics - 1);
        place += u16at(d, face.hmtx + entry * 4);
    }
    fwd = sf;
    inv = si;
}

bool canvas::set_font(const unsigned char *data, int nbytes, float size) {
    if (data && nbytes) {
        face.data.clear();
        face.cmap = face.glyf = face.head = face.hhea = face.hmtx = face.loca = face.maxp = face.os_2 = 0;
        if (nbytes < 6) return false;
        int version = (data[0] << 24 | data[1] << 16 | data[2] << 8 | data[3] << 0);
        int tables = data[4] << 8 | data[5];
        if ((version != 0x00010000 && version != 0x74727565) || nbytes < tables * 16 + 12) return false;
        face.data.insert(face.data.end(), data, data + tables * 16 + 12);
        for (int t = 0; t < tables; ++t) {
            int tag = s32at(face.data, t * 16 + 12);
            int off = s32at(face.data, t * 16 + 20);
            int span = s32at(face.data, t * 16 + 24);
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
            face.data.insert(face.data.end(), data + off, data + off + span);
        }
        if (!face.cmap || !face.glyf || !face.head || !face.hhea || !face.hmtx || !face.loca ||
            !face.maxp || !face.os_2) {
            face.data.clear();
            return false;
        }
    }
    if (face.data.empty()) return false;
    int upem = u16at(face.data, face.head + 18);
    face.scale = size / static_cast<float>(upem);
    return true;
}

float canvas::measure_text(const char *text) {
    if (face.data.empty() || !text) return 0.0f;
    int hmetrics = u16at(face.data, face.hhea + 34);
    int width = 0;
    for (int i = 0; text[i];) {
        int g = glyph_of(text, i);
        int entry = loi(g, hmetrics - 1);
        width += u16at(face.data, face.hmtx + entry * 4);
    }
    return static_cast<float>(width) * face.scale;
}

// ---- dashing and stroke expansion (hpp:1858-2100) ----
void canvas::apply_dash() {
    if (dash.empty()) return;
    lines.pts.swap(scratch.pts);
    lines.pts.clear();
    lines.subs.swap(scratch.subs);
    lines.subs.clear();
    float total = std::accumulate(dash.begin(), dash.end(), 0.0f);
    float offset = fmodf(line_dash_offset, total);
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
        size_t merge_pt = lines.pts.size();
        size_t merge_sub = lines.subs.size();
        bool merge_emit = emit;
        float next = dash[start] - offset;
        for (; i + 1 < end; ++i) {
            vec2 from = scratch.pts[i], to = scratch.pts[i + 1];
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

void canvas::half_stroke(size_t begin, size_t end, bool closed) {
    float half = lw * 0.5f;
    float ratio = miter_lim * miter_lim * half * half;
    vec2 in_dir = mk(0.0f, 0.0f);
    float in_len = 0.0f;
    vec2 point = apply(inv, scratch.pts[begin]);
    size_t finish = begin, i = begin;
    const float eps = 1.0e-4f;
    do {
        vec2 next = apply(inv, scratch.pts[i]);
        vec2 out_dir = unit(sub(next, point));
        float out_len = norm(sub(next, point));
        if (in_len != 0.0f && out_len >= eps) {
            if (closed && finish == begin) finish = i;
            vec2 side_in = add(point, scl(half, perp(in_dir)));
            vec2 side_out = add(point, scl(half, perp(out_dir)));
            float turn = dot(perp(in_dir), out_dir);
            if (fabsf(turn) < eps) turn = 0.0f;
            vec2 off = turn == 0.0f ? mk(0.0f, 0.0f) : scl(half / turn, sub(out_dir, in_dir));
            bool tight = (dot(off, in_dir) < -in_len && dot(off, out_dir) > out_len);
            if (turn > 0.0f && tight) {
                std::swap(side_in, side_out);
                std::swap(in_dir, out_dir);
                lines.pts.push_back(apply(fwd, side_out));
                lines.pts.push_back(apply(fwd, point));
                lines.pts.push_back(apply(fwd, side_in));
            }
            if ((turn > 0.0f && !tight) || (turn != 0.0f && line_join == miter && dot(off, off) <= ratio)) {
                lines.pts.push_back(apply(fwd, add(point, off)));
            } else if (line_join == rounded) {
                float cosine = dot(in_dir, out_dir);
                float angle = join_acos(lo(hi(cosine, -1.0f), 1.0f));
                float alpha = 4.0f / 3.0f * join_tan(0.25f * angle);
                lines.pts.push_back(apply(fwd, side_in));
                bezier(apply(fwd, side_in), apply(fwd, add(side_in, scl(alpha * half, in_dir))),
                       apply(fwd, sub(side_out, scl(alpha * half, out_dir))), apply(fwd, side_out), -1.0f);
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
    vec2 ahead = scl(half, in_dir);
    vec2 side = perp(ahead);
    if (line_cap == butt) {
        lines.pts.push_back(apply(fwd, add(point, side)));
        lines.pts.push_back(apply(fwd, sub(point, side)));
    } else if (line_cap == square) {
        lines.pts.push_back(apply(fwd, add(add(point, ahead), side)));
        lines.pts.push_back(apply(fwd, sub(add(point, ahead), side)));
    } else if (line_cap == circle) {
        const float k = 0.55228475f;
        lines.pts.push_back(apply(fwd, add(point, side)));
        bezier(apply(fwd, add(point, side)), apply(fwd, add(add(point, side), scl(k, ahead))),
               apply(fwd, add(add(point, ahead), scl(k, side))), apply(fwd, add(point, ahead)), -1.0f);
        bezier(apply(fwd, add(point, ahead)), apply(fwd, sub(add(point, ahead), scl(k, side))),
               apply(fwd, add(sub(point, side), scl(k, ahead))), apply(fwd, sub(point, side)), -1.0f);
    }
}

void canvas::stroke_outline() {
    if (fwd.a * fwd.d - fwd.b * fwd.c == 0.0f) return;
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

// ---- scan conversion (hpp:2109-2253) ----
void canvas::scan_segment(vec2 from, vec2 to) {
    const float eps = 2.0e-5f;
    if (fabsf(to.y - from.y) < eps) return;
    float sign = to.y > from.y ? 1.0f : -1.0f;
    if (from.x > to.x) std::swap(from, to);
    vec2 now = from;
    vec2 pixel = mk(floorf(now.x), floorf(now.y));
    vec2 corner = add(pixel, mk(1.0f, to.y > from.y ? 1.0f : 0.0f));
    vec2 slope = mk((to.x - from.x) / (to.y - from.y), (to.y - from.y) / (to.x - from.x));
    vec2 nx = (to.x - from.x < eps) ? to : mk(corner.x, now.y + (corner.x - now.x) * slope.y);
    vec2 ny = mk(now.x + (corner.y - now.y) * slope.x, corner.y);
    if ((from.y < to.y && to.y < ny.y) || (from.y > to.y && to.y > ny.y)) ny = to;
    float ystep = to.y > from.y ? 1.0f : -1.0f;
    do {
        float carry = 0.0f;
        while (nx.x < ny.x) {
            float strip = lo(hi((nx.y - now.y) * ystep, 0.0f), 1.0f);
            float mid = (nx.x + now.x) * 0.5f;
            float area = (mid - pixel.x) * strip;
            run r = {static_cast<unsigned short>(pixel.x), static_cast<unsigned short>(pixel.y),
                     (carry + strip - area) * sign};
            runs.push_back(r);
            carry = area;
            now = nx;
            nx.x += 1.0f;
            nx.y = (nx.x - from.x) * slope.y + from.y;
            pixel.x += 1.0f;
        }
        float strip = lo(hi((ny.y - now.y) * ystep, 0.0f), 1.0f);
        float mid = (ny.x + now.x) * 0.5f;
        float area = (mid - pixel.x) * strip;
        run r1 = {static_cast<unsigned short>(pixel.x), static_cast<unsigned short>(pixel.y),
                  (carry + strip - area) * sign};
        run r2 = {static_cast<unsigned short>(pixel.x + 1.0f), static_cast<unsigned short>(pixel.y),
                  area * sign};
        runs.push_back(r1);
        runs.push_back(r2);
        now = ny;
        ny.y += ystep;
        ny.x = (ny.y - from.y) * slope.x + from.x;
        pixel.y += ystep;
        if ((from.y < to.y && to.y < ny.y) || (from.y > to.y && to.y > ny.y)) ny = to;
    } while (now.y != to.y);
}

void canvas::scan(vec2 offset, int padding) {
    runs.clear();
    float width = static_cast<float>(W + padding);
    float height = static_cast<float>(H + padding);
    size_t end = 0;
    for (size_t s = 0; s < lines.subs.size(); ++s) {
        size_t begin = end;
        end += lines.subs[s].count;
        scratch.pts.clear();
        for (size_t i = begin; i < end; ++i) scratch.pts.push_back(add(offset, lines.pts[i]));
        // Sutherland-Hodgman against x >= 0, y >= 0, x <= width, y <= height.
        for (int edge = 0; edge < 4; ++edge) {
            vec2 normal = mk(edge == 0 ? 1.0f : edge == 2 ? -1.0f : 0.0f,
                             edge == 1 ? 1.0f : edge == 3 ? -1.0f : 0.0f);
            float place = edge == 2 ? width : edge == 3 ? height : 0.0f;
            size_t first = scratch.pts.size();
            for (size_t i = 0; i < first; ++i) {
                vec2 from = scratch.pts[(i ? i : first) - 1];
                vec2 to = scratch.pts[i];
                float fs = dot(from, normal) + place;
                float ts = dot(to, normal) + place;
                if (fs * ts < 0.0f) scratch.pts.push_back(mix(from, to, fs / (fs - ts)));
                if (ts >= 0.0f) scratch.pts.push_back(to);
            }
            scratch.pts.erase(scratch.pts.begin(), scratch.pts.begin() + static_cast<ptrdiff_t>(first));
        }
        size_t last = scratch.pts.size();
        for (size_t i = 0; i < last; ++i) {
            vec2 from = scratch.pts[(i ? i : last) - 1];
            vec2 to = scratch.pts[i];
            scan_segment(mk(lo(hi(from.x, 0.0f), width), lo(hi(from.y, 0.0f), height)),
                         mk(lo(hi(to.x, 0.0f), width), lo(hi(to.y, 0.0f), height)));
        }
    }
    if (runs.empty()) return;
    std::sort(runs.begin(), runs.end(), run_before);
    size_t to = 0;
    for (size_t from = 1; from < runs.size(); ++from) {
        if (runs[from].x == runs[to].x && runs[from].y == runs[to].y) runs[to].delta += runs[from].delta;
        else if (runs[from].delta != 0.0f) runs[++to] = runs[from];
    }
    runs.erase(runs.begin() + static_cast<ptrdiff_t>(to) + 1, runs.end());
}

// ---- binned coverage (the library's sort-free variant, CYO_BINNED) ----
// The same cell walk as scan_segment (add_runs, hpp:2109-2170), but a row
// adds to a per-pixel 32-bit integer accumulation image: cell m adds
// round(C_m * 2^22) minus the same for the cell before, where C_m = sign *
// (S_m - area_m), S_m the row's vertical extent from its entry point to
// the cell's right crossing and area_m the cell's trapezoid; the cell past
// the exit adds what completes sign * S of the whole row.  Cells at x >= W or
// rows outside [0, H) are dropped.
static const float kAccScale = 4194304.0f;   // 2^22
static const float kAccInv = 1.0f / 4194304.0f;

void canvas::scan_segment_binned(vec2 from, vec2 to) {
    const float eps = 2.0e-5f;
    if (fabsf(to.y - from.y) < eps) return;
    float sign = to.y > from.y ? 1.0f : -1.0f;
    if (from.x > to.x) std::swap(from, to);
    vec2 now = from;
    vec2 pixel = mk(floorf(now.x), floorf(now.y));
    vec2 corner = add(pixel, mk(1.0f, to.y > from.y ? 1.0f : 0.0f));
    vec2 slope = mk((to.x - from.x) / (to.y - from.y), (to.y - from.y) / (to.x - from.x));
    vec2 nx = (to.x - from.x < eps) ? to : mk(corner.x, now.y + (corner.x - now.x) * slope.y);
    vec2 ny = mk(now.x + (corner.y - now.y) * slope.x, corner.y);
    if ((from.y < to.y && to.y < ny.y) || (from.y > to.y && to.y > ny.y)) ny = to;
    float ystep = to.y > from.y ? 1.0f : -1.0f;
    auto put = [&](float x, float y, int dq) {
        int ix = static_cast<int>(x), iy = static_cast<int>(y);
        if (dq != 0 && ix >= 0 && ix < W && iy >= 0 && iy < H)
            acc[static_cast<size_t>(iy) * W + ix] = static_cast<int32_t>(
                static_cast<uint32_t>(acc[static_cast<size_t>(iy) * W + ix]) + static_cast<uint32_t>(dq));
    };
    auto q_of = [&](vec2 entry, vec2 left, vec2 right, float px) {
        float strip = lo(hi((right.y - left.y) * ystep, 0.0f), 1.0f);
        float mid = (right.x + left.x) * 0.5f;
        float area = (mid - px) * strip;
        float S = lo(hi((right.y - entry.y) * ystep, 0.0f), 1.0f);
        return static_cast<int>(rintf((S - area) * sign * kAccScale));
    };
    do {
        const vec2 entry = now;
        int qprev = 0;
        while (nx.x < ny.x) {
            int q = q_of(entry, now, nx, pixel.x);
            put(pixel.x, pixel.y, q - qprev);
            qprev = q;
            now = nx;
            nx.x += 1.0f;
            nx.y = (nx.x - from.x) * slope.y + from.y;
            pixel.x += 1.0f;
        }
        int q = q_of(entry, now, ny, pixel.x);
        put(pixel.x, pixel.y, q - qprev);
        float S = lo(hi((ny.y - entry.y) * ystep, 0.0f), 1.0f);
        int q2 = static_cast<int>(rintf(S * sign * kAccScale));
        put(pixel.x + 1.0f, pixel.y, q2 - q);
        now = ny;
        ny.y += ystep;
        ny.x = (ny.y - from.y) * slope.x + from.x;
        pixel.y += ystep;
        if ((from.y < to.y && to.y < ny.y) || (from.y > to.y && to.y > ny.y)) ny = to;
    } while (now.y != to.y);
}

// Where u -> v crosses an edge, fs and ts the signed distances of u and v
// from it: the reference's u + t (v - u) (hpp:2220-2221), except when u lies
// 2^24 or more beyond the edge and v nearer, where that loses the crossing
// to cancellation (1e30 and 48 differ by nothing in float): then from v.
static inline vec2 crossing(vec2 u, vec2 v, float fs, float ts) {
    return std::fabs(fs) >= 16777216.0f && std::fabs(fs) > std::fabs(ts) ? mix(v, u, ts / (ts - fs))
                                                                         : mix(u, v, fs / (fs - ts));
}

// One polyline segment clipped to [0,width] x [0,height] on its own, as the
// binned coverage does it: the polygon clip of scan (hpp:2204-2239) followed
// by the clamp replaces the part of an edge left of x = 0 by its projection
// onto that side, and parts above y = 0 or below y = height become
// horizontal and add nothing; per segment the same pieces come out (inside,
// left side), each clamped.  The left piece lies on x = 0, so clamping its
// ends to [0, height] clips it exactly.  The part right of x = width is
// dropped: its projection onto that side adds only to cells at x >= width,
// which no pixel reads.  A segment with a non-finite end gives none.  In
// exact arithmetic the pieces of all segments add up to the clipped
// polygon's coverage; in float they differ from it by rounding only.
static int clip_segment(vec2 a, vec2 b, float width, float height, vec2 *pa, vec2 *pb) {
    if (!(std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(b.x) && std::isfinite(b.y))) return 0;
    vec2 ma = a, mb = b, la{}, lb{};
    bool has_main = true, has_left = false;
    {
        float fs = ma.x, ts = mb.x;
        if (fs < 0.0f && ts < 0.0f) {
            has_main = false;
            has_left = true;
            la = mk(0.0f, ma.y);
            lb = mk(0.0f, mb.y);
        } else if (fs * ts < 0.0f) {
            vec2 cut = crossing(ma, mb, fs, ts);
            has_left = true;
            if (fs < 0.0f) {
                la = mk(0.0f, ma.y);
                lb = mk(0.0f, cut.y);
                ma = cut;
            } else {
                la = mk(0.0f, cut.y);
                lb = mk(0.0f, mb.y);
                mb = cut;
            }
        }
    }
    auto keep_below = [](bool &has, vec2 &u, vec2 &v, float place, float dir) {
        // keep the part where dir * (y - place) >= 0
        if (!has) return;
        float fs = (u.y - place) * dir, ts = (v.y - place) * dir;
        if (fs < 0.0f && ts < 0.0f) {
            has = false;
            return;
        }
        if (fs * ts < 0.0f) {
            vec2 cut = crossing(u, v, fs, ts);
            if (fs < 0.0f) u = cut;
            else v = cut;
        }
    };
    keep_below(has_main, ma, mb, 0.0f, 1.0f);
    if (has_main) {
        float fs = width - ma.x, ts = width - mb.x;
        if (fs < 0.0f && ts < 0.0f) {
            has_main = false;
        } else if (fs * ts < 0.0f) {
            vec2 cut = crossing(ma, mb, fs, ts);
            if (fs < 0.0f) ma = cut;
            else mb = cut;
        }
    }
    keep_below(has_main, ma, mb, height, -1.0f);
    int n = 0;
    auto put = [&](vec2 u, vec2 v) {
        pa[n] = mk(lo(hi(u.x, 0.0f), width), lo(hi(u.y, 0.0f), height));
        pb[n] = mk(lo(hi(v.x, 0.0f), width), lo(hi(v.y, 0.0f), height));
        ++n;
    };
    if (has_main) put(ma, mb);
    if (has_left) put(la, lb);
    return n;
}

// scan() of the draw itself (no offset, no padding) into `acc`: each
// segment clipped on its own, then the binned cell walk of every piece.  A
// point with a non-finite coordinate is left out and its neighbours joined,
// as the polygon clip drops it (its comparisons fail for NaN, hpp:2218-2223):
// the segment ending at it is skipped, and the one leaving it starts from
// the nearest finite point before it.
void canvas::scan_binned() {
    acc.assign(static_cast<size_t>(W) * static_cast<size_t>(H), 0);
    float width = static_cast<float>(W), height = static_cast<float>(H);
    auto finite = [](vec2 p) { return std::isfinite(p.x) && std::isfinite(p.y); };
    size_t end = 0;
    for (size_t s = 0; s < lines.subs.size(); ++s) {
        size_t begin = end;
        end += lines.subs[s].count;
        size_t n = end - begin;
        for (size_t i = 0; i < n; ++i) {
            vec2 to = add(mk(0.0f, 0.0f), lines.pts[begin + i]);
            if (!finite(to)) continue;
            size_t j = (i ? i : n) - 1;
            while (!finite(lines.pts[begin + j]) && j != i) j = (j ? j : n) - 1;
            if (j == i) continue;
            vec2 from = add(mk(0.0f, 0.0f), lines.pts[begin + j]);
            vec2 pa[2], pb[2];
            int pieces = clip_segment(from, to, width, height, pa, pb);
            for (int k = 0; k < pieces; ++k) scan_segment_binned(pa[k], pb[k]);
        }
    }
}

// ---- paint (hpp:2265-2377) ----
static inline float keys_weight(float t) {
    return t < 1.0f ? (1.5f * t - 2.5f) * t * t + 1.0f : ((-0.5f * t + 2.5f) * t - 4.0f) * t + 2.0f;
}

col canvas::paint(vec2 p, const brush &br, bool clamp_edges) {
    if (br.colors.empty()) return mkc(0, 0, 0, 0);
    if (br.kind == brush::solid) return br.colors.front();
    p = apply(inv, p);
    if (br.kind == brush::image) {
        float width = static_cast<float>(br.w), height = static_cast<float>(br.h);
        if (((br.rep & 2) && (p.x < 0.0f || width <= p.x)) || ((br.rep & 1) && (p.y < 0.0f || height <= p.y)))
            return mkc(0, 0, 0, 0);
        float sx = fabsf(inv.a) + fabsf(inv.c);
        float sy = fabsf(inv.b) + fabsf(inv.d);
        sx = hi(1.0f, lo(sx, width * 0.25f));
        sy = hi(1.0f, lo(sy, height * 0.25f));
        float rx = 1.0f / sx, ry = 1.0f / sy;
        p = sub(p, mk(0.5f, 0.5f));
        int left = static_cast<int>(ceilf(p.x - sx * 2.0f));
        int topy = static_cast<int>(ceilf(p.y - sy * 2.0f));
        int right = static_cast<int>(ceilf(p.x + sx * 2.0f));
        int bot = static_cast<int>(ceilf(p.y + sy * 2.0f));
        col total = mkc(0, 0, 0, 0);
        float wsum = 0.0f;
        for (int py = topy; py < bot; ++py) {
            float wy = keys_weight(fabsf(ry * (static_cast<float>(py) - p.y)));
            int yy = py % br.h;
            if (yy < 0) yy += br.h;
            if (clamp_edges) yy = loi(hii(py, 0), br.h - 1);
            for (int px = left; px < right; ++px) {
                float wx = keys_weight(fabsf(rx * (static_cast<float>(px) - p.x)));
                int xx = px % br.w;
                if (xx < 0) xx += br.w;
                if (clamp_edges) xx = loi(hii(px, 0), br.w - 1);
                float wgt = wx * wy;
                total = cadd(total, cscl(wgt, br.colors[static_cast<size_t>(yy * br.w + xx)]));
                wsum += wgt;
            }
        }
        return cscl(1.0f / wsum, total);
    }
    float offset;
    vec2 rel = sub(p, br.p0);
    vec2 line = sub(br.p1, br.p0);
    float grad = dot(rel, line);
    float span = dot(line, line);
    if (br.kind == brush::linear) {
        if (span == 0.0f) return mkc(0, 0, 0, 0);
        offset = grad / span;
    } else {
        float initial = br.r0;
        float change = br.r1 - initial;
        float a = span - change * change;
        float b = -2.0f * (grad + initial * change);
        float c = dot(rel, rel) - initial * initial;
        float disc = b * b - 4.0f * a * c;
        if (disc < 0.0f || (span == 0.0f && change == 0.0f)) return mkc(0, 0, 0, 0);
        float root = sqrtf(disc);
        float recip = 1.0f / (2.0f * a);
        float o1 = (-b - root) * recip;
        float o2 = (-b + root) * recip;
        float rad1 = initial + change * o1;
        float rad2 = initial + change * o2;
        if (rad2 >= 0.0f) offset = o2;
        else if (rad1 >= 0.0f) offset = o1;
        else return mkc(0, 0, 0, 0);
    }
    size_t k = static_cast<size_t>(std::upper_bound(br.stops.begin(), br.stops.end(), offset) - br.stops.begin());
    if (k == 0) return premul(br.colors.front());
    if (k == br.stops.size()) return premul(br.colors.back());
    float t = (offset - br.stops[k - 1]) / (br.stops[k] - br.stops[k - 1]);
    col delta = csub(br.colors[k], br.colors[k - 1]);
    return premul(cadd(br.colors[k - 1], cscl(t, delta)));
}

// One Porter-Duff style blend of `fore` into `back` (hpp:2522-2533, 2583-2591).
static inline void blend_into(col &back, col fore, int op, float visibility) {
    float mf = op & 1 ? back.a : 0.0f;
    if (op & 2) mf = 1.0f - mf;
    float mb = op & 4 ? fore.a : 0.0f;
    if (op & 8) mb = 1.0f - mb;
    col b = cadd(cscl(mf, fore), cscl(mb, back));
    b.a = lo(b.a, 1.0f);
    back = cadd(cscl(visibility, b), cscl(1.0f - visibility, back));
}

// ---- shadow (hpp:2395-2539) ----
void canvas::render_shadow(const brush &br, bool clamp_edges) {
    if (sh_color.a == 0.0f || (sh_blur == 0.0f && shadow_offset_x == 0.0f && shadow_offset_y == 0.0f)) return;
    float sigma2 = 0.25f * sh_blur * sh_blur;
    size_t radius = static_cast<size_t>(0.5f * sqrtf(4.0f * sigma2 + 1.0f) - 0.5f);
    int border = 3 * (static_cast<int>(radius) + 1);
    vec2 offset = mk(static_cast<float>(border) + shadow_offset_x, static_cast<float>(border) + shadow_offset_y);
    scan(offset, 2 * border);
    int left = W + 2 * border, right = 0, topy = H + 2 * border, bot = 0;
    for (size_t i = 0; i < runs.size(); ++i) {
        left = loi(left, static_cast<int>(runs[i].x));
        right = hii(right, static_cast<int>(runs[i].x));
        topy = loi(topy, static_cast<int>(runs[i].y));
        bot = hii(bot, static_cast<int>(runs[i].y));
    }
    left = hii(left - border, 0);
    right = loi(right + border, W + 2 * border) + 1;
    topy = hii(topy - border, 0);
    bot = loi(bot + border, H + 2 * border);
    size_t width = static_cast<size_t>(hii(right - left, 0));
    size_t height = static_cast<size_t>(hii(bot - topy, 0));
    size_t working = width * height;
    shadow.clear();
    shadow.resize(working + std::max(width, height));
    {
        int x = -1, y = -1;
        float sum = 0.0f;
        for (size_t i = 0; i < runs.size(); ++i) {
            run next = runs[i];
            float coverage = cover(sum);
            int to = next.y == y ? next.x : x + 1;
            if (coverage >= kVisible)
                for (; x < to; ++x)
                    shadow[static_cast<size_t>(y - topy) * width + static_cast<size_t>(x - left)] =
                        coverage * paint(sub(mk(static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f), offset),
                                         br, clamp_edges).a;
            if (next.y != y) sum = 0.0f;
            x = next.x;
            y = next.y;
            sum += next.delta;
        }
    }
    float alpha = static_cast<float>(2 * radius + 1) *
                  (static_cast<float>(radius * (radius + 1)) - sigma2) /
                  (2.0f * sigma2 - static_cast<float>(6 * (radius + 1) * (radius + 1)));
    float divisor = 2.0f * (alpha + static_cast<float>(radius)) + 1.0f;
    float w1 = alpha / divisor;
    float w2 = (1.0f - alpha) / divisor;
    for (size_t y = 0; y < height; ++y)
        for (int pass = 0; pass < 3; ++pass) {
            for (size_t x = 0; x < width; ++x) shadow[working + x] = shadow[y * width + x];
            float acc = w1 * shadow[working + radius + 1];
            for (size_t x = 0; x <= radius; ++x) acc += (w1 + w2) * shadow[working + x];
            shadow[y * width] = acc;
            for (size_t x = 1; x < width; ++x) {
                if (x >= radius + 1) acc -= w2 * shadow[working + x - radius - 1];
                if (x >= radius + 2) acc -= w1 * shadow[working + x - radius - 2];
                if (x + radius < width) acc += w2 * shadow[working + x + radius];
                if (x + radius + 1 < width) acc += w1 * shadow[working + x + radius + 1];
                shadow[y * width + x] = acc;
            }
        }
    for (size_t x = 0; x < width; ++x)
        for (int pass = 0; pass < 3; ++pass) {
            for (size_t y = 0; y < height; ++y) shadow[working + y] = shadow[y * width + x];
            float acc = w1 * shadow[working + radius + 1];
            for (size_t y = 0; y <= radius; ++y) acc += (w1 + w2) * shadow[working + y];
            shadow[x] = acc;
            for (size_t y = 1; y < height; ++y) {
                if (y >= radius + 1) acc -= w2 * shadow[working + y - radius - 1];
                if (y >= radius + 2) acc -= w1 * shadow[working + y - radius - 2];
                if (y + radius < height) acc += w2 * shadow[working + y + radius];
                if (y + radius + 1 < height) acc += w1 * shadow[working + y + radius + 1];
                shadow[y * width + x] = acc;
            }
        }
    int op = global_composite_operation;
    int x = -1, y = -1;
    float sum = 0.0f;
    for (size_t i = 0; i < mask.size(); ++i) {
        run next = mask[i];
        float vis = lo(fabsf(sum), 1.0f);
        int to = loi(next.y == y ? next.x : x + 1, right - border);
        if (vis >= kVisible && topy <= y + border && y + border < bot)
            for (; x < to; ++x) {
                col &back = bitmap[static_cast<size_t>(y * W + x)];
                col fore = cscl(g_alpha * shadow[static_cast<size_t>(y + border - topy) * width +
                                                 static_cast<size_t>(x + border - left)],
                                sh_color);
                blend_into(back, fore, op, vis);
            }
        if (next.y != y) sum = 0.0f;
        x = hii(static_cast<int>(next.x), left - border);
        y = next.y;
        sum += next.delta;
    }
}

// ---- main render (hpp:2551-2605) ----
void canvas::render(const brush &br, bool clamp_edges) {
    if (fwd.a * fwd.d - fwd.b * fwd.c == 0.0f) return;
    render_shadow(br, clamp_edges);
#ifdef CYO_BINNED
    // Every pixel the reference's walk visits gets the coverage of the
    // row's accumulated area up to it and the clip visibility of the walk:
    // min(|mask sum|, 1) from the row's first to its last mask run, else 0.
    {
        scan_binned();
        int op = global_composite_operation;
        std::vector<float> vis(static_cast<size_t>(W));
        size_t ci = 0;
        for (int y = 0; y < H; ++y) {
            std::fill(vis.begin(), vis.end(), 0.0f);
            while (ci < mask.size() && mask[ci].y < y) ++ci;
            size_t c0 = ci;
            while (ci < mask.size() && mask[ci].y == y) ++ci;
            if (ci > c0) {
                float csum = 0.0f;
                for (size_t k = c0; k < ci; ++k) {
                    csum += mask[k].delta;
                    int xa = mask[k].x, xb = k + 1 < ci ? mask[k + 1].x : mask[k].x + 1;
                    float v = lo(fabsf(csum), 1.0f);
                    for (int x = xa; x < xb && x < W; ++x) vis[static_cast<size_t>(x)] = v;
                }
            }
            uint32_t s = 0;
            for (int x = 0; x < W; ++x) {
                s += static_cast<uint32_t>(acc[static_cast<size_t>(y) * W + x]);
                float coverage = cover(static_cast<float>(static_cast<int32_t>(s)) * kAccInv);
                float v = vis[static_cast<size_t>(x)];
                if ((coverage >= kVisible || ~op & 8) && v >= kVisible) {
                    col &back = bitmap[static_cast<size_t>(y * W + x)];
                    col fore = cscl(coverage * g_alpha, paint(mk(static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f),
                                                             br, clamp_edges));
                    blend_into(back, fore, op, v);
                }
            }
        }
        return;
    }
#endif
    scan(mk(0.0f, 0.0f), 0);
    int op = global_composite_operation;
    int x = -1, y = -1;
    float psum = 0.0f, csum = 0.0f;
    size_t pi = 0, ci = 0;
    while (ci < mask.size()) {
        bool from_path = pi < runs.size() && run_before(runs[pi], mask[ci]);
        run next = from_path ? runs[pi] : mask[ci];
        float coverage = cover(psum);
        float vis = lo(fabsf(csum), 1.0f);
        int to = next.y == y ? next.x : x + 1;
        if ((coverage >= kVisible || ~op & 8) && vis >= kVisible)
            for (; x < to; ++x) {
                col &back = bitmap[static_cast<size_t>(y * W + x)];
                col fore = cscl(coverage * g_alpha,
                                paint(mk(static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f), br, clamp_edges));
                blend_into(back, fore, op, vis);
            }
        x = next.x;
        if (next.y != y) {
            y = next.y;
            psum = 0.0f;
            csum = 0.0f;
        }
        if (from_path) psum += runs[pi++].delta;
        else csum += mask[ci++].delta;
    }
}

// ---- clip (hpp:3057-3099) ----
void canvas::clip() {
    flatten(false);
    scan(mk(0.0f, 0.0f), 0);
    cur_rule = fill_rule;
    size_t part = runs.size();
    runs.insert(runs.end(), mask.begin(), mask.end());
    mask.clear();
    int y = -1;
    float last = 0.0f, s1 = 0.0f, s2 = 0.0f;
    size_t i1 = 0, i2 = part;
    while (i1 < part && i2 < runs.size()) {
        bool first = run_before(runs[i1], runs[i2]);
        run next = first ? runs[i1] : runs[i2];
        if (next.y != y) {
            y = next.y;
            last = 0.0f;
            s1 = 0.0f;
            s2 = 0.0f;
        }
        if (first) s1 += runs[i1++].delta;
        else s2 += runs[i2++].delta;
        float vis = cover(s1) * lo(fabsf(s2), 1.0f);
        if (vis == last) continue;
        if (!mask.empty() && mask.back().x == next.x && mask.back().y == next.y) {
            mask.back().delta += vis - last;
        } else {
            run r = {next.x, next.y, vis - last};
            mask.push_back(r);
        }
        last = vis;
    }
    cur_rule = 0;
}

// ---- hit test (hpp:3101-3132) ----
bool canvas::is_point_in_path(float x, float y) {
    flatten(false);
    int winding = 0;
    size_t s = 0, begin = 0, end = 0;
    for (size_t i = 0; i < lines.pts.size(); ++i) {
        while (i >= end) {
            begin = end;
            end += lines.subs[s++].count;
        }
        vec2 from = lines.pts[i];
        vec2 to = lines.pts[i + 1 < end ? i + 1 : begin];
        if ((from.y < y && y <= to.y) || (to.y < y && y <= from.y)) {
            float side = dot(perp(sub(to, from)), sub(mk(x, y), from));
            if (side == 0.0f) return true;
            winding += side > 0.0f ? 1 : -1;
        } else if (from.y == y && y == to.y && ((from.x <= x && x <= to.x) || (to.x <= x && x <= from.x))) {
            return true;
        }
    }
    return fill_rule ? (winding & 2) != 0 : winding != 0;   // each crossing edge counts +-1 on each side: twice the winding number
}

// ---- rectangles and images (hpp:3134-3346) ----
void canvas::clear_rectangle(float x, float y, float w, float h) {
    composite_operation sop = global_composite_operation;
    float sa = g_alpha, ssa = sh_color.a;
    brush::kind_t skind = fill_br.kind;
    global_composite_operation = destination_out;
    g_alpha = 1.0f;
    sh_color.a = 0.0f;
    fill_br.kind = brush::solid;
    fill_rectangle(x, y, w, h);
    fill_br.kind = skind;
    sh_color.a = ssa;
    g_alpha = sa;
    global_composite_operation = sop;
}
void canvas::fill_rectangle(float x, float y, float w, float h) {
    if (w == 0.0f || h == 0.0f) return;
    lines.pts.clear();
    lines.subs.clear();
    lines.pts.push_back(apply(fwd, mk(x, y)));
    lines.pts.push_back(apply(fwd, mk(x + w, y)));
    lines.pts.push_back(apply(fwd, mk(x + w, y + h)));
    lines.pts.push_back(apply(fwd, mk(x, y + h)));
    subpath e = {4, true};
    lines.subs.push_back(e);
    render(fill_br, false);
}
void canvas::stroke_rectangle(float x, float y, float w, float h) {
    if (w == 0.0f && h == 0.0f) return;
    lines.pts.clear();
    lines.subs.clear();
    if (w == 0.0f || h == 0.0f) {
        lines.pts.push_back(apply(fwd, mk(x, y)));
        lines.pts.push_back(apply(fwd, mk(x + w, y + h)));
        subpath e = {2, false};
        lines.subs.push_back(e);
    } else {
        lines.pts.push_back(apply(fwd, mk(x, y)));
        lines.pts.push_back(apply(fwd, mk(x + w, y)));
        lines.pts.push_back(apply(fwd, mk(x + w, y + h)));
        lines.pts.push_back(apply(fwd, mk(x, y + h)));
        lines.pts.push_back(apply(fwd, mk(x, y)));
        subpath e = {5, true};
        lines.subs.push_back(e);
    }
    stroke_outline();
    render(stroke_br, false);
}
void canvas::draw_image(const unsigned char *img, int w, int h, int stride, float x, float y, float tw, float th) {
    if (!img || w <= 0 || h <= 0 || tw == 0.0f || th == 0.0f) return;
    std::swap(fill_br, image_br);
    set_pattern(fill_style, img, w, h, stride, repeat);
    std::swap(fill_br, image_br);
    lines.pts.clear();
    lines.subs.clear();
    lines.pts.push_back(apply(fwd, mk(x, y)));
    lines.pts.push_back(apply(fwd, mk(x + tw, y)));
    lines.pts.push_back(apply(fwd, mk(x + tw, y + th)));
    lines.pts.push_back(apply(fwd, mk(x, y + th)));
    subpath e = {4, true};
    lines.subs.push_back(e);
    mat sf = fwd, si = inv;
    translate(x + lo(0.0f, tw), y + lo(0.0f, th));
    scale(fabsf(tw) / static_cast<float>(w), fabsf(th) / static_cast<float>(h));
    render(image_br, true);
    fwd = sf;
    inv = si;
}

// ---- pixel I/O (hpp:3348-3408) ----
void canvas::get_image_data(unsigned char *img, int w, int h, int stride, int x, int y) {
    if (!img) return;
    static const float bayer[4][4] = {
        {0.03125f, 0.53125f, 0.15625f, 0.65625f},
        {0.78125f, 0.28125f, 0.90625f, 0.40625f},
        {0.21875f, 0.71875f, 0.09375f, 0.59375f},
        {0.96875f, 0.46875f, 0.84375f, 0.34375f}};
    for (int iy = 0; iy < h; ++iy)
        for (int ix = 0; ix < w; ++ix) {
            int i = iy * stride + ix * 4;
            int cx = x + ix, cy = y + iy;
            col c = mkc(0, 0, 0, 0);
            if (0 <= cx && cx < W && 0 <= cy && cy < H) c = bitmap[static_cast<size_t>(cy * W + cx)];
            float t = bayer[cy & 3][cx & 3];
            c = cadd(mkc(t, t, t, t), cscl(255.0f, to_srgb(clamp01(unpremul(c)))));
            img[i + 0] = static_cast<unsigned char>(c.r);
            img[i + 1] = static_cast<unsigned char>(c.g);
            img[i + 2] = static_cast<unsigned char>(c.b);
            img[i + 3] = static_cast<unsigned char>(c.a);
        }
}
void canvas::put_image_data(const unsigned char *img, int w, int h, int stride, int x, int y) {
    if (!img) return;
    for (int iy = 0; iy < h; ++iy)
        for (int ix = 0; ix < w; ++ix) {
            int i = iy * stride + ix * 4;
            int cx = x + ix, cy = y + iy;
            if (cx < 0 || W <= cx || cy < 0 || H <= cy) continue;
            col c = mkc(img[i + 0] / 255.0f, img[i + 1] / 255.0f, img[i + 2] / 255.0f, img[i + 3] / 255.0f);
            bitmap[static_cast<size_t>(cy * W + cx)] = premul(to_linear(c));
        }
}

// ---- state stack (hpp:3410-3465) ----
void canvas::save() {
    state s;
    s.op = global_composite_operation; s.sox = shadow_offset_x; s.soy = shadow_offset_y;
    s.cap = line_cap; s.join = line_join; s.dash_off = line_dash_offset;
    s.align = text_align; s.baseline = text_baseline; s.fwd = fwd; s.inv = inv;
    s.alpha = g_alpha; s.shcol = sh_color; s.shblur = sh_blur; s.lw = lw; s.miter = miter_lim;
    s.dash = dash; s.fill = fill_br; s.stroke = stroke_br; s.mask = mask; s.face = face;
    stack.push_back(s);
}
void canvas::restore() {
    if (stack.empty()) return;
    state &s = stack.back();
    global_composite_operation = s.op; shadow_offset_x = s.sox; shadow_offset_y = s.soy;
    line_cap = s.cap; line_join = s.join; line_dash_offset = s.dash_off;
    text_align = s.align; text_baseline = s.baseline; fwd = s.fwd; inv = s.inv;
    g_alpha = s.alpha; sh_color = s.shcol; sh_blur = s.shblur; lw = s.lw; miter_lim = s.miter;
    dash.swap(s.dash); fill_br = s.fill; stroke_br = s.stroke; mask.swap(s.mask); face = s.face;
    stack.pop_back();
}

struct traits {
    typedef canvas canvas_type;
    typedef cyo::brush_type brush_type;
    typedef cyo::composite_operation composite_operation;
    typedef cyo::cap_style cap_style;
    typedef cyo::join_style join_style;
    typedef cyo::repetition_style repetition_style;
    typedef cyo::align_style align_style;
    typedef cyo::baseline_style baseline_style;
    static std::unique_ptr<canvas> make(int w, int h) { return std::unique_ptr<canvas>(new canvas(w, h)); }
    static bool set_fill_rule(canvas &c, int rule) {
        if (rule != 0 && rule != 1) return false;
        c.fill_rule = rule;
        return true;
    }
};

}  // namespace cyo

extern "C" {

// Replay a recorded call list through the oracle (see include/cy_replay.hpp).
int cyo_replay(const void *trace, size_t trace_len, void *images, size_t images_cap, size_t *images_len,
               float *results, int results_cap, int *results_len) {
    return cy_trace::replay_to_buffers<cyo::traits>(trace, trace_len, images, images_cap, images_len,
                                                     results, results_cap, results_len);
}

}

extern "C" int cyo_replay_linear(const void *trace, size_t trace_len, float *out, size_t out_floats, int *width,
                                 int *height) {
    cy_trace::output sink;
    std::unique_ptr<cyo::canvas> keep;
    int rc = cy_trace::replay<cyo::traits>(static_cast<const uint8_t *>(trace), trace_len, sink, &keep);
    if (rc != 0 || !keep) return rc ? rc : -1;
    const std::vector<cyo::col> &px = keep->pixels();
    int w = 0, h = 0;
    std::memcpy(&w, static_cast<const uint8_t *>(trace) + 12, 4);
    std::memcpy(&h, static_cast<const uint8_t *>(trace) + 16, 4);
    if (width) *width = w;
    if (height) *height = h;
    if (px.size() * 4 > out_floats) return -2;
    std::memcpy(out, px.data(), px.size() * sizeof(cyo::col));
    return 0;
}
