// device.cuh -- device-side restatement of the reference's per-pixel math.
//
// Everything here is compiled with --fmad=false and IEEE division/sqrt so
// that each float operation rounds exactly like the reference's x86-64 SSE
// code (no fused multiply-add).  hpp = src/canvas_ity.hpp.
#ifndef CY_DEVICE_CUH
#define CY_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine_types.h"

namespace cyg {

// std::min / std::max semantics (first argument wins ties and NaN cases).
__device__ __forceinline__ float lo(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float hi(float a, float b) { return a < b ? b : a; }

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 scl2(float s, float2 a) { return f2(a.x * s, a.y * s); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float2 perp2(float2 a) { return f2(-a.y, a.x); }
__device__ __forceinline__ float2 mix2(float2 a, float2 b, float t) { return add2(a, scl2(t, sub2(b, a))); }

static constexpr float kVisible = 1.0f / 8160.0f;   // hpp:2433, 2571
static constexpr float kFixedOne = 4294967296.0f;   // coverage fixed point: 2^32
static constexpr float kFixedInv = 1.0f / 4294967296.0f;

// ------------------------------------------------------------ flattening
// Flattening of one cubic, hpp:1331-1387 (add_tessellation) and
// hpp:1398-1487 (add_bezier).  angular = -1 is fill mode (end points only);
// stroking passes the cosine limit of hpp:1499-1500 and also keeps the
// control points of the flat pieces.  The recursion becomes an explicit
// depth-first stack; EMIT=false only counts the points.
struct tess_frame { float2 p1, c1, c2, p2; int limit; };

template <bool EMIT>
__device__ int tessellate(float2 p1, float2 c1, float2 c2, float2 p2, float angular, float2 *out, int cap) {
    const float flat = 0.125f * 0.125f;
    const bool stroking = angular > -1.0f;
    tess_frame stack[22];
    int depth = 0, n = 0;
    // the whole curve is the first frame, held in registers: a curve that
    // is flat at once (most join and cap arcs) never touches the stack
    tess_frame f = {p1, c1, c2, p2, 20};
    for (;;) {
        for (;;) {
            float2 seg = sub2(f.p2, f.p1);
            float2 e1 = sub2(f.c1, f.p1), e3 = sub2(f.p2, f.c2);
            float lsq = hi(1.0e-4f, dot2(seg, seg));
            float t1 = lo(hi(dot2(e1, seg) / lsq, 0.0f), 1.0f);
            float t2 = lo(hi(dot2(e3, seg) / lsq, 0.0f), 1.0f);
            float2 d1 = sub2(add2(f.p1, scl2(t1, seg)), f.c1);
            float2 d2 = sub2(sub2(f.p2, scl2(t2, seg)), f.c2);
            float q1 = 0.0f, q2 = 0.0f, q3 = 0.0f, cosine = 1.0f;
            if (stroking) {
                float2 e2 = sub2(f.c2, f.c1);
                q1 = dot2(e1, e1);
                q2 = dot2(e2, e2);
                q3 = dot2(e3, e3);
                if (q1 * q3 != 0.0f) cosine = dot2(e1, e3) / sqrtf(q1 * q3);
                else if (q1 * q2 != 0.0f) cosine = dot2(e1, e2) / sqrtf(q1 * q2);
                else if (q2 * q3 != 0.0f) cosine = dot2(e2, e3) / sqrtf(q2 * q3);
            }
            if ((dot2(d1, d1) <= flat && dot2(d2, d2) <= flat && cosine >= angular) || !f.limit) {
                if (stroking && q1 != 0.0f) {
                    if (EMIT && n < cap) out[n] = f.c1;
                    ++n;
                }
                if (stroking && q2 != 0.0f) {
                    if (EMIT && n < cap) out[n] = f.c2;
                    ++n;
                }
                if (!stroking || q3 != 0.0f) {
                    if (EMIT && n < cap) out[n] = f.p2;
                    ++n;
                }
                break;
            }
            float2 l1 = mix2(f.p1, f.c1, 0.5f), m = mix2(f.c1, f.c2, 0.5f), r2 = mix2(f.c2, f.p2, 0.5f);
            float2 l2 = mix2(l1, m, 0.5f), r1 = mix2(m, r2, 0.5f), sp = mix2(l2, r1, 0.5f);
            stack[depth++] = {sp, r1, r2, f.p2, f.limit - 1};
            f = {f.p1, l1, l2, sp, f.limit - 1};
        }
        if (depth == 0) break;
        f = stack[--depth];
    }
    return n;
}

__device__ __forceinline__ void axis_extrema(float a, float b, float c, float *at, int &cuts) {
    const float eps = 1.0e-4f;   // hpp:1420-1447
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

template <bool EMIT>
__device__ int flatten_cubic(float2 p1, float2 c1, float2 c2, float2 p2, float angular, float2 *out, int cap) {
    float2 e1 = sub2(c1, p1), e2 = sub2(c2, c1), e3 = sub2(p2, c2);
    if (dot2(e1, e1) == 0.0f && dot2(e3, e3) == 0.0f) {
        if (EMIT && cap > 0) out[0] = p2;
        return 1;
    }
    float at[7] = {0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int cuts = 2;
    float2 ea = add2(scl2(-9.0f, e2), scl2(3.0f, sub2(p2, p1)));
    float2 eb = sub2(scl2(6.0f, add2(p1, c2)), scl2(12.0f, c1));
    float2 ec = scl2(3.0f, e1);
    axis_extrema(ea.x, eb.x, ec.x, at, cuts);
    axis_extrema(ea.y, eb.y, ec.y, at, cuts);
    float k1 = dot2(perp2(e1), e2), k2 = dot2(perp2(e1), e3), k3 = dot2(perp2(e2), e3);
    float ca = k1 - k2 + k3, cb = -2.0f * k1 + k2;
    if (fabsf(ca) > 1.0e-4f && fabsf(cb) > 1.0e-4f) at[cuts++] = -0.5f * cb / ca;
    for (int i = 1; i < cuts; ++i) {   // insertion sort, hpp:1458-1465
        float v = at[i];
        int j = i - 1;
        for (; 0 <= j && v < at[j]; --j) at[j + 1] = at[j];
        at[j + 1] = v;
    }
    int n = 0;
    float2 s1 = p1;
    for (int i = 0; i < cuts - 1; ++i) {
        if (!(0.0f <= at[i] && at[i + 1] <= 1.0f && at[i] != at[i + 1])) continue;
        float t = at[i + 1], ratio = at[i] / t;
        float2 q1 = mix2(p1, c1, t), q2 = mix2(c1, c2, t), q3 = mix2(c2, p2, t);
        float2 q4 = mix2(q1, q2, t), q5 = mix2(q2, q3, t), q6 = mix2(q1, q4, ratio);
        float2 s2 = mix2(q4, q5, t);
        float2 sc2 = mix2(q4, s2, ratio);
        float2 sc1 = mix2(q6, sc2, ratio);
        n += tessellate<EMIT>(s1, sc1, sc2, s2, angular, out + (EMIT ? n : 0), cap - n);
        s1 = s2;
    }
    return n;
}

// ------------------------------------------------------ scan conversion
// A segment piece inside the (padded) canvas, prepared for the row-by-row
// restatement of add_runs (hpp:2109-2170).  The reference walks the pixel
// cells of a segment left to right with a DDA; each row of that walk only
// depends on values the reference computes directly from the segment
// (crossing points at integer x and integer y), so any row can be
// reconstructed independently and rows can be processed in parallel with
// results identical to the sequential walk.
struct dda_piece {
    float fx, fy, tx, ty;   // endpoints ordered by x (from.x <= to.x)
    float sx, sy;           // slope.x = dx/dy, slope.y = dy/dx
    float sign, ystep;
    float px0, py0;         // floor(from)
    bool up, vert;
    int nrows;
};

__device__ __forceinline__ bool dda_setup(float2 a, float2 b, dda_piece &p) {
    if (!(fabsf(b.y - a.y) >= 2.0e-5f)) return false;   // hpp:2113-2115 (NaN-safe)
    p.sign = b.y > a.y ? 1.0f : -1.0f;
    if (a.x > b.x) { float2 t = a; a = b; b = t; }
    p.fx = a.x; p.fy = a.y; p.tx = b.x; p.ty = b.y;
    p.up = b.y > a.y;
    p.px0 = floorf(a.x);
    p.py0 = floorf(a.y);
    p.sx = (b.x - a.x) / (b.y - a.y);
    p.sy = (b.y - a.y) / (b.x - a.x);
    p.vert = b.x - a.x < 2.0e-5f;
    p.ystep = p.up ? 1.0f : -1.0f;
    int last = p.up ? static_cast<int>(ceilf(b.y)) - static_cast<int>(p.py0) - 1
                    : static_cast<int>(p.py0) - static_cast<int>(floorf(b.y));
    p.nrows = (last < 0 ? 0 : last) + 1;
    return true;
}

// Exit point of row k (the reference's next_y for that row).
__device__ __forceinline__ float2 dda_exit(const dda_piece &p, int k) {
    float corner = p.py0 + (p.up ? 1.0f : 0.0f) + static_cast<float>(k) * p.ystep;
    bool reached = p.up ? (p.ty < corner) : (p.ty > corner);
    if (reached) return f2(p.tx, p.ty);
    return f2((corner - p.fy) * p.sx + p.fx, corner);
}

// Number of lattice crossings x = px0 + m (m >= 1) strictly left of e.
__device__ __forceinline__ int crossings_before(const dda_piece &p, float e) {
    int c = static_cast<int>(ceilf(e)) - 1 - static_cast<int>(p.px0);
    return c < 0 ? 0 : c;
}

// Cell range of row k: the reference's pixel.x at the start of the row (ps)
// and at its end (pe); the row emits cells ps..pe+1.  `entry` is the row's
// entry point (the previous row's exit), `ex` its exit point.
__device__ __forceinline__ void dda_span(const dda_piece &p, int k, float2 entry, float2 ex, int &ps, int &pe) {
    if (!p.vert) {
        int before = k == 0 ? 0 : crossings_before(p, entry.x);
        int upto = crossings_before(p, ex.x);
        ps = static_cast<int>(p.px0) + before;
        pe = static_cast<int>(p.px0) + (upto > before ? upto : before);
    } else {
        bool consumed_before = k > 0 && p.tx < entry.x;
        bool consumed_now = !consumed_before && p.tx < ex.x;
        ps = static_cast<int>(p.px0) + (consumed_before ? 1 : 0);
        pe = ps + (consumed_now ? 1 : 0);
    }
}

__device__ __forceinline__ int dda_row_index(const dda_piece &p, int k) {
    return static_cast<int>(p.py0) + (p.up ? k : -k);
}

// Emit the signed-area deltas of row k (cells ps..pe+1, in order) through
// `emit(x, d)`: the body of add_runs' row loop (hpp:2131-2169).
template <class Emit>
__device__ __forceinline__ void dda_cells(const dda_piece &p, float2 entry, float2 ex, int ps, int pe, Emit &emit) {
    float2 now = entry;
    float carry = 0.0f;
    for (int m = ps; m < pe; ++m) {
        float2 X;
        if (!p.vert) {
            float cx = static_cast<float>(m + 1);
            X = f2(cx, (cx - p.fx) * p.sy + p.fy);
        } else {
            X = f2(p.tx, p.ty);
        }
        float strip = lo(hi((X.y - now.y) * p.ystep, 0.0f), 1.0f);
        float mid = (X.x + now.x) * 0.5f;
        float area = (mid - static_cast<float>(m)) * strip;
        emit(m, (carry + strip - area) * p.sign);
        carry = area;
        now = X;
    }
    float strip = lo(hi((ex.y - now.y) * p.ystep, 0.0f), 1.0f);
    float mid = (ex.x + now.x) * 0.5f;
    float area = (mid - static_cast<float>(pe)) * strip;
    emit(pe, (carry + strip - area) * p.sign);
    emit(pe + 1, area * p.sign);
}

// Emit row k of the piece through `emit(x, y, d)` (used by host-side checks).
template <class Emit>
__device__ __forceinline__ void dda_row(const dda_piece &p, int k, Emit &emit) {
    float2 entry = k == 0 ? f2(p.fx, p.fy) : dda_exit(p, k - 1);
    float2 ex = dda_exit(p, k);
    int ps, pe;
    dda_span(p, k, entry, ex, ps, pe);
    int row = dda_row_index(p, k);
    auto e2 = [&](int x, float d) { emit(x, row, d); };
    dda_cells(p, entry, ex, ps, pe, e2);
}

// Where u -> v crosses an edge, fs and ts the signed distances of u and v
// from it: the reference's u + t (v - u) (hpp:2220-2221), except when u lies
// 2^24 or more beyond the edge and v nearer, where that loses the crossing
// to cancellation (1e30 and 48 differ by nothing in float): then from v.
__device__ __forceinline__ float2 crossing2(float2 u, float2 v, float fs, float ts) {
    return fabsf(fs) >= 16777216.0f && fabsf(fs) > fabsf(ts) ? mix2(v, u, ts / (ts - fs))
                                                             : mix2(u, v, fs / (fs - ts));
}

// Clip one polyline segment to [0,width] x [0,height] the way the
// reference's Sutherland-Hodgman pass and clamp do (hpp:2204-2239), summed
// over a polygon (far-off ends aside, crossing2): the part left of x = 0 is
// replaced by its projection onto that edge, clamped to [0, height]; parts
// above y = 0 or below y = height contribute nothing, and so does the part
// right of x = width, whose projection onto that edge adds only to cells at
// x >= width, which no pixel reads.  Up to two pieces in fixed slots (0
// inside, 1 the left edge, each clamped); returns the mask of the slots
// filled, none for a segment with a non-finite end.
__device__ __forceinline__ unsigned clip_segment(float2 a, float2 b, float width, float height, float2 (&pa)[2],
                                                 float2 (&pb)[2]) {
    if (!(isfinite(a.x) && isfinite(a.y) && isfinite(b.x) && isfinite(b.y))) return 0u;
    float2 ma = a, mb = b, la = a, lb = b;
    bool has_main = true, has_left = false;
    // x >= 0
    {
        float fs = ma.x, ts = mb.x;
        if (fs < 0.0f && ts < 0.0f) {
            has_main = false;
            has_left = true;
            la = f2(0.0f, ma.y);
            lb = f2(0.0f, mb.y);
        } else if (fs * ts < 0.0f) {
            float2 I = crossing2(ma, mb, fs, ts);
            has_left = true;
            if (fs < 0.0f) { la = f2(0.0f, ma.y); lb = f2(0.0f, I.y); ma = I; }
            else { la = f2(0.0f, I.y); lb = f2(0.0f, mb.y); mb = I; }
        }
    }
    // keep where dir * (y - place) >= 0; the rest lies on a horizontal edge
    auto keep_y = [](bool &has, float2 &u, float2 &v, float fs, float ts) {
        if (!has) return;
        if (fs < 0.0f && ts < 0.0f) { has = false; return; }
        if (fs * ts < 0.0f) {
            float2 I = crossing2(u, v, fs, ts);
            if (fs < 0.0f) u = I; else v = I;
        }
    };
    keep_y(has_main, ma, mb, ma.y, mb.y);
    // x <= width: the part beyond is dropped
    if (has_main) {
        float fs = width - ma.x, ts = width - mb.x;
        if (fs < 0.0f && ts < 0.0f) {
            has_main = false;
        } else if (fs * ts < 0.0f) {
            float2 I = crossing2(ma, mb, fs, ts);
            if (fs < 0.0f) ma = I; else mb = I;
        }
    }
    keep_y(has_main, ma, mb, height - ma.y, height - mb.y);
    // The left piece lies on x = 0: clamping its ends to [0, height] is its
    // clip to the rectangle, exactly (a crossing would be interpolated).
    auto clamp2 = [&](float2 u) { return f2(lo(hi(u.x, 0.0f), width), lo(hi(u.y, 0.0f), height)); };
    pa[0] = clamp2(ma);
    pb[0] = clamp2(mb);
    pa[1] = clamp2(la);
    pb[1] = clamp2(lb);
    return (has_main ? 1u : 0u) | (has_left ? 2u : 0u);
}

// Coverage of an accumulated signed area s under a fill rule: nonzero
// (the reference's, hpp:2568-2570) min(|s|, 1); even-odd the distance from s
// to the nearest even integer, so each further winding toggles coverage.
__device__ __forceinline__ float cover_of(float s, int rule) {
    return rule ? lo(fabsf(s - 2.0f * rintf(0.5f * s)), 1.0f) : lo(fabsf(s), 1.0f);
}

// ------------------------------------------------------------------ paint
__device__ __forceinline__ float4 premul(float4 c) { return make_float4(c.x * c.w, c.y * c.w, c.z * c.w, c.w); }

__device__ __forceinline__ float keys_weight(float t) {
    return t < 1.0f ? (1.5f * t - 2.5f) * t * t + 1.0f : ((-0.5f * t + 2.5f) * t - 4.0f) * t + 2.0f;
}

struct paint_src {
    const float *stop_off;
    const float4 *stop_col;
    const float4 *texels;
};

// paint_pixel (hpp:2265-2377) at pixel-centre point (px, py).
__device__ float4 paint_at(const command &c, const paint_src &s, float px, float py) {
    const float4 none = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (c.paint == 0) return none;
    if (c.paint == 1) return make_float4(c.color[0], c.color[1], c.color[2], c.color[3]);
    float x = c.inv[0] * px + c.inv[2] * py + c.inv[4];
    float y = c.inv[1] * px + c.inv[3] * py + c.inv[5];
    if (c.paint == 4) {
        float width = static_cast<float>(c.pat_w), height = static_cast<float>(c.pat_h);
        if (((c.pat_rep & 2) && (x < 0.0f || width <= x)) || ((c.pat_rep & 1) && (y < 0.0f || height <= y)))
            return none;
        float scale_x = fabsf(c.inv[0]) + fabsf(c.inv[2]);
        float scale_y = fabsf(c.inv[1]) + fabsf(c.inv[3]);
        scale_x = hi(1.0f, lo(scale_x, width * 0.25f));
        scale_y = hi(1.0f, lo(scale_y, height * 0.25f));
        float rx = 1.0f / scale_x, ry = 1.0f / scale_y;
        x = x - 0.5f;
        y = y - 0.5f;
        int left = static_cast<int>(ceilf(x - scale_x * 2.0f));
        int top = static_cast<int>(ceilf(y - scale_y * 2.0f));
        int right = static_cast<int>(ceilf(x + scale_x * 2.0f));
        int bottom = static_cast<int>(ceilf(y + scale_y * 2.0f));
        float4 total = none;
        float wsum = 0.0f;
        const float4 *tex = c.pat_ptr ? reinterpret_cast<const float4 *>(c.pat_ptr) : s.texels + c.pat_first;
        if (right - left == 4 && bottom - top == 4) {
            // The usual case (no minification): 4 x 4 taps with the weights
            // and wrapped columns in registers; the same sums in the same order.
            float wx[4];
            int col[4];
            int xx = left % c.pat_w;
            if (xx < 0) xx += c.pat_w;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int px_ = left + j;
                wx[j] = keys_weight(fabsf(rx * (static_cast<float>(px_) - x)));
                col[j] = c.clamp ? (px_ < 0 ? 0 : (px_ > c.pat_w - 1 ? c.pat_w - 1 : px_)) : xx;
                if (++xx == c.pat_w) xx = 0;
            }
            int yy = top % c.pat_h;
            if (yy < 0) yy += c.pat_h;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                int py_ = top + i;
                float wy = keys_weight(fabsf(ry * (static_cast<float>(py_) - y)));
                int ry_ = c.clamp ? (py_ < 0 ? 0 : (py_ > c.pat_h - 1 ? c.pat_h - 1 : py_)) : yy;
                if (++yy == c.pat_h) yy = 0;
                const float4 *rowp = tex + static_cast<size_t>(ry_) * c.pat_w;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float w = wx[j] * wy;
                    float4 t = rowp[col[j]];
                    total.x = total.x + t.x * w;
                    total.y = total.y + t.y * w;
                    total.z = total.z + t.z * w;
                    total.w = total.w + t.w * w;
                    wsum += w;
                }
            }
            float r = 1.0f / wsum;
            return make_float4(total.x * r, total.y * r, total.z * r, total.w * r);
        }
        // The column weights and wrapped columns are the same for every row
        // of taps: computed once (same values, same order of the sums).
        constexpr int kTaps = 8;
        float wxs[kTaps];
        int xxs[kTaps];
        const int ncols = right - left;
        const bool cached = ncols <= kTaps;
        int x0w = left % c.pat_w;
        if (x0w < 0) x0w += c.pat_w;
        if (cached) {
            int xx = x0w;
            for (int j = 0; j < ncols; ++j) {
                int px_ = left + j;
                wxs[j] = keys_weight(fabsf(rx * (static_cast<float>(px_) - x)));
                xxs[j] = c.clamp ? (px_ < 0 ? 0 : (px_ > c.pat_w - 1 ? c.pat_w - 1 : px_)) : xx;
                if (++xx == c.pat_w) xx = 0;
            }
        }
        int yy = top % c.pat_h;
        if (yy < 0) yy += c.pat_h;
        for (int py_ = top; py_ < bottom; ++py_) {
            float wy = keys_weight(fabsf(ry * (static_cast<float>(py_) - y)));
            int ry_ = c.clamp ? (py_ < 0 ? 0 : (py_ > c.pat_h - 1 ? c.pat_h - 1 : py_)) : yy;
            if (++yy == c.pat_h) yy = 0;
            const float4 *rowp = tex + static_cast<size_t>(ry_) * c.pat_w;
            int xx = x0w;
            for (int j = 0; j < ncols; ++j) {
                int px_ = left + j;
                float wx;
                int col;
                if (cached) {
                    wx = wxs[j];
                    col = xxs[j];
                } else {
                    wx = keys_weight(fabsf(rx * (static_cast<float>(px_) - x)));
                    col = c.clamp ? (px_ < 0 ? 0 : (px_ > c.pat_w - 1 ? c.pat_w - 1 : px_)) : xx;
                    if (++xx == c.pat_w) xx = 0;
                }
                float w = wx * wy;
                float4 t = rowp[col];
                total.x = total.x + t.x * w;
                total.y = total.y + t.y * w;
                total.z = total.z + t.z * w;
                total.w = total.w + t.w * w;
                wsum += w;
            }
        }
        float r = 1.0f / wsum;
        return make_float4(total.x * r, total.y * r, total.z * r, total.w * r);
    }
    float rx = x - c.p0x, ry = y - c.p0y;
    float lx = c.p1x - c.p0x, ly = c.p1y - c.p0y;
    float grad = rx * lx + ry * ly;
    float span = lx * lx + ly * ly;
    float offset;
    if (c.paint == 2) {
        if (span == 0.0f) return none;
        offset = grad / span;
    } else {
        float initial = c.r0;
        float change = c.r1 - initial;
        float a = span - change * change;
        float b = -2.0f * (grad + initial * change);
        float cc = (rx * rx + ry * ry) - initial * initial;
        float disc = b * b - 4.0f * a * cc;
        if (disc < 0.0f || (span == 0.0f && change == 0.0f)) return none;
        float root = sqrtf(disc);
        float recip = 1.0f / (2.0f * a);
        float o1 = (-b - root) * recip;
        float o2 = (-b + root) * recip;
        float rad1 = initial + change * o1;
        float rad2 = initial + change * o2;
        if (rad2 >= 0.0f) offset = o2;
        else if (rad1 >= 0.0f) offset = o1;
        else return none;
    }
    const float *stops = s.stop_off + c.stop_first;
    const float4 *cols = s.stop_col + c.stop_first;
    // std::upper_bound (hpp:2366-2368).  add_color_stop keeps the stops
    // sorted, so a linear walk finds the same index; the first eight stops
    // are loaded together before the walk.
    int n = c.stop_count, k = 0;
    float st[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) st[i] = i < n ? stops[i] : 0.0f;
    bool done = false;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (!done) {
            if (i < n && !(offset < st[i])) ++k;
            else done = true;
        }
    }
    if (!done)
        while (k < n && !(offset < stops[k])) ++k;
    if (k == 0) return premul(cols[0]);
    if (k == n) return premul(cols[n - 1]);
    float t = (offset - stops[k - 1]) / (stops[k] - stops[k - 1]);
    float4 c0 = cols[k - 1], c1 = cols[k];
    float4 m = make_float4(c0.x + t * (c1.x - c0.x), c0.y + t * (c1.y - c0.y), c0.z + t * (c1.z - c0.z),
                           c0.w + t * (c1.w - c0.w));
    return premul(m);
}

// Composite `fore` into `back` with a 4-bit operation code and clip
// visibility (hpp:2522-2533, 2583-2591).
__device__ __forceinline__ float4 blend(float4 back, float4 fore, int op, float vis) {
    float mf = op & 1 ? back.w : 0.0f;
    if (op & 2) mf = 1.0f - mf;
    float mb = op & 4 ? fore.w : 0.0f;
    if (op & 8) mb = 1.0f - mb;
    float4 b = make_float4(fore.x * mf + back.x * mb, fore.y * mf + back.y * mb, fore.z * mf + back.z * mb,
                           fore.w * mf + back.w * mb);
    b.w = lo(b.w, 1.0f);
    // Full visibility: visibility * blend + (1 - visibility) * back is blend
    // (up to the sign of a zero).
    if (vis == 1.0f) return b;
    float iv = 1.0f - vis;
    return make_float4(b.x * vis + back.x * iv, b.y * vis + back.y * iv, b.z * vis + back.z * iv,
                       b.w * vis + back.w * iv);
}

// get_image_data's per-pixel conversion (hpp:3348-3381): unpremultiply,
// clamp, delinearize, x255 plus the 4x4 Bayer threshold, truncate.  The
// colour bytes come from a table built on the host with the reference's own
// formula: g_srgb_thr[d][q] is the least clamped value whose byte under
// Bayer cell d is at least q, so the byte is the count of thresholds at or
// below the value.  A fast estimate lands within a step or two of it and
// the table settles it; the bytes are then exactly the host formula's.
__device__ float g_srgb_thr[16][256];

__device__ __constant__ float kBayer[16] = {0.03125f, 0.53125f, 0.15625f, 0.65625f, 0.78125f, 0.28125f,
                                            0.90625f, 0.40625f, 0.21875f, 0.71875f, 0.09375f, 0.59375f,
                                            0.96875f, 0.46875f, 0.84375f, 0.34375f};

__device__ __forceinline__ int srgb_byte(float u, int d, float t) {
    float s = u < 0.0031308f ? 12.92f * u : 1.055f * __powf(u, 1.0f / 2.4f) - 0.055f;
    int q = __float2int_rz(t + 255.0f * s);
    q = q < 0 ? 0 : q > 255 ? 255 : q;
    const float *T = g_srgb_thr[d];
    while (q < 255 && u >= T[q + 1]) ++q;
    while (q > 0 && u < T[q]) --q;
    return q;
}

__device__ __forceinline__ uchar4 to_srgb8(float4 c, int cx, int cy) {
    float4 u;
    if (c.w < kVisible) {
        u = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else {
        float r = 1.0f / c.w;
        u = make_float4(r * c.x, r * c.y, r * c.z, c.w);
    }
    u.x = lo(hi(u.x, 0.0f), 1.0f);
    u.y = lo(hi(u.y, 0.0f), 1.0f);
    u.z = lo(hi(u.z, 0.0f), 1.0f);
    u.w = lo(hi(u.w, 0.0f), 1.0f);
    int d = ((cy & 3) << 2) | (cx & 3);
    float t = kBayer[d];
    float a = t + 255.0f * u.w;
    return make_uchar4(static_cast<unsigned char>(srgb_byte(u.x, d, t)),
                       static_cast<unsigned char>(srgb_byte(u.y, d, t)),
                       static_cast<unsigned char>(srgb_byte(u.z, d, t)),
                       static_cast<unsigned char>(__float2int_rz(a) & 0xff));
}

}  // namespace cyg

#endif
