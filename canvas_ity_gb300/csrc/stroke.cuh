// stroke.cuh -- stroke expansion on the device.
//
// The reference turns a stroked path into a fill: the path is flattened with
// the stroking angle limit (path_to_lines, hpp:1495-1524), split by the dash
// pattern (dash_lines, hpp:1858-1934) and traced forwards and backwards to
// add the two half strokes with their joins and caps (add_half_stroke,
// stroke_lines, hpp:1949-2100).  The dash phase is a float running sum
// carried along a subpath (one warp per subpath, lane 0 carries it); the
// walk's point acceptance is resolved 32 positions at a time (one warp per
// piece), after which every join and cap is independent and computed by one
// warp per 32 walk positions over all canvases at once.  Each pass counts,
// scans, then writes.  The float operations are the reference's, in its
// order; the one exception is the round join's acosf/tanf, taken in double
// precision and rounded to float.
#ifndef CY_STROKE_CUH
#define CY_STROKE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace cyg {

static constexpr int kDashCap = 1 << 22;     // dashed points one subpath may produce

__device__ __forceinline__ float2 xform(const float *m, float2 p) {
    return f2(m[0] * p.x + m[2] * p.y + m[4], m[1] * p.x + m[3] * p.y + m[5]);
}
__device__ __forceinline__ float len2(float2 a) { return sqrtf(dot2(a, a)); }
__device__ __forceinline__ float2 unit2(float2 a) { return scl2(1.0f / hi(1.0e-6f, len2(a)), a); }

// A round join's or round cap's curve, flattened in fill mode: one copy of
// the flattening code for all call sites of a kernel.
template <bool EMIT>
__device__ __noinline__ int curve_points(float2 a, float2 b, float2 c, float2 d, float2 *out, int cap) {
    return flatten_cubic<EMIT>(a, b, c, d, -1.0f, out, cap);
}

// One join of add_half_stroke (hpp:1966-2041) at `point` between the
// accepted segments in_dir/in_len and out_dir/out_len (user space).  Returns
// the number of device-space points it adds.  A round join's factor
// 4/3 tan(angle / 4) is computed when counting (EMIT=false) and stored in
// `alpha`; writing (EMIT=true) takes it from there.
template <bool EMIT>
__device__ int stroke_join(float2 point, float2 in_dir, float in_len, float2 out_dir, float out_len,
                           const stroke_style &s, float2 *out, int cap, float &alpha) {
    const float half = s.half;
    const float eps = 1.0e-4f;
    int n = 0;
    auto put = [&](float2 user) {
        if (EMIT && n < cap) out[n] = xform(s.fwd, user);
        ++n;
    };
    float2 side_in = add2(point, scl2(half, perp2(in_dir)));
    float2 side_out = add2(point, scl2(half, perp2(out_dir)));
    float turn = dot2(perp2(in_dir), out_dir);
    if (fabsf(turn) < eps) turn = 0.0f;
    float2 offset = turn == 0.0f ? f2(0.0f, 0.0f) : scl2(half / turn, sub2(out_dir, in_dir));
    bool tight = dot2(offset, in_dir) < -in_len && dot2(offset, out_dir) > out_len;
    if (turn > 0.0f && tight) {
        float2 t = side_in;
        side_in = side_out;
        side_out = t;
        t = in_dir;
        in_dir = out_dir;
        out_dir = t;
        put(side_out);
        put(point);
        put(side_in);
    }
    if ((turn > 0.0f && !tight) || (turn != 0.0f && s.join == 0 && dot2(offset, offset) <= s.ratio)) {
        put(add2(point, offset));
    } else if (s.join == 2) {
        if (!EMIT) {
            float cosine = dot2(in_dir, out_dir);
            float angle = static_cast<float>(acos(static_cast<double>(lo(hi(cosine, -1.0f), 1.0f))));
            alpha = 4.0f / 3.0f * static_cast<float>(tan(static_cast<double>(0.25f * angle)));
        }
        put(side_in);
        n += curve_points<EMIT>(xform(s.fwd, side_in), xform(s.fwd, add2(side_in, scl2(alpha * half, in_dir))),
                                xform(s.fwd, sub2(side_out, scl2(alpha * half, out_dir))), xform(s.fwd, side_out),
                                out + (EMIT ? n : 0), cap - n);
    } else {
        put(side_in);
        put(side_out);
    }
    if (turn > 0.0f && tight) {
        put(side_out);
        put(point);
        put(side_in);
    }
    return n;
}

// The cap of an open half stroke (hpp:2044-2057) at its last point.
template <bool EMIT>
__device__ int stroke_cap(float2 point, float2 in_dir, const stroke_style &s, float2 *out, int cap) {
    int n = 0;
    auto put = [&](float2 user) {
        if (EMIT && n < cap) out[n] = xform(s.fwd, user);
        ++n;
    };
    float2 ahead = scl2(s.half, in_dir);
    float2 side = perp2(ahead);
    if (s.cap == 0) {
        put(add2(point, side));
        put(sub2(point, side));
    } else if (s.cap == 1) {
        put(add2(add2(point, ahead), side));
        put(sub2(add2(point, ahead), side));
    } else if (s.cap == 2) {
        const float k = 0.55228475f;   // 4/3 tan(pi/8)
        put(add2(point, side));
        n += curve_points<EMIT>(xform(s.fwd, add2(point, side)), xform(s.fwd, add2(add2(point, side), scl2(k, ahead))),
                                xform(s.fwd, add2(add2(point, ahead), scl2(k, side))), xform(s.fwd, add2(point, ahead)),
                                out + (EMIT ? n : 0), cap - n);
        n += curve_points<EMIT>(xform(s.fwd, add2(point, ahead)), xform(s.fwd, sub2(add2(point, ahead), scl2(k, side))),
                                xform(s.fwd, add2(sub2(point, side), scl2(k, ahead))), xform(s.fwd, sub2(point, side)),
                                out + (EMIT ? n : 0), cap - n);
    }
    return n;
}

// Inputs of the stroke kernels.
// The dash walk's state where a centre-line segment starts (hpp:1880-1888
// and the loop of 1889-1925): the write pass replays each segment from it.
struct dash_state {
    float next;                  // distance left in the current pattern entry
    int32_t seg;                 // current pattern entry
    int32_t np, ns, first;       // points and dashes written so far, first point of the open dash
    int32_t emit;                // 1 while inside a dash
};

struct stroke_in {
    const float2 *flat;          // flattened centre lines (flattening output)
    const int32_t *item_off;     // flattening offsets per flat_item
    const stroke_group *groups;
    const stroke_style *styles;
    const float *dash;           // dash patterns
    float2 *dash_pts;            // dashed centre lines, group g's at dash_off[g]
    int2 *dash_subs;             // (count, closed) per dash, group g's at dash_off[g]
    const int32_t *dash_off;
    int32_t *dash_nsub;          // dashes per group
    dash_state *dash_state_at;   // per centre-line point of a dashed group: the state where its segment starts
    int32_t nflat;               // centre-line points before the dashed ones in slot numbering
    int n;
    int32_t *error;              // set to 1 when a subpath exceeds a cap
};

static constexpr int kStrokeWarps = 4;   // warps per block of the stroke kernels

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Dash pass, one warp per subpath.  Counting (EMIT=false): the lanes
// measure 32 segments at a time (the user-space lengths of hpp:1895), lane 0
// carries the pattern phase through them in order -- a float running sum,
// so it stays sequential -- and records the walk's state where each segment
// starts (and after the last one); each group's dashed point count goes to
// `counts` (0 without a pattern).  Writing (EMIT=true): every lane replays
// its own segments from their recorded states, so the writes run 32 wide,
// then lane 0 closes the last dash.
template <bool EMIT>
__global__ void __launch_bounds__(kStrokeWarps * 32) k_dash(stroke_in in, int32_t *__restrict__ counts) {
    __shared__ float lens[kStrokeWarps][32];
    __shared__ float2 ends[kStrokeWarps][33];   // the chunk's points (segment ends)
    __shared__ float pat[kStrokeWarps][64];     // the pattern, when it has at most 64 entries
    __shared__ dash_state states[kStrokeWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = blockIdx.x * kStrokeWarps + w;
    if (g >= in.n) return;
    stroke_group gr = in.groups[g];
    const stroke_style s = in.styles[gr.style];
    if (s.dash_n <= 0) {
        if (!EMIT && lane == 0) counts[g] = 0;
        return;
    }
    const float *dash = in.dash + s.dash_first;
    if (s.dash_n <= 64) {
        for (int i = lane; i < s.dash_n; i += 32) pat[w][i] = dash[i];
        __syncwarp();
        dash = pat[w];
    }
    const int a = in.item_off[gr.head], n = in.item_off[gr.end] - a;
    const float2 *pts = in.flat + a;
    dash_state *state_at = in.dash_state_at + a;
    const bool merge_emit = (~s.dash_start & 1) != 0;
    if (!EMIT) {
        // lane 0's state (hpp:1880-1888)
        int np = 0, ns = 0, first = 0, seg = s.dash_start;
        bool emit = merge_emit;
        float next = s.dash_next;
        bool over = false;
        for (int c = 0; c + 1 < n; c += 32) {
            const int i = c + lane, m = min(32, n - 1 - c);
            float line = 0.0f;
            if (i < n) ends[w][lane] = pts[i];
            if (lane == 0 && c + 32 < n) ends[w][32] = pts[c + 32];
            if (i + 1 < n) line = len2(sub2(xform(s.inv, pts[i + 1]), xform(s.inv, pts[i])));
            lens[w][lane] = line;
            __syncwarp();
            if (lane == 0 && !over) {
                for (int k = 0; k < m; ++k) {
                    states[w][k] = dash_state{next, seg, np, ns, first, emit ? 1 : 0};
                    const float len = lens[w][k];
                    if (emit) ++np;
                    while (next < len) {
                        if (np >= kDashCap) {
                            over = true;
                            break;
                        }
                        ++np;
                        if (emit) {
                            ++ns;
                            first = np;
                        }
                        seg = seg + 1 < s.dash_n ? seg + 1 : 0;
                        emit = !emit;
                        next += dash[seg];
                    }
                    if (over) break;
                    next -= len;
                }
            }
            __syncwarp();
            if (lane < m) state_at[c + lane] = states[w][lane];
            __syncwarp();
        }
        if (lane == 0) {
            if (n > 0 && !over) state_at[n - 1] = dash_state{next, seg, np, ns, first, emit ? 1 : 0};
            if (emit && !over && n > 0) ++np;   // the last dash ends at the last point
            if (over) atomicOr(in.error, 1);
            counts[g] = over ? 0 : np;
        }
        return;
    }
    const int o = in.dash_off[g], cap = in.dash_off[g + 1] - o;
    float2 *out = in.dash_pts + o;
    int2 *subs = in.dash_subs + o;
    if (cap <= 0) {
        if (lane == 0) in.dash_nsub[g] = 0;
        return;
    }
    // every segment from the state where it starts (the loop of hpp:1889-1925)
    for (int i = lane; i + 1 < n; i += 32) {
        const dash_state st = state_at[i];
        const float2 from = pts[i], to = pts[i + 1];
        const float len = len2(sub2(xform(s.inv, to), xform(s.inv, from)));
        int np = st.np, ns = st.ns, first = st.first, seg = st.seg;
        bool emit = st.emit != 0;
        float next = st.next;
        if (emit) {
            if (np < cap) out[np] = from;
            ++np;
        }
        while (next < len && np < cap) {
            out[np] = mix2(from, to, next / len);
            ++np;
            if (emit) {
                if (ns < cap) subs[ns] = make_int2(np - first, 0);
                ++ns;
                first = np;
            }
            seg = seg + 1 < s.dash_n ? seg + 1 : 0;
            emit = !emit;
            next += dash[seg];
        }
    }
    __syncwarp();
    int count = 0, np = 0, ns = 0;   // (lane 0) the rotation below, the totals
    if (lane == 0 && n > 0) {
        const dash_state st = state_at[n - 1];
        np = st.np;
        ns = st.ns;
        if (st.emit) {
            if (np < cap) out[np] = pts[n - 1];
            ++np;
            if (ns < cap) subs[ns] = make_int2(np - st.first, 0);
            ++ns;
            if (gr.closed && merge_emit) {
                if (ns == 1) {
                    subs[0].y = 1;
                } else {
                    count = np - st.first;
                    subs[0].x += count;
                    --ns;
                }
            }
        }
    }
    // Closed subpath whose first and last dashes are drawn: the last dash
    // moves in front of the first (std::rotate by three reversals).
    count = __shfl_sync(0xffffffffu, count, 0);
    np = __shfl_sync(0xffffffffu, np, 0);
    __syncwarp();
    if (count > 0 && np == cap) {
        auto reverse = [&](int lo_, int hi_) {
            int len = hi_ - lo_;
            for (int t = lane; t < len / 2; t += 32) {
                float2 x = out[lo_ + t];
                out[lo_ + t] = out[hi_ - 1 - t];
                out[hi_ - 1 - t] = x;
            }
            __syncwarp();
        };
        reverse(0, np - count);
        reverse(np - count, np);
        reverse(0, np);
    }
    if (lane == 0) in.dash_nsub[g] = np == cap ? ns : 0;
}

// ------------------------------------------------------------ the walks
// stroke_lines (hpp:2070-2100) traces every piece (subpath after dashing)
// forwards and backwards with add_half_stroke.  A walk accepts a point when
// it lies at least eps from the last accepted one, and each accepted point
// after the first two completes the join at the accepted point before it; a
// closed walk wraps around until it reaches the position of its first join,
// an open one ends with a cap.  So once the accepted points are known, every
// join is independent: k_walk resolves acceptance 32 walk positions at a
// time into chunk records, and k_join computes the joins of all chunks of
// all canvases in parallel, one warp per chunk.

// One chunk of up to 32 consecutive positions of one walk.
struct walk_chunk {
    int32_t pts;          // unified index of the piece's first point (centre lines, then dashes)
    int32_t cnt;          // points of the piece
    int32_t flags;        // 1 backward, 2 closed, 4 wrap part (positions revisit the first points)
    int32_t style;
    uint32_t acc;         // accepted positions (bit = lane)
    int32_t c1, c2;       // the last two accepted points before the chunk (c2 -1: none yet)
    int32_t pos0;         // position of lane 0 within its part
    int32_t n;            // lanes in use
    int32_t poly0, poly1; // chunks of the chunk's polygon: [poly0, poly1)
    int32_t pad;
};

// One piece to walk (a subpath after dashing).
struct stroke_piece {
    int32_t pts;     // unified index of the first point (centre lines, then dashes)
    int32_t cnt;
    int32_t closed;
    int32_t style;
};

__device__ __forceinline__ const float2 *piece_points(const stroke_in &in, int32_t base) {
    return base < in.nflat ? in.flat + base : in.dash_pts + (base - in.nflat);
}

// Walk position -> point of the piece.
__device__ __forceinline__ int walk_index(int pos, int cnt, bool backward) { return backward ? cnt - 1 - pos : pos; }

// Position of the first join of a closed walk (where the second point after
// the start is accepted), or -1: one lane, usually a few steps.
__device__ int first_join(const float2 *pp, int cnt, bool backward, const stroke_style &s) {
    const float eps = 1.0e-4f;
    float2 pt = xform(s.inv, pp[walk_index(0, cnt, backward)]);
    int seen = 0;
    for (int pos = 1; pos < cnt; ++pos) {
        float2 x = xform(s.inv, pp[walk_index(pos, cnt, backward)]);
        if (len2(sub2(x, pt)) >= eps) {
            if (++seen == 2) return pos;
            pt = x;
        }
    }
    return -1;
}

// Pieces of each group: 1 without a dash pattern, else its dashes.
__global__ void k_piece_count(stroke_in in, int32_t *__restrict__ counts) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= in.n) return;
    const stroke_style &s = in.styles[in.groups[g].style];
    counts[g] = s.dash_n > 0 ? in.dash_nsub[g] : 1;
}

// The piece records of each group, from base[g].
__global__ void k_pieces(stroke_in in, const int32_t *__restrict__ base, stroke_piece *__restrict__ pieces) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= in.n) return;
    stroke_group gr = in.groups[g];
    const stroke_style &s = in.styles[gr.style];
    stroke_piece *out = pieces + base[g];
    if (s.dash_n > 0) {
        const int d0 = in.dash_off[g], ns = in.dash_nsub[g];
        int q = 0;
        for (int k = 0; k < ns; ++k) {
            int2 sub = in.dash_subs[d0 + k];
            out[k] = stroke_piece{in.nflat + d0 + q, sub.x, sub.y, gr.style};
            q += sub.x;
        }
    } else {
        const int a = in.item_off[gr.head], b = in.item_off[gr.end];
        out[0] = stroke_piece{a, b - a, gr.closed, gr.style};
    }
}

// Chunks of one walk: its first part (an open walk has the cap position
// after its points), then the wrap of a closed walk up to its first join.
__device__ __forceinline__ int walk_chunk_count(int cnt, bool closed, int fin) {
    return ((closed ? cnt : cnt + 1) + 31) / 32 + (closed && fin > 0 ? (fin + 31) / 32 : 0);
}

// Chunks of each piece (both walks), without walking.
__global__ void k_piece_chunks(stroke_in in, const stroke_piece *__restrict__ pieces, int n,
                               int32_t *__restrict__ counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    stroke_piece pc = pieces[i];
    int c = 0;
    if (pc.cnt >= 2) {
        const stroke_style &s = in.styles[pc.style];
        const float2 *pp = piece_points(in, pc.pts);
        int ff = pc.closed ? first_join(pp, pc.cnt, false, s) : -1;
        int fb = pc.closed ? first_join(pp, pc.cnt, true, s) : -1;
        c = walk_chunk_count(pc.cnt, pc.closed != 0, ff) + walk_chunk_count(pc.cnt, pc.closed != 0, fb);
    }
    counts[i] = c;
}

// k_walk: one warp per piece, writing its chunks from chunk_base[piece].
__global__ void __launch_bounds__(kStrokeWarps * 32) k_walk(stroke_in in, const stroke_piece *__restrict__ pieces,
                                                            int n_pieces, const int32_t *__restrict__ chunk_base,
                                                            walk_chunk *__restrict__ chunks) {
    const float eps = 1.0e-4f;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int pi = blockIdx.x * kStrokeWarps + w;
    if (pi >= n_pieces) return;
    const stroke_piece pc = pieces[pi];
    const int cnt = pc.cnt;
    if (cnt < 2) return;
    const bool closed = pc.closed != 0;
    const stroke_style s = in.styles[pc.style];
    const float2 *pp = piece_points(in, pc.pts);
    const int cb = chunk_base[pi];
    int nch = 0;
    auto walk = [&](bool backward, int fin, int poly0, int poly1) {
        const int begin = walk_index(0, cnt, backward);
        int c1 = begin, c2 = -1;
        bool synced = true;
        float2 point = xform(s.inv, pp[begin]);
        const int n1 = closed ? cnt : cnt + 1;
        for (int part = 0; part < 2; ++part) {
            const int np_all = part == 0 ? n1 : (closed && fin > 0 ? fin : 0);
            for (int p0 = 0; p0 < np_all; p0 += 32) {
                const int np = min(32, np_all - p0);
                const int pos = p0 + lane;
                const bool point_lane = lane < np && pos < cnt;   // not the cap position
                const int idx = point_lane ? walk_index(pos, cnt, backward) : begin;
                float2 q = xform(s.inv, pp[idx]);
                float2 qprev = q;
                if (point_lane) {
                    int pp_pos = pos > 0 ? pos - 1 : (part == 1 ? cnt - 1 : 0);
                    qprev = xform(s.inv, pp[walk_index(pp_pos, cnt, backward)]);
                }
                const bool is_start = part == 0 && pos == 0;
                bool ok = !point_lane || is_start || len2(sub2(q, qprev)) >= eps;
                unsigned acc;
                if (synced && __all_sync(full, ok)) {
                    acc = __ballot_sync(full, point_lane && !is_start);
                } else {
                    // lane 0 replays the acceptance from the last accepted point
                    unsigned m = 0;
                    if (lane == 0) {
                        float2 pt = point;
                        for (int t = 0; t < np; ++t) {
                            int ps = p0 + t;
                            if ((part == 0 && ps == 0) || ps >= cnt) continue;
                            float2 x = xform(s.inv, pp[walk_index(ps, cnt, backward)]);
                            if (len2(sub2(x, pt)) >= eps) {
                                m |= 1u << t;
                                pt = x;
                            }
                        }
                    }
                    acc = __shfl_sync(full, m, 0);
                }
                if (lane == 0) {
                    walk_chunk h;
                    h.pts = pc.pts;
                    h.cnt = cnt;
                    h.flags = (backward ? 1 : 0) | (closed ? 2 : 0) | (part == 1 ? 4 : 0);
                    h.style = pc.style;
                    h.acc = acc;
                    h.c1 = c1;
                    h.c2 = c2;
                    h.pos0 = p0;
                    h.n = np;
                    h.poly0 = cb + poly0;
                    h.poly1 = cb + poly1;
                    h.pad = 0;
                    chunks[cb + nch] = h;
                }
                ++nch;
                if (acc) {
                    int hb = 31 - __clz(acc);
                    unsigned rest = acc & ~(1u << hb);
                    c2 = rest ? walk_index(p0 + (31 - __clz(rest)), cnt, backward) : c1;
                    c1 = walk_index(p0 + hb, cnt, backward);
                    point = xform(s.inv, pp[c1]);
                }
                // in step when the last position with a point was accepted
                int last = min(np, cnt - p0) - 1;
                synced = last >= 0 && (((acc >> last) & 1u) || (part == 0 && p0 + last == 0));
            }
        }
    };
    int ff = -1, fb = -1;
    if (closed) {
        int a = 0, b = 0;
        if (lane == 0) {
            a = first_join(pp, cnt, false, s);
            b = first_join(pp, cnt, true, s);
        }
        ff = __shfl_sync(full, a, 0);
        fb = __shfl_sync(full, b, 0);
    }
    const int nf = walk_chunk_count(cnt, closed, ff), nb = walk_chunk_count(cnt, closed, fb);
    if (closed) {
        walk(false, ff, 0, nf);
        walk(true, fb, nf, nf + nb);
    } else {
        walk(false, ff, 0, nf + nb);
        walk(true, fb, 0, nf + nb);
    }
}

// The walk positions of every chunk, packed: pos_base[c] (an exclusive
// scan of the chunks' lane counts) is chunk c's first packed position, and
// pos_chunk[p] the chunk of packed position p.  A piece of a few points
// makes a chunk of a few lanes; packed, the joins of many such chunks share
// a warp.
__global__ void k_chunk_lanes(const walk_chunk *__restrict__ chunks, int n_chunks, int32_t *__restrict__ lanes) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n_chunks) lanes[c] = chunks[c].n;
}

__global__ void k_chunk_positions(const walk_chunk *__restrict__ chunks, int n_chunks,
                                  const int32_t *__restrict__ pos_base, int32_t *__restrict__ pos_chunk) {
    const int lane = threadIdx.x & 31;
    const int c = static_cast<int>((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
    if (c >= n_chunks) return;
    if (lane < chunks[c].n) pos_chunk[pos_base[c] + lane] = c;
}

// k_join: one thread per packed walk position.  EMIT=false writes the
// position's point count to jcnt[p] (and a round join's factor to
// jalpha[p]); EMIT=true writes the join (or cap) at joff[p] (the exclusive
// scan of the counts), with prev links: the point before, except for a
// polygon's first point, linked to the polygon's last.
template <bool EMIT>
__global__ void __launch_bounds__(kStrokeWarps * 32) k_join(stroke_in in, const walk_chunk *__restrict__ chunks,
                                                            const int32_t *__restrict__ pos_base,
                                                            const int32_t *__restrict__ pos_chunk, int n_pos,
                                                            int32_t *__restrict__ jcnt, float *__restrict__ jalpha,
                                                            const int64_t *__restrict__ joff,
                                                            float2 *__restrict__ out, int32_t *__restrict__ prev,
                                                            int32_t base, int64_t cap) {
    const int p = static_cast<int>(static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
    if (p >= n_pos) return;
    const int c = pos_chunk[p];
    const int lane = p - pos_base[c];
    const walk_chunk h = chunks[c];
    const stroke_style s = in.styles[h.style];
    const float2 *pp = piece_points(in, h.pts);
    const bool backward = h.flags & 1, closed = h.flags & 2;
    const int cnt = h.cnt;
    const int pos = h.pos0 + lane;
    const bool is_cap = !closed && !(h.flags & 4) && pos == cnt;
    // the two accepted points before this lane's position
    unsigned below = h.acc & ((1u << lane) - 1u);
    int p1 = h.c1, p2 = h.c2;
    if (below) {
        int b1 = 31 - __clz(below);
        p1 = walk_index(h.pos0 + b1, cnt, backward);
        unsigned rest = below & ~(1u << b1);
        p2 = rest ? walk_index(h.pos0 + (31 - __clz(rest)), cnt, backward) : h.c1;
    }
    const bool join = ((h.acc >> lane) & 1u) && p2 >= 0;
    const bool capped = is_cap && p2 >= 0;
    float2 jp = f2(0.0f, 0.0f), din = jp, dout = jp;
    if (join || capped) {
        jp = xform(s.inv, pp[p1]);
        din = sub2(jp, xform(s.inv, pp[p2]));
    }
    if (join) dout = sub2(xform(s.inv, pp[walk_index(pos, cnt, backward)]), jp);
    int n = 0;
    float alpha = 0.0f;
    if (!EMIT) {
        if (join) n = stroke_join<false>(jp, unit2(din), len2(din), unit2(dout), len2(dout), s, nullptr, 0, alpha);
        else if (capped) n = stroke_cap<false>(jp, unit2(din), s, nullptr, 0);
        jalpha[p] = alpha;
        if (n > (1 << 24)) {   // a join or cap far beyond any canvas (line width ~1e11)
            atomicOr(in.error, 1);
            n = 0;
        }
        jcnt[p] = n;
        return;
    }
    n = jcnt[p];
    const int64_t at = joff[p];
    if (n == 0 || at < 0 || at + n > cap) return;
    alpha = jalpha[p];
    if (join) stroke_join<true>(jp, unit2(din), len2(din), unit2(dout), len2(dout), s, out + at, n, alpha);
    else stroke_cap<true>(jp, unit2(din), s, out + at, n);
    const int64_t first = joff[pos_base[h.poly0]], last = joff[pos_base[h.poly1]] - 1;
    for (int k = 0; k < n; ++k) {
        int64_t e = at + k;
        prev[e] = base + static_cast<int32_t>(e == first ? last : e - 1);
    }
}

// Output range of each group: goff[g] = the offset of its first piece's
// first chunk's first position (g <= n).
__global__ void k_group_off(const int32_t *__restrict__ piece_base, const int32_t *__restrict__ chunk_base,
                            const int32_t *__restrict__ pos_base, const int64_t *__restrict__ joff, int n,
                            int64_t *__restrict__ goff) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g <= n) goff[g] = joff[pos_base[chunk_base[piece_base[g]]]];
}

}  // namespace cyg

#endif
