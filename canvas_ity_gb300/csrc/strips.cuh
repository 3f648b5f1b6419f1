// strips.cuh -- the batched ("strip") render path.
//
// After all scan conversions of a frame are done (row-sorted runs with
// running sums, see kernels.cuh), one persistent kernel renders every canvas
// of the frame.  A work item is a horizontal strip of one canvas, at most
// `strip_pixels` pixels; its premultiplied linear float pixels live in shared
// memory while the kernel applies, in call order, every command of the
// canvas: shadow composite and paint of draws, put_image_data,
// get_image_data.  Pixels are read from HBM at most once (when the canvas
// already had content) and written once (RGBA8 for the reads, float state
// for a canvas that persists).  Each pixel of a strip is always handled by
// the same thread (fixed 32-pixel chunk to warp assignment), so no barrier
// is needed between commands.
#ifndef CY_STRIPS_CUH
#define CY_STRIPS_CUH

#include "kernels.cuh"

namespace cyg {

struct strip_canvas {
    int32_t W, H, TH;         // size and strip height
    int32_t cmd_first, cmd_count;
    int32_t flags;            // 1: load float state from `bitmap`, 2: store it back
    float4 *bitmap;
};

struct strip_cmd {            // per command extras resolved at the flush
    int32_t main_row_base;    // rows of the command's main scan job (sorted-run coverage)
    int32_t bin_base;         // binned coverage: first row-band bin of the main job
    int32_t band_h;           // binned coverage: rows per band
    int32_t has_shadow;
    int64_t shadow_img;       // float offset of the blurred shadow image
    const float *vis;         // clip visibility (null: whole canvas)
    int64_t get_out;          // GET: byte offset of the compact RGBA8 output
    int32_t get_x, get_y, get_w, get_h;
};

struct strip_params {
    const strip_canvas *canvases;
    const int2 *items;        // (canvas, first row) in processing order
    int n_items;
    int *counter;             // work-queue cursor (reset per run)
    const command *cmds;
    const strip_cmd *ext;
    row_view rv;
    paint_src src;
    const shadow_rect *rects; // per command (valid for shadows)
    const float *shadow_imgs;
    const uint8_t *put_px;
    const float *lut;
    uint8_t *get_buf;
    int strip_pixels;         // pixels of the largest strip (shared memory per strip)
    int strip_words;          // binned: 32-bit words of the largest strip's chunk marks
    const int64_t *bin_off;   // binned coverage: first entry of each bin (and the end)
    const float4 *bin_seg;    // binned coverage: segment end points
};

// ------------------------------------------------- binned coverage (strips)
// Signed areas are accumulated in shared memory as 32-bit fixed point with
// kAccBits fractional bits.  A row of a segment is walked cell by cell as
// add_runs walks it (hpp:2131-2169); the value C_m that its cells up to m
// add to every pixel from m on is sign * (S_m - area_m), where S_m is the
// row's vertical extent from its entry point to the cell's right crossing
// and area_m the cell's own trapezoid, and cell pe + 1 (past the exit)
// completes the row with sign * S_pe.  Each cell adds round(C_m * 2^kAccBits)
// minus the same for the cell before, so a row's integers telescope and the
// prefix sum of a pixel row is off by at most half a unit per segment row to
// its left.  Every C_m has this closed form, so the part of a row left of a
// column is known without walking it.  Integer adds commute, so the result
// does not depend on which lane or warp gets where first.  Windings beyond
// +-2^(31-kAccBits) wrap: coverage is only wrong where the winding is a
// nonzero multiple of 2^(32-kAccBits) (1024 overlapping layers of one path).
static constexpr int kAccBits = 22;
static constexpr float kAccScale = 4194304.0f;          // 2^kAccBits
static constexpr float kAccInv = 1.0f / 4194304.0f;

// Where the walk of row k enters cell m > ps: the crossing of x = m.
__device__ __forceinline__ float2 dda_cross(const dda_piece &p, int m) {
    if (p.vert) return f2(p.tx, p.ty);
    float cx = static_cast<float>(m);
    return f2(cx, (cx - p.fx) * p.sy + p.fy);
}

// The fixed-point C_m of cell m in [ps, pe] from its left point L and right
// point R, the row's entry point E.
__device__ __forceinline__ int acc_q(const dda_piece &p, int m, float2 E, float2 L, float2 R) {
    float strip = lo(hi((R.y - L.y) * p.ystep, 0.0f), 1.0f);
    float mid = (R.x + L.x) * 0.5f;
    float area = (mid - static_cast<float>(m)) * strip;
    float S = lo(hi((R.y - E.y) * p.ystep, 0.0f), 1.0f);
    return __float2int_rn((S - area) * p.sign * kAccScale);
}

// Accumulate the cells of row k of piece p that lie in columns [xa, xb)
// into row_acc; returns the row's integer total over the columns left of xa
// (0 when xa == 0).  [x0, x1] receives the columns of the cells written.
__device__ __forceinline__ int raster_row(const dda_piece &p, int k, int *row_acc, int W, int xa, int xb, int &x0,
                                          int &x1) {
    float2 E = k == 0 ? f2(p.fx, p.fy) : dda_exit(p, k - 1);
    float2 X = dda_exit(p, k);
    int ps, pe;
    dda_span(p, k, E, X, ps, pe);
    // Segments are clamped to [0, W] x [0, H], so a row's cells lie in
    // [0, W + 1]; anything else comes from non-finite input: skipped.
    if (!(ps >= 0 && pe >= ps && pe <= W + 1)) return 0;
    if (ps >= xb) return 0;
    int m = ps, qprev = 0, left = 0;
    float2 L = E;
    if (xa > ps) {
        // cells ps .. xa-1 belong to columns left of this range
        const int ms = min(pe + 1, xa - 1);
        if (ms == pe + 1) {
            float S = lo(hi((X.y - E.y) * p.ystep, 0.0f), 1.0f);
            return __float2int_rn(S * p.sign * kAccScale);
        }
        float2 Lm = ms == ps ? E : dda_cross(p, ms);
        float2 Rm = ms < pe ? dda_cross(p, ms + 1) : X;
        qprev = left = acc_q(p, ms, E, Lm, Rm);
        m = ms + 1;
        L = Rm;
    }
    for (; m <= pe + 1 && m < xb; ++m) {
        int q;
        if (m <= pe) {
            float2 R = m < pe ? dda_cross(p, m + 1) : X;
            q = acc_q(p, m, E, L, R);
            L = R;
        } else {
            float S = lo(hi((X.y - E.y) * p.ystep, 0.0f), 1.0f);
            q = __float2int_rn(S * p.sign * kAccScale);
        }
        int dq = q - qprev;
        qprev = q;
        if (dq != 0 && m < W) {
            atomicAdd(row_acc + m, dq);
            x0 = min(x0, m);
            x1 = max(x1, m);
        }
    }
    return left;
}

// Accumulate pair (piece p, row k) for the warp owning chunks [cb, ce):
// the row's cells inside the warp's columns of that row, the chunk marks,
// and (first row only) what the columns left of the warp add.
__device__ __forceinline__ void raster_pair(const dda_piece &p, int k, int y0, int W, int cpr, int rA, int rB,
                                            int xa0, int xb1, int *acc, unsigned *cmask, int &carry) {
    int ly = dda_row_index(p, k) - y0;
    int xa = ly == rA ? xa0 : 0, xb = ly == rB ? xb1 : W;
    int x0 = 0x7fffffff, x1 = -1;
    int left = raster_row(p, k, acc + ly * W, W, xa, xb, x0, x1);
    if (ly == rA) carry += left;
    if (x0 <= x1) {
        int c0 = ly * cpr + (x0 >> 5), c1 = ly * cpr + (x1 >> 5);
        for (int w = c0 >> 5; w <= (c1 >> 5); ++w) {
            int lo_b = max(c0, w << 5) - (w << 5), hi_b = min(c1, (w << 5) + 31) - (w << 5);
            unsigned bits = (hi_b >= 31 ? 0xffffffffu : ((2u << hi_b) - 1u)) & ~((1u << lo_b) - 1u);
            atomicOr(cmask + w, bits);
        }
    }
}

// One warp's share of a draw over its own chunks [cb, ce) of the strip
// (row-major, cpr chunks of 32 pixels per row): the entries of the draw's
// bins whose bands overlap the warp's rows.  32 entries at a time, each lane
// prepares one segment and counts its rows inside the warp's rows; when no
// lane has more than one, each does its own, else the (segment, row) pairs
// are dealt out to the lanes (the prepared segment travels by shuffles).
// Each pair accumulates the row's cells inside the warp's columns of that
// row and marks the chunks it touched in cmask (one bit per chunk of the
// strip).  Returns, in every lane, what the columns left of the warp's first
// chunk add to its first row.
__device__ int raster_chunks(const strip_params &P, const strip_cmd &e, int W, int H, int y0, int cb, int ce,
                             int cpr, int *acc, unsigned *cmask, int lane) {
    const int band_h = e.band_h;
    const int rA = cb / cpr, rB = (ce - 1) / cpr;          // local rows of the range
    const int xa0 = (cb - rA * cpr) << 5;                  // first column of the first row
    const int xb1 = min(W, (ce - rB * cpr) << 5);          // end column of the last row
    const int ya = y0 + rA, yb = min(y0 + rB, H - 1);
    int carry = 0;
    if (ya > yb) return 0;
    const int b0 = ya / band_h, b1 = yb / band_h;
    const int64_t *off = P.bin_off + e.bin_base;
    const int64_t first = off[b0], last = off[b1 + 1];
    for (int64_t base = first; base < last; base += 32) {
        const int64_t ei = base + lane;
        int cnt = 0, klo = 0;
        dda_piece p;
        p.nrows = 0;
        if (ei < last) {
            const float4 sg = P.bin_seg[ei];
            int band = b0;
            while (band < b1 && ei >= off[band + 1]) ++band;
            // the warp's rows inside the entry's band, and inside the rows
            // the segment can touch, [floor(min y), ceil(max y)] (a cheap
            // test before the setup: most entries of a band lie in other
            // warps' rows)
            int ylo = max(ya, band * band_h), yhi = min(yb, (band + 1) * band_h - 1);
            ylo = max(ylo, static_cast<int>(floorf(fminf(sg.y, sg.w))));
            yhi = min(yhi, static_cast<int>(ceilf(fmaxf(sg.y, sg.w))));
            if (ylo <= yhi && dda_setup(f2(sg.x, sg.y), f2(sg.z, sg.w), p)) {
                int n = p.nrows < H + 2 ? p.nrows : H + 2;
                int py0 = static_cast<int>(p.py0);
                int k0 = p.up ? ylo - py0 : py0 - yhi;
                int k1 = p.up ? yhi - py0 : py0 - ylo;
                k0 = max(k0, 0);
                k1 = min(k1, n - 1);
                if (k0 <= k1) {
                    cnt = k1 - k0 + 1;
                    klo = k0;
                }
            }
        }
        if (__all_sync(0xffffffffu, cnt <= 1)) {
            if (cnt == 1) raster_pair(p, klo, y0, W, cpr, rA, rB, xa0, xb1, acc, cmask, carry);
            continue;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int first_k = klo - (incl - cnt);   // k of pair q is first_k + q for the owning lane
        const int vert = p.vert ? 1 : 0;
        for (int q0 = 0; q0 < total; q0 += 32) {
            const int q = q0 + lane;
            // the lane whose inclusive end first exceeds q owns pair q
            int lo_i = 0, hi_i = 31;
#pragma unroll
            for (int it = 0; it < 5; ++it) {
                int mid = (lo_i + hi_i) >> 1;
                int v = __shfl_sync(0xffffffffu, incl, mid);
                if (v > q) hi_i = mid; else lo_i = mid + 1;
            }
            const int src = lo_i;
            dda_piece r;
            r.fx = __shfl_sync(0xffffffffu, p.fx, src);
            r.fy = __shfl_sync(0xffffffffu, p.fy, src);
            r.tx = __shfl_sync(0xffffffffu, p.tx, src);
            r.ty = __shfl_sync(0xffffffffu, p.ty, src);
            r.sx = __shfl_sync(0xffffffffu, p.sx, src);
            r.sy = __shfl_sync(0xffffffffu, p.sy, src);
            r.sign = __shfl_sync(0xffffffffu, p.sign, src);
            r.ystep = __shfl_sync(0xffffffffu, p.ystep, src);
            r.px0 = __shfl_sync(0xffffffffu, p.px0, src);
            r.py0 = __shfl_sync(0xffffffffu, p.py0, src);
            r.vert = __shfl_sync(0xffffffffu, vert, src) != 0;
            r.up = r.ystep > 0.0f;
            r.nrows = 0;
            const int k = __shfl_sync(0xffffffffu, first_k, src) + q;
            if (q < total) raster_pair(r, k, y0, W, cpr, rA, rB, xa0, xb1, acc, cmask, carry);
        }
    }
    return static_cast<int>(__reduce_add_sync(0xffffffffu, static_cast<unsigned>(carry)));
}

// First marked chunk in [c, c_end), or c_end.
__device__ __forceinline__ int next_marked(const unsigned *cmask, int c, int c_end) {
    while (c < c_end) {
        unsigned w = cmask[c >> 5] & (0xffffffffu << (c & 31));
        if (w) {
            int f = ((c >> 5) << 5) + __ffs(w) - 1;
            return f < c_end ? f : c_end;
        }
        c = ((c >> 5) + 1) << 5;
    }
    return c_end;
}

// BINNED selects the coverage of draws: false walks the row-sorted runs
// (the float canvas is then the reference's bit for bit); true has each
// warp accumulate the draw's binned segments over its own chunks of the
// strip in shared memory (raster_chunks), then prefix-sum its rows with
// shuffles while it paints.  A warp only ever touches its own chunks, so no
// barrier is needed between draws.  Shared memory: the strip's float4
// pixels, and for BINNED an int32 accumulation image of the strip and one
// bit per chunk.
template <int THREADS, bool BINNED>
__global__ void __launch_bounds__(THREADS, BINNED ? 512 / THREADS : 1) k_strips(strip_params P) {
    extern __shared__ float4 px[];
    __shared__ int item_slot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int *acc = BINNED ? reinterpret_cast<int *>(px + P.strip_pixels) : nullptr;
    unsigned *cmask = BINNED ? reinterpret_cast<unsigned *>(acc + P.strip_pixels) : nullptr;
    if (BINNED) {   // zero once: each draw's paint clears what its raster wrote
        for (int i = threadIdx.x; i < P.strip_pixels; i += blockDim.x) acc[i] = 0;
        for (int i = threadIdx.x; i < P.strip_words; i += blockDim.x) cmask[i] = 0;
    }
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) item_slot = atomicAdd(P.counter, 1);
        __syncthreads();
        int it = item_slot;
        if (it >= P.n_items) break;
        int2 item = P.items[it];
        const strip_canvas cv = P.canvases[item.x];
        const int W = cv.W, y0 = item.y;
        const int rows = min(cv.TH, cv.H - y0);
        const int cpr = (W + 31) >> 5;           // 32-pixel chunks per row
        const int chunks = rows * cpr;
        // Each warp owns a contiguous range of chunks (row-major) for the
        // whole item, so every pixel is always touched by the same thread.
        // Binned: whole rows per warp when the rows divide evenly enough, so
        // no two warps walk the same segment rows.
        int per = (chunks + nwarps - 1) / nwarps;
        if (BINNED && rows >= nwarps && (rows % nwarps == 0 || rows >= 4 * nwarps))
            per = ((rows + nwarps - 1) / nwarps) * cpr;
        const int cb = min(chunks, warp * per), ce = min(chunks, cb + per);
        for (int ch = cb; ch < ce; ++ch) {
            int ly = ch / cpr, x = ((ch - ly * cpr) << 5) + lane;
            if (x >= W) continue;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (cv.flags & 1) v = cv.bitmap[static_cast<size_t>(y0 + ly) * W + x];
            px[ly * W + x] = v;
        }
        // Canvas rows this warp's chunks span: draws wholly above or below
        // them are skipped by the warp (the fixed chunk ownership needs no
        // agreement between warps).
        const int wy0 = y0 + (cb < ce ? cb / cpr : 0), wy1 = y0 + (cb < ce ? (ce - 1) / cpr : -1);
        for (int ci = cv.cmd_first; ci < cv.cmd_first + cv.cmd_count; ++ci) {
            const command &c = P.cmds[ci];
            const strip_cmd &e = P.ext[ci];
            if (c.kind == CMD_CLIP) continue;
            if (c.kind == CMD_PUT) {
                for (int ch = cb; ch < ce; ++ch) {
                    int ly = ch / cpr, x = ((ch - ly * cpr) << 5) + lane;
                    int y = y0 + ly;
                    int ix = x - c.put_x, iy = y - c.put_y;
                    if (x >= W || ix < 0 || ix >= c.put_w || iy < 0 || iy >= c.put_h) continue;
                    const uint8_t *p = P.put_px + c.put_first + (static_cast<size_t>(iy) * c.put_w + ix) * 4;
                    float a = static_cast<float>(p[3]) / 255.0f;
                    px[ly * W + x] = make_float4(P.lut[p[0]] * a, P.lut[p[1]] * a, P.lut[p[2]] * a, a);
                }
                continue;
            }
            if (c.kind == CMD_GET) {
                for (int ch = cb; ch < ce; ++ch) {
                    int ly = ch / cpr, x = ((ch - ly * cpr) << 5) + lane;
                    int y = y0 + ly;
                    int ix = x - e.get_x, iy = y - e.get_y;
                    if (x >= W || ix < 0 || ix >= e.get_w || iy < 0 || iy >= e.get_h) continue;
                    uchar4 o = to_srgb8(px[ly * W + x], x, y);
                    reinterpret_cast<uchar4 *>(P.get_buf + e.get_out)[static_cast<size_t>(iy) * e.get_w + ix] = o;
                }
                continue;
            }
            const int op = c.op;
            const bool clearing = !(op & 8);
            if (e.has_shadow) {
                // render_shadow's composite (hpp:2504-2538)
                const shadow_rect r = P.rects[ci];
                const float *img = P.shadow_imgs + e.shadow_img;
                int b = c.sh_border;
                int sx0 = max(0, r.left - b), sx1 = min(W, r.right - b);
                if (r.width > 0 && r.height > 0 && r.top - b <= wy1 && r.bottom - b - 1 >= wy0) {
                    for (int ch = cb; ch < ce; ++ch) {
                        int ly = ch / cpr, x = ((ch - ly * cpr) << 5) + lane;
                        int y = y0 + ly;
                        if (x < sx0 || x >= sx1 || y + b < r.top || y + b >= r.bottom) continue;
                        float vis = e.vis ? e.vis[static_cast<size_t>(y) * W + x] : 1.0f;
                        if (vis < kVisible) continue;
                        float s = img[static_cast<size_t>(y + b - r.top) * r.width + (x + b - r.left)];
                        float k = c.alpha * s;
                        float4 fore = make_float4(c.sh_color[0] * k, c.sh_color[1] * k, c.sh_color[2] * k,
                                                  c.sh_color[3] * k);
                        px[ly * W + x] = blend(px[ly * W + x], fore, op, vis);
                    }
                }
            }
            if (BINNED) {
                if (cb >= ce || (!clearing && (c.gy1 < wy0 || c.gy0 > wy1))) continue;
                // the draw's fields every pixel needs, read once
                const int rule = c.fill_rule, paint = c.paint;
                const float alpha = c.alpha;
                const float4 solid = make_float4(c.color[0], c.color[1], c.color[2], c.color[3]);
                const float *vis_plane = e.vis;
                const int carry0 = raster_chunks(P, e, W, cv.H, y0, cb, ce, cpr, acc, cmask, lane);
                __syncwarp();
                const int rA = cb / cpr, rB = (ce - 1) / cpr;
                for (int ly = rA; ly <= rB; ++ly) {
                    const int row0 = ly * cpr, y = y0 + ly;
                    const int c_hi = min(ce, row0 + cpr);
                    int ch = max(cb, row0);
                    int carry = ly == rA ? carry0 : 0;
                    int *arow = acc + ly * W;
                    while (ch < c_hi) {
                        const bool marked = (cmask[ch >> 5] >> (ch & 31)) & 1u;
                        if (!marked && !clearing && cover_of(static_cast<float>(carry) * kAccInv, rule) < kVisible) {
                            // no area here and the sum so far is invisible:
                            // on to the next chunk that holds area
                            ch = next_marked(cmask, ch + 1, c_hi);
                            continue;
                        }
                        const int x = ((ch - row0) << 5) + lane;
                        int v = 0;
                        if (marked) {
                            if (x < W) {
                                v = arow[x];
                                if (v) arow[x] = 0;
                            }
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1) {
                                int t = __shfl_up_sync(0xffffffffu, v, o);
                                if (lane >= o) v += t;
                            }
                        }
                        const int sum = carry + v;
                        if (marked) carry = __shfl_sync(0xffffffffu, sum, 31);
                        ++ch;
                        if (x >= W) continue;
                        float cov = cover_of(static_cast<float>(sum) * kAccInv, rule);
                        float vis = vis_plane ? vis_plane[static_cast<size_t>(y) * W + x] : 1.0f;
                        if ((cov >= kVisible || clearing) && vis >= kVisible) {
                            // paint_pixel (hpp:2265-2377); a solid colour is the brush's own
                            float4 pp = paint == 1 ? solid
                                      : paint_at(c, P.src, static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f);
                            float kk = cov * alpha;
                            float4 fore = make_float4(pp.x * kk, pp.y * kk, pp.z * kk, pp.w * kk);
                            px[ly * W + x] = blend(px[ly * W + x], fore, op, vis);
                        }
                    }
                }
                // clear the marks of the warp's chunks (other warps' bits in
                // the same words are left alone)
                __syncwarp();
                for (int w = (cb >> 5) + lane; w <= ((ce - 1) >> 5); w += 32) {
                    int lo_b = max(cb, w << 5) - (w << 5), hi_b = min(ce - 1, (w << 5) + 31) - (w << 5);
                    unsigned bits = (hi_b >= 31 ? 0xffffffffu : ((2u << hi_b) - 1u)) & ~((1u << lo_b) - 1u);
                    atomicAnd(cmask + w, ~bits);
                }
                __syncwarp();
                continue;
            }
            // Rows [gy0, gy1] hold all of the draw's runs; elsewhere only a
            // clearing operation changes pixels.
            if (!clearing && (c.gy1 < wy0 || c.gy0 > wy1)) continue;
            // render_main (hpp:2551-2605).  Walk each row's sorted runs with a
            // warp-wide cursor: the coverage sum in force at a pixel is the
            // running sum after the last run at or left of it.
            // Rows of the warp's chunk range; in each, only the chunks from
            // the first run to the last (all of them for clearing ops).
            const int ly_first = cb / cpr, ly_last = cb < ce ? (ce - 1) / cpr : -1;
            for (int ly = ly_first; ly <= ly_last; ++ly) {
                int n, first_x, last_x, next_x, j = 0;
                const run *r;
                const float *sm;
                float carry = 0.0f;
                {
                    int row = e.main_row_base + y0 + ly;
                    int4 mt = P.rv.meta[row];   // with the offset: one round trip per row
                    long long off = P.rv.row_off[row];
                    n = mt.w;
                    r = P.rv.runs + off;
                    sm = P.rv.sums + off;
                    first_x = mt.x;
                    next_x = first_x;   // x of run j, the first one not yet in `carry`
                    // Past the last run the row's final sum still paints
                    // up to the clip's end when it is visible (see k_paint).
                    last_x = n ? (cover_of(__int_as_float(mt.z), c.fill_rule) >= kVisible ? W - 1 : mt.y) : -1;
                }
                const int xs = clearing ? 0 : first_x;
                const int xe = clearing ? W - 1 : min(last_x, W - 1);
                if (xs > xe) continue;
                const int row0 = ly * cpr;
                const int c_hi = min(ce, row0 + (xe >> 5) + 1);
                for (int ch = max(cb, row0 + (xs >> 5)); ch < c_hi; ++ch) {
                const int x0 = (ch - row0) << 5;
                float v;
                if (next_x >= x0 + 32) {
                    // No pending run reaches this chunk: every pixel takes
                    // the carried sum.
                    v = carry;
                    if (!clearing && cover_of(carry, c.fill_rule) < kVisible) {
                        // Nothing visible up to the next run: jump to the
                        // chunk that holds it (or past this row).
                        int target = (next_x < W && next_x <= xe) ? row0 + (next_x >> 5) : c_hi;
                        if (target > ch + 1) ch = min(target, c_hi) - 1;
                        continue;
                    }
                } else {
                    // Consume the runs left of this chunk (they only set the carry).
                    int rx = 0x7fffffff;
                    float rs = 0.0f;
                    for (;;) {
                        int idx = j + lane;
                        rx = idx < n ? r[idx].x : 0x7fffffff;
                        rs = idx < n ? sm[idx] : 0.0f;
                        unsigned below = __ballot_sync(0xffffffffu, rx < x0);
                        int nb = __popc(below);
                        if (nb > 0) carry = __shfl_sync(0xffffffffu, rs, nb - 1);
                        j += nb;
                        if (nb < 32) {
                            if (nb > 0) {   // realign the window at the new cursor
                                rx = __shfl_down_sync(0xffffffffu, rx, nb);
                                rs = __shfl_down_sync(0xffffffffu, rs, nb);
                                if (lane + nb >= 32) {
                                    int k2 = j + lane;
                                    rx = k2 < n ? r[k2].x : 0x7fffffff;
                                    rs = k2 < n ? sm[k2] : 0.0f;
                                }
                            }
                            break;
                        }
                    }
                    // Runs inside the chunk: at most 32, one per distinct x.
                    bool in_chunk = rx < x0 + 32;
                    unsigned pos_mask = __reduce_or_sync(0xffffffffu, in_chunk ? (1u << (rx - x0)) : 0u);
                    int k = __popc(__ballot_sync(0xffffffffu, in_chunk));
                    unsigned upto = pos_mask & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u));
                    v = carry;
                    int src = upto ? __popc(upto) - 1 : 0;
                    float from_run = __shfl_sync(0xffffffffu, rs, src);
                    if (upto) v = from_run;
                    if (k > 0) carry = __shfl_sync(0xffffffffu, rs, k - 1);
                    j += k;
                    next_x = k < 32 ? __shfl_sync(0xffffffffu, rx, k) : (j < n ? r[j].x : 0x7fffffff);
                    if (!clearing && k == 0 && cover_of(carry, c.fill_rule) < kVisible) {
                        int target = (next_x < W && next_x <= xe) ? row0 + (next_x >> 5) : c_hi;
                        if (target > ch + 1) ch = min(target, c_hi) - 1;
                        continue;
                    }
                }
                int x = x0 + lane;
                if (x < xs || x > xe) continue;
                int y = y0 + ly;
                float cov = cover_of(v, c.fill_rule);
                float vis = e.vis ? e.vis[static_cast<size_t>(y) * W + x] : 1.0f;
                if ((cov >= kVisible || clearing) && vis >= kVisible) {
                    float4 p = paint_at(c, P.src, static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f);
                    float kk = cov * c.alpha;
                    float4 fore = make_float4(p.x * kk, p.y * kk, p.z * kk, p.w * kk);
                    px[ly * W + x] = blend(px[ly * W + x], fore, op, vis);
                }
                }
            }
        }
        if (cv.flags & 2) {
            for (int ch = cb; ch < ce; ++ch) {
                int ly = ch / cpr, x = ((ch - ly * cpr) << 5) + lane;
                if (x >= W) continue;
                cv.bitmap[static_cast<size_t>(y0 + ly) * W + x] = px[ly * W + x];
            }
        }
    }
}

// ------------------------------------------------ frame-wide shadow passes
// All shadows of a frame are prepared before the strip kernel: working
// rectangle, alpha raster and blur of every shadowed draw, batched.
struct shadow_job {
    int32_t cmd;            // command index
    int32_t job;            // scan job (padded canvas) index
    int32_t row_base;       // its first row in the shared row arrays
    int32_t W, H, border;   // canvas size and border
    int64_t img;            // float offset of its image (and of its scratch)
    int32_t radius;
    float w1, w2;
    int32_t pad;
};

__global__ void k_shadow_rects(const shadow_job *sj, int n, const cover_box *boxes, shadow_rect *rects) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const shadow_job &s = sj[i];
    int ext_w = s.W + 2 * s.border, ext_h = s.H + 2 * s.border;
    int left = ext_w, right = 0, top = ext_h, bottom = 0;
    cover_box b = boxes[s.job];
    if (b.x0 <= b.x1) {
        left = min(left, b.x0); right = max(right, b.x1);
        top = min(top, b.y0); bottom = max(bottom, b.y1);
    }
    if (b.first_key != 0x7fffffffffffffffll) {
        int fx = static_cast<int>(b.first_key & 0xffffffffll), fy = static_cast<int>(b.first_key >> 32);
        left = min(left, fx); right = max(right, fx);
        top = min(top, fy); bottom = max(bottom, fy);
    }
    left = max(left - s.border, 0);
    right = min(right + s.border, ext_w) + 1;
    top = max(top - s.border, 0);
    bottom = min(bottom + s.border, ext_h);
    shadow_rect r;
    r.left = left; r.right = right; r.top = top; r.bottom = bottom;
    r.width = max(right - left, 0);
    r.height = max(bottom - top, 0);
    rects[s.cmd] = r;
}

// Raster: blockIdx.y selects the shadow, warps cover its working rows.
__global__ void k_shadow_raster_all(const shadow_job *sj, const command *cmds, paint_src src, row_view rv,
                                    const shadow_rect *rects, float *imgs) {
    const shadow_job &s = sj[blockIdx.y];
    const command &c = cmds[s.cmd];
    const shadow_rect rc = rects[s.cmd];
    int lane = threadIdx.x & 31;
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    float *out = imgs + s.img;
    for (int y = rc.top + wid; y < rc.bottom; y += nw) {
        int row = s.row_base + y;
        int n = rv.row_len[row];
        const run *r = rv.runs + rv.row_off[row];
        const float *sm = rv.sums + rv.row_off[row];
        int first = n ? r[0].x : 0x7fffffff, last = n ? r[n - 1].x : -1;
        for (int x = rc.left + lane; x < rc.right; x += 32) {
            float val = 0.0f;
            if (x >= first && x <= last) {
                float cov = cover_of(sum_at(r, sm, n, x), c.fill_rule);
                if (cov >= kVisible) {
                    float pxx = (static_cast<float>(x) + 0.5f) - c.sh_offx;
                    float pyy = (static_cast<float>(y) + 0.5f) - c.sh_offy;
                    val = cov * paint_at(c, src, pxx, pyy).w;
                }
            }
            // Column-major, so the row blur below reads with unit stride across threads.
            out[static_cast<size_t>(x - rc.left) * rc.height + (y - rc.top)] = val;
        }
    }
}

// Exact running-sum blur (hpp:2453-2503), rows then columns, batched over
// shadows through blockIdx.y, one thread per row (then per column) running
// the reference's sequential sums.  The row pass works on the column-major
// raster, the image is then transposed, and the column pass works row-major,
// so neighbouring threads always touch neighbouring addresses.
//
// The three passes of a line run as one sweep: pass k produces its value at
// x once its input is known up to x + r + 1, so after reading element t the
// passes emit x = t - (r+1), t - 2(r+1), t - 3(r+1).  Each pass keeps its
// input window [x - r - 2, x + r + 1] in a 32-entry ring; the additions are
// the reference's, in its order, so the result is the same as three full
// passes.  Output lags input, so the line is blurred in place.
static constexpr int kBlurRing = 32;
static constexpr int kBlurMaxFused = (kBlurRing - 4) / 2;   // radius the rings hold

struct blur_pass {
    float acc;
    float ring[kBlurRing];
};

// Value of one pass at x (0 <= x < n) from its input ring (hpp:2461-2478).
__device__ __forceinline__ float blur_step(blur_pass &p, int x, int n, int r, float w1, float w2) {
    const int m = kBlurRing - 1;
    if (x == 0) {
        float acc = r + 1 < n ? w1 * p.ring[(r + 1) & m] : 0.0f;
        for (int i = 0; i <= r && i < n; ++i) acc += (w1 + w2) * p.ring[i & m];
        p.acc = acc;
        return acc;
    }
    float acc = p.acc;
    if (x >= r + 1) acc -= w2 * p.ring[(x - r - 1) & m];
    if (x >= r + 2) acc -= w1 * p.ring[(x - r - 2) & m];
    if (x + r < n) acc += w2 * p.ring[(x + r) & m];
    if (x + r + 1 < n) acc += w1 * p.ring[(x + r + 1) & m];
    p.acc = acc;
    return acc;
}

// Three blur passes over line[i * stride], i < n, in place.  Input values
// are fetched kPrefetch steps ahead so a thread keeps several loads in
// flight (a line's recurrence is sequential; its loads are not).
static constexpr int kPrefetch = 8;

__device__ void blur_line_fused(float *line, size_t stride, int n, int r, float w1, float w2) {
    const int m = kBlurRing - 1, L = r + 1;
    blur_pass p[3];
    const int steps = n + 3 * L;
    for (int t0 = 0; t0 < steps; t0 += kPrefetch) {
        float in[kPrefetch];
#pragma unroll
        for (int k = 0; k < kPrefetch; ++k) {
            int t = t0 + k;
            in[k] = t < n ? line[static_cast<size_t>(t) * stride] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < kPrefetch; ++k) {
            int t = t0 + k;
            if (t >= steps) break;
            if (t < n) p[0].ring[t & m] = in[k];
            int x1 = t - L, x2 = t - 2 * L, x3 = t - 3 * L;
            if (x1 >= 0 && x1 < n) p[1].ring[x1 & m] = blur_step(p[0], x1, n, r, w1, w2);
            if (x2 >= 0 && x2 < n) p[2].ring[x2 & m] = blur_step(p[1], x2, n, r, w1, w2);
            if (x3 >= 0 && x3 < n) line[static_cast<size_t>(x3) * stride] = blur_step(p[2], x3, n, r, w1, w2);
        }
    }
}

// Radius known at compile time: the three rings live in registers (every
// ring index is a constant once a block of RING steps is unrolled).  RING is
// exactly the size of a pass's window [x - R - 2, x + R + 1]: 2R + 4.
template <int RING>
__device__ __forceinline__ constexpr int ring_at(int v) { return ((v % RING) + RING) % RING; }

template <int R, int RING>
__device__ __forceinline__ float blur_step_reg(const float (&ring)[RING], float &acc, int x, int n, float w1,
                                               float w2, int k) {
    // k is the step's position in the unrolled block; x % RING == k % RING.
    if (x == 0) {
        float a = R + 1 < n ? w1 * ring[ring_at<RING>(k + R + 1)] : 0.0f;
#pragma unroll
        for (int i = 0; i <= R; ++i)
            if (i < n) a += (w1 + w2) * ring[ring_at<RING>(k + i)];
        acc = a;
        return a;
    }
    float a = acc;
    if (x >= R + 1) a -= w2 * ring[ring_at<RING>(k - R - 1)];
    if (x >= R + 2) a -= w1 * ring[ring_at<RING>(k - R - 2)];
    if (x + R < n) a += w2 * ring[ring_at<RING>(k + R)];
    if (x + R + 1 < n) a += w1 * ring[ring_at<RING>(k + R + 1)];
    acc = a;
    return a;
}

template <int R>
__device__ void blur_line_reg(float *line, size_t stride, int n, float w1, float w2) {
    constexpr int RING = 2 * R + 4;
    constexpr int L = R + 1;
    float r0[RING], r1[RING], r2[RING];
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    const int steps = n + 3 * L;
    for (int t0 = 0; t0 < steps; t0 += RING) {
        float in[RING];
#pragma unroll
        for (int k = 0; k < RING; ++k) {
            int t = t0 + k;
            in[k] = t < n ? line[static_cast<size_t>(t) * stride] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < RING; ++k) {
            int t = t0 + k;
            if (t < n) r0[k] = in[k];
            int x1 = t - L, x2 = t - 2 * L, x3 = t - 3 * L;
            if (x1 >= 0 && x1 < n) r1[ring_at<RING>(k - L)] = blur_step_reg<R, RING>(r0, a0, x1, n, w1, w2, k - L);
            if (x2 >= 0 && x2 < n)
                r2[ring_at<RING>(k - 2 * L)] = blur_step_reg<R, RING>(r1, a1, x2, n, w1, w2, k - 2 * L);
            if (x3 >= 0 && x3 < n)
                line[static_cast<size_t>(x3) * stride] = blur_step_reg<R, RING>(r2, a2, x3, n, w1, w2, k - 3 * L);
        }
    }
}

// The same three passes with a full copy of the line per pass (any radius).
__device__ void blur_line_copy(float *line, float *tmp, size_t stride, size_t n, size_t r, float w1, float w2) {
    for (int pass = 0; pass < 3; ++pass) {
        for (size_t x = 0; x < n; ++x) tmp[x * stride] = line[x * stride];
        float acc = r + 1 < n ? w1 * tmp[(r + 1) * stride] : 0.0f;
        for (size_t x = 0; x <= r && x < n; ++x) acc += (w1 + w2) * tmp[x * stride];
        if (n > 0) line[0] = acc;
        for (size_t x = 1; x < n; ++x) {
            if (x >= r + 1) acc -= w2 * tmp[(x - r - 1) * stride];
            if (x >= r + 2) acc -= w1 * tmp[(x - r - 2) * stride];
            if (x + r < n) acc += w2 * tmp[(x + r) * stride];
            if (x + r + 1 < n) acc += w1 * tmp[(x + r + 1) * stride];
            line[x * stride] = acc;
        }
    }
}

// Three passes over one line: registers for radius 0..7, local rings up to
// kBlurMaxFused, else full copies.
__device__ void blur_line(float *line, float *tmp, size_t stride, int n, int r, float w1, float w2) {
    switch (r) {
    case 0: blur_line_reg<0>(line, stride, n, w1, w2); return;
    case 1: blur_line_reg<1>(line, stride, n, w1, w2); return;
    case 2: blur_line_reg<2>(line, stride, n, w1, w2); return;
    case 3: blur_line_reg<3>(line, stride, n, w1, w2); return;
    case 4: blur_line_reg<4>(line, stride, n, w1, w2); return;
    case 5: blur_line_reg<5>(line, stride, n, w1, w2); return;
    case 6: blur_line_reg<6>(line, stride, n, w1, w2); return;
    case 7: blur_line_reg<7>(line, stride, n, w1, w2); return;
    default: break;
    }
    if (r <= kBlurMaxFused) blur_line_fused(line, stride, n, r, w1, w2);
    else blur_line_copy(line, tmp, stride, n, r, w1, w2);
}

__global__ void k_blur_rows_all(const shadow_job *sj, const shadow_rect *rects, float *imgs, float *scratch) {
    const shadow_job &s = sj[blockIdx.y];
    const shadow_rect rc = rects[s.cmd];
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= rc.height) return;
    blur_line(imgs + s.img + y, scratch + s.img + y, rc.height, rc.width, s.radius, s.w1, s.w2);
}

// Column-major -> row-major, 32x32 tiles (blockIdx.z selects the shadow).
__global__ void k_transpose_all(const shadow_job *sj, const shadow_rect *rects, const float *in, float *out) {
    __shared__ float tile[32][33];
    const shadow_job &s = sj[blockIdx.z];
    const shadow_rect rc = rects[s.cmd];
    int h = rc.height, w = rc.width;
    int tx = blockIdx.x * 32, ty = blockIdx.y * 32;
    if (tx >= w || ty >= h) return;
    const float *src = in + s.img;
    float *dst = out + s.img;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int x = tx + i, y = ty + threadIdx.x;
        if (x < w && y < h) tile[i][threadIdx.x] = src[static_cast<size_t>(x) * h + y];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int y = ty + i, x = tx + threadIdx.x;
        if (x < w && y < h) dst[static_cast<size_t>(y) * w + x] = tile[threadIdx.x][i];
    }
}

__global__ void k_blur_cols_all(const shadow_job *sj, const shadow_rect *rects, float *imgs, float *scratch) {
    const shadow_job &s = sj[blockIdx.y];
    const shadow_rect rc = rects[s.cmd];
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= rc.width) return;
    blur_line(imgs + s.img + x, scratch + s.img + x, rc.width, rc.height, s.radius, s.w1, s.w2);
}

}  // namespace cyg

#endif
