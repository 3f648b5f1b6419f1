// kernels.cuh -- CUDA kernels of the per-canvas ("plain") render path.
//
// The reference renders sparsely: sorted per-pixel signed-area runs are
// walked row by row with float running sums.  Rows are independent, so each
// step here is row-parallel and reproduces the reference's per-row float
// operation order: runs are bucketed per row, each row is sorted, coalesced
// and prefix-summed by one thread, and the pixels of the row are then
// painted and composited in parallel by a warp carrying the row's running
// sums forward.  Shadows, clip masks and the blur follow the same rule.
// Fills and clips of Bezier paths are flattened on the GPU first, for the
// whole flush at once.
#ifndef CY_KERNELS_CUH
#define CY_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"
#include "flatten.cuh"
#include "hit.cuh"
#include "pack.cuh"

namespace cyg {

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ int warp_id_global() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int warps_total() { return (gridDim.x * blockDim.x) >> 5; }

__device__ __forceinline__ long long warp_inclusive_scan(long long v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// --------------------------------------------------------------- patterns
// set_pattern / draw_image texels: premultiplied(linearized(rgba8 / 255))
// (hpp:2841-2864).  `lut` holds linearized(i / 255) computed on the host.
__global__ void k_pattern_prep(const uchar4 *__restrict__ src, float4 *__restrict__ dst, int n,
                               const float *__restrict__ lut) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uchar4 c = src[i];
    float a = static_cast<float>(c.w) / 255.0f;
    dst[i] = make_float4(lut[c.x] * a, lut[c.y] * a, lut[c.z] * a, a);
}

// ------------------------------------------------------------------- scan
// Exclusive scan of int32 in tiles of 4096 (1024 threads x 4).
__global__ void k_scan_tiles(const int32_t *__restrict__ in, int32_t *__restrict__ out, int n,
                             int32_t *__restrict__ tile_sums) {
    __shared__ int32_t warp_sums[32];
    int base = blockIdx.x * 4096 + threadIdx.x * 4;
    int32_t v[4];
    int32_t local = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        v[j] = base + j < n ? in[base + j] : 0;
        local += v[j];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
        int32_t s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    int32_t run = incl - local + (w > 0 ? warp_sums[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 1023 && tile_sums) tile_sums[blockIdx.x] = warp_sums[31];
}

__global__ void k_scan_add(int32_t *__restrict__ out, int n, const int32_t *__restrict__ tile_offs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] += tile_offs[i >> 12];
}

// Exclusive scan of int32 counts into int64 offsets, tiles of 4096.
template <class In>
__global__ void k_scan_tiles64(const In *__restrict__ in, int64_t *__restrict__ out, int n,
                               int64_t *__restrict__ tile_sums) {
    __shared__ long long warp_sums[32];
    int base = blockIdx.x * 4096 + threadIdx.x * 4;
    long long v[4];
    long long local = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        v[j] = base + j < n ? static_cast<long long>(in[base + j]) : 0;
        local += v[j];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
        long long s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    long long run = incl - local + (w > 0 ? warp_sums[w - 1] : 0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 1023 && tile_sums) tile_sums[blockIdx.x] = warp_sums[31];
}

__global__ void k_scan_add64(int64_t *__restrict__ out, int n, const int64_t *__restrict__ tile_offs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] += tile_offs[i >> 12];
}

// ------------------------------------------------------- scan conversion
// lines_to_runs (hpp:2193-2253), row-parallel.  Every queued scan
// conversion (a draw, its shadow, a clip) is a "job".  A job whose points can
// leave its rectangle first goes through the reference's Sutherland-Hodgman
// clip (four passes, each a count, a scan and an emit over all points of all
// such jobs); jobs that stay inside are scanned straight from their
// polylines, which the clip would return unchanged.  Then pass 1 counts the
// cells each segment touches in each job row (one atomic per segment row);
// pass 2 reserves that many slots in the row's bucket and writes the cells'
// signed-area changes (zeros included, dropped later).  Then every row of
// every job is sorted, coalesced and prefix-summed independently.
struct scan_job {
    int32_t geom;          // 0: host polylines, 1: GPU-flattened polylines
    int32_t line_first;    // first polyline point
    int32_t seg_count;     // polyline points (= segments, each closing on its predecessor)
    int32_t clip;          // 1: points may leave [0,width] x [0,height] (runs jobs only)
    int32_t row_base;      // first row of this job in the shared row arrays
    int32_t rows, cols;    // rows and cells per row of the (padded) canvas
    float width, height;   // clip rectangle [0,width] x [0,height]
    float offx, offy;      // added to every point first (shadow offset)
    int32_t need_box;      // 1: track the exact bounds of nonzero cells
    int32_t binned;        // 1: segments go to row-band bins (k_bin) instead of runs
    int32_t bin_base;      // binned: first bin of this job
    int32_t band_h;        // binned: rows per band
};

// Segment ranges of a list of jobs: entry i = (first segment, job index),
// sorted by first segment.
__device__ __forceinline__ int table_find(const int2 *tab, int n, int s) {
    int lo_i = 0, hi_i = n;   // last entry with first <= s
    while (hi_i - lo_i > 1) {
        int mid = (lo_i + hi_i) >> 1;
        if (tab[mid].x <= s) lo_i = mid; else hi_i = mid;
    }
    return lo_i;
}

// One polygon point of a clip pass: the segment ending at it, its job, and
// whether it starts its polygon (then `last` is the polygon's last point).
struct poly_point {
    float2 from, to;
    int job;
    bool start;
    int last;
};

struct clip_pass {
    // pass 0 reads the polylines of the clipped jobs
    const scan_job *jobs;
    const int2 *tab;           // clipped jobs: (first input point, job)
    int n_tab;
    const float2 *src_pts[2];
    const int32_t *src_prev[2];
    // passes 1-3 read the previous pass's polygons
    const float2 *in_pts;
    const int32_t *in_prev, *in_job;
    int n;                     // input points
    int edge;                  // 0: x >= 0, 1: y >= 0, 2: x <= width, 3: y <= height
    int32_t *cnt;              // per input point: points emitted (n + 1 entries)
    const int32_t *off;        // exclusive scan of cnt
    float2 *out_pts;
    int32_t *out_prev, *out_job;
};

template <bool FIRST>
__device__ __forceinline__ poly_point clip_point(const clip_pass &P, int k) {
    poly_point q;
    if (FIRST) {
        int c = table_find(P.tab, P.n_tab, k);
        const scan_job &j = P.jobs[P.tab[c].y];
        // a select, not an index into the parameter arrays: an index would
        // copy them to local memory
        const float2 *pts = j.geom ? P.src_pts[1] : P.src_pts[0];
        const int32_t *prev = j.geom ? P.src_prev[1] : P.src_prev[0];
        int i = j.line_first + (k - P.tab[c].x);
        int pi = prev[i];
        float2 a = pts[pi], b = pts[i];
        q.from = f2(j.offx + a.x, j.offy + a.y);   // scan's add(offset, point) (hpp:2205)
        q.to = f2(j.offx + b.x, j.offy + b.y);
        q.job = P.tab[c].y;
        q.start = pi >= i;
        q.last = k + (pi - i);
    } else {
        int pk = P.in_prev[k];
        q.from = P.in_pts[pk];
        q.to = P.in_pts[k];
        q.job = P.in_job[k];
        q.start = pk >= k;
        q.last = pk;
    }
    if (q.last >= P.n) q.last = P.n - 1;
    return q;
}

// Signed distances of the segment's ends from clip edge `edge` of the job,
// as the reference computes them: dot(point, normal) + place (hpp:2209-2218).
__device__ __forceinline__ void edge_sides(const clip_pass &P, const poly_point &q, float &fs, float &ts) {
    const scan_job &j = P.jobs[q.job];
    float nx = P.edge == 0 ? 1.0f : P.edge == 2 ? -1.0f : 0.0f;
    float ny = P.edge == 1 ? 1.0f : P.edge == 3 ? -1.0f : 0.0f;
    float place = P.edge == 2 ? j.width : P.edge == 3 ? j.height : 0.0f;
    fs = (q.from.x * nx + q.from.y * ny) + place;
    ts = (q.to.x * nx + q.to.y * ny) + place;
}

template <bool FIRST>
__global__ void k_clip_count(clip_pass P) {
    int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= P.n; k += stride) {
        if (k == P.n) { P.cnt[k] = 0; continue; }
        poly_point q = clip_point<FIRST>(P, k);
        float fs, ts;
        edge_sides(P, q, fs, ts);
        P.cnt[k] = (fs * ts < 0.0f ? 1 : 0) + (ts >= 0.0f ? 1 : 0);
    }
}

// Emit a pass's polygon points: the crossing with the edge, then the end
// point if it is inside (hpp:2213-2216).  Each point links to the one before
// it; k_clip_link then closes every polygon.
template <bool FIRST>
__global__ void k_clip_emit(clip_pass P) {
    int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += stride) {
        poly_point q = clip_point<FIRST>(P, k);
        float fs, ts;
        edge_sides(P, q, fs, ts);
        int o = P.off[k];
        if (fs * ts < 0.0f) {
            P.out_pts[o] = mix2(q.from, q.to, fs / (fs - ts));
            P.out_prev[o] = o - 1;
            P.out_job[o] = q.job;
            ++o;
        }
        if (ts >= 0.0f) {
            P.out_pts[o] = q.to;
            P.out_prev[o] = o - 1;
            P.out_job[o] = q.job;
        }
    }
}

// The first emitted point of each polygon closes on its last one.
template <bool FIRST>
__global__ void k_clip_link(clip_pass P) {
    int stride = gridDim.x * blockDim.x;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += stride) {
        bool start;
        int last;
        if (FIRST) {
            int c = table_find(P.tab, P.n_tab, k);
            const scan_job &j = P.jobs[P.tab[c].y];
            int i = j.line_first + (k - P.tab[c].x);
            int pi = (j.geom ? P.src_prev[1] : P.src_prev[0])[i];
            start = pi >= i;
            last = k + (pi - i);
        } else {
            int pk = P.in_prev[k];
            start = pk >= k;
            last = pk;
        }
        if (!start) continue;
        if (last >= P.n) last = P.n - 1;
        int first_out = P.off[k], end_out = P.off[last + 1];
        if (end_out > first_out) P.out_prev[first_out] = end_out - 1;
    }
}

struct job_tables {
    const scan_job *jobs;
    // unclipped jobs: segments straight from the polylines
    const int2 *tab;          // (first segment, job)
    int n_tab;
    const int32_t *tab_idx;   // or null: entry holding segment b << kTabShift, b = 0 .. last + 1
    const float2 *pts[2];
    const int32_t *prev[2];
    // clipped jobs: the last clip pass's polygons (offset already applied)
    const float2 *cl_pts;
    const int32_t *cl_prev, *cl_job;
    cover_box *boxes;       // one per job
    int32_t *row_cnt;       // count pass: cells per row (all jobs)
    const int64_t *row_off; // emit pass: bucket offsets
    int32_t *row_cur;       // emit pass: bucket cursors
    run *runs;
};

constexpr int kTabShift = 10;

// The table entry holding segment s: a search between the entries of its
// block of 2^kTabShift segments when the table has a block index.
__device__ __forceinline__ int job_entry(const job_tables &t, int s) {
    if (!t.tab_idx) return table_find(t.tab, t.n_tab, s);
    const int b = s >> kTabShift;
    int lo_i = t.tab_idx[b], hi_i = t.tab_idx[b + 1] + 1;   // tab[lo_i].x <= s < tab[hi_i].x
    while (hi_i - lo_i > 1) {
        int mid = (lo_i + hi_i) >> 1;
        if (t.tab[mid].x <= s) lo_i = mid; else hi_i = mid;
    }
    return lo_i;
}

// Segment s of table entry c, its end points moved by the job's offset as
// scan does with add(offset, point) (hpp:2205).  Returns the job index.
__device__ __forceinline__ int segment_at(const job_tables &t, int c, int s, float2 &a, float2 &b) {
    const int ji = t.tab[c].y;
    const scan_job &jj = t.jobs[ji];
    int k = jj.line_first + (s - t.tab[c].x);
    // a select, not an index into the parameter arrays: an index would copy
    // them to local memory
    const float2 *pts = jj.geom ? t.pts[1] : t.pts[0];
    const int32_t *prev = jj.geom ? t.prev[1] : t.prev[0];
    float2 pb = pts[k];
    float2 pa = pts[prev[k]];
    a = f2(jj.offx + pa.x, jj.offy + pa.y);
    b = f2(jj.offx + pb.x, jj.offy + pb.y);
    return ji;
}

// Segment s of a binned job: the segment ending at its point k, from the
// nearest point before k with finite coordinates.  A non-finite point is
// left out and its neighbours joined, as the polygon clip drops it (its
// comparisons fail for NaN, hpp:2218-2223): the segment ending at it is
// dropped (false), and the one leaving it starts further back.
__device__ __forceinline__ bool binned_segment(const job_tables &t, int c, int s, float2 &a, float2 &b, int &ji) {
    ji = t.tab[c].y;
    const scan_job &jj = t.jobs[ji];
    const int k = jj.line_first + (s - t.tab[c].x);
    const float2 *pts = jj.geom ? t.pts[1] : t.pts[0];
    const int32_t *prev = jj.geom ? t.prev[1] : t.prev[0];
    auto finite = [](float2 p) { return isfinite(p.x) && isfinite(p.y); };
    float2 pb = pts[k];
    b = f2(jj.offx + pb.x, jj.offy + pb.y);
    if (!finite(b)) return false;
    int j = prev[k];
    float2 pa = pts[j];
    a = f2(jj.offx + pa.x, jj.offy + pa.y);
    // the links of a subpath form a cycle through k: the walk ends there
    for (int guard = 0; !finite(a) && j != k && guard < jj.seg_count; ++guard) {
        j = prev[j];
        pa = pts[j];
        a = f2(jj.offx + pa.x, jj.offy + pa.y);
    }
    return finite(a) && j != k;
}

// Segment s of the scan (the table's, or the last clip pass's polygons).
template <bool CLIPPED>
__device__ __forceinline__ int segment_raw(const job_tables &t, int s, float2 &a, float2 &b) {
    if (CLIPPED) {
        a = t.cl_pts[t.cl_prev[s]];
        b = t.cl_pts[s];
        return t.cl_job[s];
    }
    return segment_at(t, job_entry(t, s), s, a, b);
}

// The same segment clamped to the job's rectangle as scan does before
// add_runs (hpp:2236-2238).
template <bool CLIPPED>
__device__ __forceinline__ int segment_of(const job_tables &t, int s, float2 &a, float2 &b) {
    int ji = segment_raw<CLIPPED>(t, s, a, b);
    const scan_job &j = t.jobs[ji];
    a = f2(lo(hi(a.x, 0.0f), j.width), lo(hi(a.y, 0.0f), j.height));
    b = f2(lo(hi(b.x, 0.0f), j.width), lo(hi(b.y, 0.0f), j.height));
    return ji;
}

// Rows of the job that a segment's cell walk touches: [r0, r1] (empty when
// r0 > r1).  Row k of the walk is dda_row_index(p, k), k < nrows, and rows
// outside [0, rows) contribute nothing (as in k_runs).
__device__ __forceinline__ void dda_rows(const dda_piece &p, int rows, int &r0, int &r1) {
    int n = p.nrows < rows + 2 ? p.nrows : rows + 2;
    int a = dda_row_index(p, 0), b = dda_row_index(p, n - 1);
    r0 = max(min(a, b), 0);
    r1 = min(max(a, b), rows - 1);
}

// ------------------------------------------------------ row-band binning
// The sort-free coverage path: instead of runs, every segment of a binned
// job is listed in each band of rows it crosses (band_h rows per band, bins
// of one job consecutive), as its clamped end points.  The tile kernel then
// accumulates the signed areas of one strip's bands in shared memory.
// Pass 1 counts entries per bin, pass 2 (after a scan) writes them.
struct bin_tables {
    int32_t *cnt;          // per bin: entries (count pass)
    int32_t *cur;          // per bin: write cursor (emit pass)
    const int64_t *off;    // per bin: first entry (exclusive scan of cnt)
    float4 *seg;           // entries: (a.x, a.y, b.x, b.y)
};

template <bool EMIT>
__global__ void k_bin(job_tables t, bin_tables bt, int total_segments) {
    // Segment s of the binned jobs' table (binned_segment: non-finite points
    // left out, their neighbours joined), clipped on its own (clip_segment:
    // the part left of the rectangle becomes its projection on x = 0, as the
    // reference's polygon clip and clamp make it in sum, hpp:2204-2239; the
    // parts above, below and right of it add to no pixel and are dropped).
    // Up to two pieces per segment in fixed slots, each listed in every band
    // it crosses.  A warp's
    // 32 consecutive segments mostly share their job and bands: per slot,
    // lanes adding to the same bin are grouped, so each bin takes one atomic
    // per warp, and each lane writes at the group's base plus its rank.
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total_segments; base += stride) {
        const int s = base + lane;
        float2 pa[2], pb[2];
        int pbin[2] = {0, 0}, pnb[2] = {0, 0};
        float2 a, b;
        int ji = 0;
        if (s < total_segments && binned_segment(t, job_entry(t, s), s, a, b, ji)) {
            const scan_job &j = t.jobs[ji];
            const unsigned has = clip_segment(a, b, j.width, j.height, pa, pb);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                dda_piece p;
                if (!(has >> i & 1u) || !dda_setup(pa[i], pb[i], p)) continue;
                int r0, r1;
                dda_rows(p, j.rows, r0, r1);
                if (r0 > r1) continue;
                pbin[i] = j.bin_base + r0 / j.band_h;
                pnb[i] = r1 / j.band_h - r0 / j.band_h + 1;
            }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int rounds = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(pnb[i])));
            for (int k = 0; k < rounds; ++k) {
                const int bin = k < pnb[i] ? pbin[i] + k : -1;
                const unsigned peers = __match_any_sync(0xffffffffu, bin);
                if (bin < 0) continue;
                const int leader = __ffs(peers) - 1;
                const int rank = __popc(peers & ((1u << lane) - 1u));
                if (!EMIT) {
                    if (lane == leader) atomicAdd(bt.cnt + bin, __popc(peers));
                } else {
                    // the bin's range is read before the atomic, so the two
                    // round trips overlap
                    const int64_t o0 = bt.off[bin], o1 = bt.off[bin + 1];
                    int first = 0;
                    if (lane == leader) first = atomicAdd(bt.cur + bin, __popc(peers));
                    first = __shfl_sync(peers, first, leader);
                    int64_t at = o0 + first + rank;
                    if (at < o1) bt.seg[at] = make_float4(pa[i].x, pa[i].y, pb[i].x, pb[i].y);
                }
            }
        }
    }
}

// Segments go to warps 32 at a time: each lane prepares one segment
// (clamped to its job's rectangle as scan does before add_runs,
// hpp:2236-2238), then the warp deals all rows of the 32 segments out to its
// lanes, so a long segment no longer holds one thread while the rest idle.
// Any row can be rebuilt on its own (dda_exit), so the split is exact.
static constexpr int kRunsWarps = 4;   // warps per block in k_runs

template <bool EMIT, bool CLIPPED>
__global__ void __launch_bounds__(kRunsWarps * 32) k_runs(job_tables t, int total_segments, int seg_per_warp) {
    __shared__ dda_piece pieces[kRunsWarps][32];
    __shared__ int seg_job[kRunsWarps][32];
    __shared__ int seg_end[kRunsWarps][32];   // inclusive prefix of row counts
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kRunsWarps + w, nw = gridDim.x * kRunsWarps;
    // seg_per_warp (a power of two up to 32) segments per warp round: fewer
    // when segments are few, so that more warps share their rows.
    for (int base = gw * seg_per_warp; base < total_segments; base += nw * seg_per_warp) {
        int s = base + lane;
        int rows_here = 0, ji = 0;
        dda_piece p;
        p.nrows = 0;
        if (lane < seg_per_warp && s < total_segments) {
            float2 a, b;
            ji = segment_of<CLIPPED>(t, s, a, b);
            const scan_job &j = t.jobs[ji];
            if (!j.binned && dda_setup(a, b, p)) rows_here = p.nrows < j.rows + 2 ? p.nrows : j.rows + 2;
        }
        int incl = rows_here;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        pieces[w][lane] = p;
        seg_job[w][lane] = ji;
        seg_end[w][lane] = incl;
        int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (int q = lane; q < total; q += 32) {
            int lo_i = 0, hi_i = 31;   // first segment whose inclusive end exceeds q
            while (lo_i < hi_i) {
                int mid = (lo_i + hi_i) >> 1;
                if (seg_end[w][mid] > q) hi_i = mid; else lo_i = mid + 1;
            }
            const dda_piece &pp = pieces[w][lo_i];
            const int jq = seg_job[w][lo_i];
            const scan_job &j = t.jobs[jq];
            int k = q - (lo_i ? seg_end[w][lo_i - 1] : 0);
            float2 entry = k == 0 ? f2(pp.fx, pp.fy) : dda_exit(pp, k - 1);
            float2 ex = dda_exit(pp, k);
            int ps, pe;
            dda_span(pp, k, entry, ex, ps, pe);
            int row = dda_row_index(pp, k);
            if (row < 0 || row >= j.rows) continue;
            // cells of a clamped segment lie in [0, cols]; other spans come
            // from non-finite input and are skipped
            if (!(ps >= 0 && pe >= ps && pe <= j.cols)) continue;
            int n = pe - ps + 2;
            int grow = j.row_base + row;
            if (!EMIT) {
                atomicAdd(t.row_cnt + grow, n);
                if (j.need_box) {
                    long long key = (static_cast<long long>(row) << 32) | static_cast<long long>(ps < 0 ? 0 : ps);
                    atomicMin(reinterpret_cast<long long *>(&t.boxes[jq].first_key), key);
                }
            } else {
                int at = atomicAdd(t.row_cur + grow, n);
                int64_t cap = t.row_off[grow + 1] - t.row_off[grow];
                if (at + n > cap) continue;
                run *out = t.runs + t.row_off[grow] + at;
                int i = 0, x0 = 0x7fffffff, x1 = -0x7fffffff;
                int cols = j.cols;
                auto emit = [&](int x, float d) {
                    bool okx = x >= 0 && x < cols;
                    out[i++] = run{okx ? x : 0, okx ? d : 0.0f};
                    if (okx && d != 0.0f) {
                        x0 = x < x0 ? x : x0;
                        x1 = x > x1 ? x : x1;
                    }
                };
                dda_cells(pp, entry, ex, ps, pe, emit);
                if (j.need_box && x0 <= x1) {
                    cover_box *box = t.boxes + jq;
                    atomicMin(&box->x0, x0);
                    atomicMax(&box->x1, x1);
                    atomicMin(&box->y0, row);
                    atomicMax(&box->y1, row);
                }
            }
        }
        __syncwarp();
    }
}

__global__ void k_box_init(cover_box *boxes, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    boxes[i].x0 = 0x7fffffff;
    boxes[i].x1 = -0x7fffffff;
    boxes[i].y0 = 0x7fffffff;
    boxes[i].y1 = -0x7fffffff;
    boxes[i].first_key = 0x7fffffffffffffffll;
}

// The reference's run order within a row (hpp:2172-2181), with ties of equal
// magnitude broken by sign so the order does not depend on arrival order.
__device__ __forceinline__ bool run_less(const run &a, const run &b) {
    if (a.x != b.x) return a.x < b.x;
    float fa = fabsf(a.delta), fb = fabsf(b.delta);
    if (fa != fb) return fa < fb;
    return a.delta < b.delta;
}

__device__ void sort_runs(run *r, int n) {
    // Shell sort with Ciura's gaps (plain insertion sort for short rows).
    const int gaps[] = {1750, 701, 301, 132, 57, 23, 10, 4, 1};
    for (int gi = 0; gi < 9; ++gi) {
        int g = gaps[gi];
        if (g >= n) continue;
        for (int i = g; i < n; ++i) {
            run v = r[i];
            int j = i;
            for (; j >= g && run_less(v, r[j - g]); j -= g) r[j] = r[j - g];
            r[j] = v;
        }
    }
}

static constexpr int kRowCap = 512;     // runs per row sorted by one warp in shared memory
static constexpr int kRowsWarps = 8;    // warps per block in k_rows
static constexpr int kLongCap = 8192;   // runs per row sorted by one block in k_rows_long
static constexpr int kLongThreads = 512;
static constexpr int kLongSmem = kLongCap * (sizeof(run) + sizeof(float));

__device__ __forceinline__ run run_pad() { return run{0x7fffffff, 0.0f}; }

// Coalesce a sorted row and store the running sum after each cell, in the
// reference's float order (hpp:2243-2252 then the walk of hpp:2551-2605):
// equal-x deltas are added in sorted order, then the cells are summed left
// to right.  In place: the k-th coalesced cell is written after element k
// has been read.  Returns the number of cells.
__device__ __forceinline__ int coalesce_sum(run *v, float *acc, int m) {
    if (m == 0) return 0;
    run cur = v[0];
    float sum = 0.0f;
    int k = 0;
    for (int i = 1; i < m; ++i) {
        run u = v[i];
        if (u.x == cur.x) {
            cur.delta += u.delta;
        } else {
            sum += cur.delta;
            v[k] = cur;
            acc[k] = sum;
            ++k;
            cur = u;
        }
    }
    sum += cur.delta;
    v[k] = cur;
    acc[k] = sum;
    return k + 1;
}

// Bitonic sort of v[0, n2) (n2 a power of two) by run_less, `lanes` threads
// with ids `id` cooperating; `sync` orders the steps.
__device__ __forceinline__ bool run_less_xd(int ax, float ad, int bx, float bd) {
    if (ax != bx) return ax < bx;
    float fa = fabsf(ad), fb = fabsf(bd);
    if (fa != fb) return fa < fb;
    return ad < bd;
}

struct warp_sync {
    __device__ void operator()() const { __syncwarp(); }
};
struct block_sync {
    __device__ void operator()() const { __syncthreads(); }
};

template <class Sync>
__device__ __forceinline__ void bitonic_sort(run *v, int n2, int id, int lanes, Sync sync) {
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = id; i < (n2 >> 1); i += lanes) {
                int lo_i = ((i & ~(j - 1)) << 1) | (i & (j - 1));
                int hi_i = lo_i + j;
                bool up = (lo_i & k) == 0;
                run a = v[lo_i], b = v[hi_i];
                if (run_less(b, a) == up) {
                    v[lo_i] = b;
                    v[hi_i] = a;
                }
            }
            sync();
        }
    }
}

// Sort and coalesce one row's runs exactly as the reference does after its
// std::sort (hpp:2243-2252), then store the running coverage sum after each
// coalesced cell (the value render_main's walk holds from that cell on).
// One warp per row: the row's nonzero runs are compacted into shared memory
// and sorted by the warp (in registers up to 32 runs, else a shared-memory
// bitonic network); the warp then coalesces equal x and sums the cells in the
// reference's order of float additions.  Rows with more than kRowCap
// nonzero runs are listed for k_rows_long.
__global__ void __launch_bounds__(kRowsWarps * 32) k_rows(const int64_t *__restrict__ row_off,
                                                          int32_t *__restrict__ row_cnt,
                                                          int32_t *__restrict__ row_cur, int32_t *__restrict__ row_len,
                                                          run *__restrict__ runs, float *__restrict__ sums,
                                                          int total_rows, int32_t *__restrict__ long_rows,
                                                          int32_t *__restrict__ n_long, int4 *__restrict__ row_meta) {
    __shared__ run buf[kRowsWarps][kRowCap];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kRowsWarps + w, nw = gridDim.x * kRowsWarps;
    run *v = buf[w];
    // The next row's bucket offsets and count are fetched while this row is
    // sorted, so the warp does not wait for them between rows.
    long long nxt_off = 0, nxt_end = 0;
    int nxt_cnt = 0;
    if (gw < total_rows) {
        nxt_off = row_off[gw];
        nxt_end = row_off[gw + 1];
        nxt_cnt = row_cur[gw];
    }
    for (int y = gw; y < total_rows; y += nw) {
        const long long off = nxt_off;
        int cap = static_cast<int>(nxt_end - off);
        int n = nxt_cnt;
        if (n > cap) n = cap;
        if (y + nw < total_rows) {
            nxt_off = row_off[y + nw];
            nxt_end = row_off[y + nw + 1];
            nxt_cnt = row_cur[y + nw];
        }
        run *r = runs + off;
        float *sm = sums + off;
        // Compact the nonzero runs.
        int m = 0;
        for (int base = 0; base < n; base += 32) {
            int i = base + lane;
            run u = i < n ? r[i] : run{0, 0.0f};
            bool keep = i < n && u.delta != 0.0f;
            unsigned bal = __ballot_sync(0xffffffffu, keep);
            int at = m + __popc(bal & ((1u << lane) - 1u));
            if (keep && at < kRowCap) v[at] = u;
            m += __popc(bal);
        }
        if (m > kRowCap) {
            if (lane == 0) long_rows[atomicAdd(n_long, 1)] = y;
            continue;
        }
        __syncwarp();
        if (m <= 32) {
            // One run per lane: a shuffle bitonic network sorts them in registers.
            int x = 0x7fffffff;
            float d = 0.0f;
            if (lane < m) {
                x = v[lane].x;
                d = v[lane].delta;
            }
            // Network over the next power of two >= m (pads sort last).
            int n2 = 1;
            while (n2 < m) n2 <<= 1;
            for (int k = 2; k <= n2; k <<= 1) {
                for (int jj = k >> 1; jj > 0; jj >>= 1) {
                    int ox = __shfl_xor_sync(0xffffffffu, x, jj);
                    float od = __shfl_xor_sync(0xffffffffu, d, jj);
                    bool keep_min = ((lane & jj) == 0) == ((lane & k) == 0);
                    if (keep_min ? run_less_xd(ox, od, x, d) : run_less_xd(x, d, ox, od)) {
                        x = ox;
                        d = od;
                    }
                }
            }
            __syncwarp();
            if (lane < m) v[lane] = run{x, d};
        } else {
            int n2 = 1;
            while (n2 < m) n2 <<= 1;
            for (int i = m + lane; i < n2; i += 32) v[i] = run_pad();
            __syncwarp();
            bitonic_sort(v, n2, lane, 32, warp_sync());
        }
        __syncwarp();
        // Coalesce and sum, 32 sorted runs at a time: the first run of each
        // x adds the rest of its x in order (the merged delta), then the
        // merged deltas are summed strictly left to right, one shuffle per
        // cell, which is the reference's order of float additions.
        int groups = 0;
        float sum = 0.0f;
        for (int c0 = 0; c0 < m; c0 += 32) {
            int i = c0 + lane;
            bool valid = i < m;
            run e = valid ? v[i] : run{0, 0.0f};
            bool start = valid && (i == 0 || v[i - 1].x != e.x);
            float merged = 0.0f;
            if (start) {
                merged = e.delta;
                for (int t = i + 1; t < m && v[t].x == e.x; ++t) merged += v[t].delta;
            }
            unsigned bal = __ballot_sync(0xffffffffu, start);
            int gi = groups + __popc(bal & ((1u << lane) - 1u));
            float mine = 0.0f;
            for (unsigned b = bal; b; b &= b - 1) {
                int src = __ffs(b) - 1;
                sum += __shfl_sync(0xffffffffu, merged, src);
                if (lane == src) mine = sum;
            }
            if (start) {
                r[gi] = run{e.x, merged};
                sm[gi] = mine;
            }
            groups += __popc(bal);
        }
        if (lane == 0) {
            row_len[y] = groups;
            row_meta[y] = groups ? make_int4(v[0].x, v[m - 1].x, __float_as_int(sum), groups)
                                 : make_int4(0x7fffffff, -1, 0, 0);
            row_cnt[y] = 0;
            row_cur[y] = 0;
        }
        __syncwarp();
    }
}

// The rows k_rows listed: one block per row, sorted in shared memory when
// they hold at most kLongCap nonzero runs, else in place by one thread.
__global__ void __launch_bounds__(kLongThreads) k_rows_long(const int64_t *__restrict__ row_off,
                                                           int32_t *__restrict__ row_cnt,
                                                           int32_t *__restrict__ row_cur,
                                                           int32_t *__restrict__ row_len, run *__restrict__ runs,
                                                           float *__restrict__ sums,
                                                           const int32_t *__restrict__ long_rows,
                                                           const int32_t *__restrict__ n_long,
                                                           int4 *__restrict__ row_meta) {
    extern __shared__ run lbuf[];   // kLongCap runs, then kLongCap floats
    float *lacc = reinterpret_cast<float *>(lbuf + kLongCap);
    __shared__ int warp_cnt[kLongThreads / 32];
    __shared__ int total;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int count = *n_long;
    for (int li = blockIdx.x; li < count; li += gridDim.x) {
        const int y = long_rows[li];
        int cap = static_cast<int>(row_off[y + 1] - row_off[y]);
        int n = row_cur[y];
        if (n > cap) n = cap;
        run *r = runs + row_off[y];
        float *sm = sums + row_off[y];
        // Count the nonzero runs, then compact them in order.
        int mine = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) mine += r[i].delta != 0.0f;
        for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
        if (lane == 0) warp_cnt[w] = mine;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int i = 0; i < kLongThreads / 32; ++i) t += warp_cnt[i];
            total = t;
        }
        __syncthreads();
        const int m = total;
        int kept = m;
        if (m <= kLongCap) {
            int base = 0;
            for (int b0 = 0; b0 < n; b0 += blockDim.x) {
                int i = b0 + threadIdx.x;
                run u = i < n ? r[i] : run{0, 0.0f};
                bool keep = i < n && u.delta != 0.0f;
                unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (lane == 0) warp_cnt[w] = __popc(bal);
                __syncthreads();
                int before = 0, all = 0;
                for (int q = 0; q < kLongThreads / 32; ++q) {
                    before += q < w ? warp_cnt[q] : 0;
                    all += warp_cnt[q];
                }
                if (keep) lbuf[base + before + __popc(bal & ((1u << lane) - 1u))] = u;
                base += all;
                __syncthreads();
            }
            int n2 = 1;
            while (n2 < m) n2 <<= 1;
            for (int i = m + threadIdx.x; i < n2; i += blockDim.x) lbuf[i] = run_pad();
            __syncthreads();
            if (n2 > 1) bitonic_sort(lbuf, n2, threadIdx.x, blockDim.x, block_sync());
            if (threadIdx.x == 0) {
                total = coalesce_sum(lbuf, lacc, m);
                row_meta[y] = total ? make_int4(lbuf[0].x, lbuf[total - 1].x, __float_as_int(lacc[total - 1]), total)
                                    : make_int4(0x7fffffff, -1, 0, 0);
            }
            __syncthreads();
            kept = total;
            for (int i = threadIdx.x; i < kept; i += blockDim.x) {
                r[i] = lbuf[i];
                sm[i] = lacc[i];
            }
        } else if (threadIdx.x == 0) {
            int k = 0;
            for (int i = 0; i < n; ++i)
                if (r[i].delta != 0.0f) r[k++] = r[i];
            sort_runs(r, k);
            int c = 0;
            float sum = 0.0f;
            for (int i = 0; i < k; ++i) {
                if (c > 0 && r[c - 1].x == r[i].x) {
                    r[c - 1].delta += r[i].delta;
                } else {
                    if (c > 0) sm[c - 1] = (sum += r[c - 1].delta);
                    r[c++] = r[i];
                }
            }
            if (c > 0) sm[c - 1] = (sum += r[c - 1].delta);
            total = c;
            row_meta[y] = c ? make_int4(r[0].x, r[c - 1].x, __float_as_int(sm[c - 1]), c)
                            : make_int4(0x7fffffff, -1, 0, 0);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            row_len[y] = total;
            row_cnt[y] = 0;
            row_cur[y] = 0;
        }
        __syncthreads();
    }
}

// Running sum in force at pixel x: the sum after the last coalesced run at or
// left of x (0 before the first run).
__device__ __forceinline__ float sum_at(const run *r, const float *sm, int n, int x) {
    int lo_i = 0, hi_i = n;
    while (lo_i < hi_i) {
        int mid = (lo_i + hi_i) >> 1;
        if (r[mid].x <= x) lo_i = mid + 1; else hi_i = mid;
    }
    return lo_i > 0 ? sm[lo_i - 1] : 0.0f;
}

struct row_view {
    const int64_t *row_off;
    const int32_t *row_len;
    const run *runs;
    const float *sums;
    const int4 *meta;   // per row: first x, last x, final sum (bits), run count
};

// ---------------------------------------------------------- main render
struct paint_args {
    const command *cmd;
    float4 *bitmap;
    int W, H;
    row_view rv;
    int row_base;
    const float *vis;    // dense clip visibility, null for the whole canvas
    int y_begin, y_end;
    paint_src src;
};

// render_main's span walk (hpp:2551-2605) as a dense pass: each pixel takes
// the row's running coverage sum in force at its x, is painted, and is
// composited through the clip visibility.  Warp per row.
__global__ void k_paint(paint_args a) {
    int lane = threadIdx.x & 31;
    const command &c = *a.cmd;
    const int op = c.op;
    const bool clearing = !(op & 8);
    for (int y = a.y_begin + warp_id_global(); y < a.y_end; y += warps_total()) {
        int row = a.row_base + y;
        int n = a.rv.row_len[row];
        if (!clearing && n == 0) continue;
        const run *r = a.rv.runs + a.rv.row_off[row];
        const float *sm = a.rv.sums + a.rv.row_off[row];
        // The reference walks the path runs merged with the clip runs, so
        // after the last path run it keeps painting with the row's final
        // sum up to the clip's end (hpp:2572-2600): that matters when the
        // float sum is left above the visibility threshold.
        int xs = clearing ? 0 : r[0].x;
        bool tail = n > 0 && cover_of(sm[n - 1], c.fill_rule) >= kVisible;
        int xe = clearing || tail ? a.W - 1 : min(r[n - 1].x, a.W - 1);
        for (int x = xs + lane; x <= xe; x += 32) {
            float cov = cover_of(sum_at(r, sm, n, x), c.fill_rule);
            float vis = a.vis ? a.vis[static_cast<size_t>(y) * a.W + x] : 1.0f;
            if ((cov >= kVisible || clearing) && vis >= kVisible) {
                float4 *px = a.bitmap + static_cast<size_t>(y) * a.W + x;
                float4 back = *px;
                float4 p = paint_at(c, a.src, static_cast<float>(x) + 0.5f, static_cast<float>(y) + 0.5f);
                float k = cov * c.alpha;
                float4 fore = make_float4(p.x * k, p.y * k, p.z * k, p.w * k);
                *px = blend(back, fore, op, vis);
            }
        }
    }
}

// ------------------------------------------------------------------ clip
struct clip_args {
    // path runs (sorted, coalesced) of this clip, rows from p_base
    const int64_t *p_off;
    const int32_t *p_len;
    const run *p_runs;
    int p_base;
    // old mask (null runs = the whole canvas: per row {0,+1}, {W,-1})
    const int32_t *o_off, *o_len;
    const run *o_runs;
    const int *o_last_row;   // last row holding old-mask runs (null: H-1)
    const cover_box *p_box;  // bounds of the path runs
    // new mask
    int32_t *n_off;          // H+1 offsets (from the capacities)
    int32_t *n_len;          // H+1: capacities, then run counts
    run *n_runs;
    float *n_sums;           // running sum after each run
    float *n_vis;            // W*H dense visibility
    int *n_last_row;
    int W, H;
    int rule;                // fill rule of the clip path
};

// All clip masks of one nesting level are made together: blockIdx.y picks
// the clip (args[first + blockIdx.y]), so a level costs four launches
// however many canvases hold a clip.

// Run capacity of each row of a new clip mask: the path's raw runs plus the
// old mask's runs (2 per row for the whole canvas).
__global__ void k_clip_caps_all(const clip_args *args, int first) {
    const clip_args &a = args[first + blockIdx.y];
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y > a.H) return;
    if (y == 0) *a.n_last_row = -1;
    if (y == a.H) {
        a.n_len[y] = 0;
        return;
    }
    int p = static_cast<int>(a.p_off[a.p_base + y + 1] - a.p_off[a.p_base + y]);
    int o = a.o_off ? a.o_off[y + 1] - a.o_off[y] : 2;
    a.n_len[y] = p + o;
}

// Exclusive scan of the H+1 capacities into the row offsets, one block (of
// 1024 threads) per clip.
__global__ void __launch_bounds__(1024) k_clip_scan_all(const clip_args *args, int first) {
    __shared__ int32_t warp_sums[32];
    __shared__ int32_t carry;
    const clip_args &a = args[first + blockIdx.y];
    const int n = a.H + 1, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        int i = base + threadIdx.x;
        int32_t v = i < n ? a.n_len[i] : 0;
        int32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sums[w] = incl;
        __syncthreads();
        if (w == 0) {
            int32_t s = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int32_t t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        int32_t before = carry + (w > 0 ? warp_sums[w - 1] : 0);
        if (i < n) a.n_off[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sums[31];
        __syncthreads();
    }
}

// clip() (hpp:3057-3099) for one row: merge the path runs with the old mask
// runs in the reference's order and emit changes of the product coverage.
// The reference stops its single merge loop when either list runs out, so
// the row where that happens is cut short and later rows stay empty.  The
// running sums of the new runs follow (the clip visibility in force from
// each run on is min(|sum|, 1), hpp:2568-2570).
__global__ void k_clip_rows_all(const clip_args *args, int first) {
    const clip_args &a = args[first + blockIdx.y];
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= a.H) return;
    int o_last = a.o_last_row ? *a.o_last_row : a.H - 1;
    int p_last = a.p_box->x0 <= a.p_box->x1 ? a.p_box->y1 : -1;
    int stop_row = min(p_last, o_last);
    int m = 0;
    run *out = a.n_runs + a.n_off[y];
    int cap = a.n_off[y + 1] - a.n_off[y];
    if (y <= stop_row) {
        const run *p = a.p_runs + a.p_off[a.p_base + y];
        int pn = a.p_len[a.p_base + y];
        run dflt[2] = {run{0, 1.0f}, run{a.W, -1.0f}};
        const run *o = a.o_runs ? a.o_runs + a.o_off[y] : dflt;
        int on = a.o_runs ? a.o_len[y] : 2;
        bool path_ends = y == p_last, mask_ends = y == o_last;
        int i1 = 0, i2 = 0;
        float last = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (;;) {
            bool p_left = i1 < pn, o_left = i2 < on;
            if (y == stop_row) {
                if ((path_ends && !p_left) || (mask_ends && !o_left)) break;
            }
            if (!p_left && !o_left) break;
            bool which;
            if (!p_left) which = false;
            else if (!o_left) which = true;
            else which = p[i1].x < o[i2].x || (p[i1].x == o[i2].x && fabsf(p[i1].delta) < fabsf(o[i2].delta));
            int nx = which ? p[i1].x : o[i2].x;
            if (which) s1 += p[i1++].delta;
            else s2 += o[i2++].delta;
            float vis = cover_of(s1, a.rule) * lo(fabsf(s2), 1.0f);
            if (vis == last) continue;
            if (m > 0 && out[m - 1].x == nx) out[m - 1].delta += vis - last;
            else if (m < cap) out[m++] = run{nx, vis - last};
            last = vis;
        }
    }
    a.n_len[y] = m;
    if (m > 0) atomicMax(a.n_last_row, y);
    float *sm = a.n_sums + a.n_off[y];
    float sum = 0.0f;
    for (int j = 0; j < m; ++j) {
        sum += out[j].delta;
        sm[j] = sum;
    }
}

// Dense visibility from the mask runs (warp per row).  Pixels outside the
// row's first..last run are never visited by the reference's walks: 0.
__global__ void k_mask_fill_all(const clip_args *args, int first) {
    const clip_args &a = args[first + blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int y = blockIdx.x * wpb + (threadIdx.x >> 5); y < a.H; y += gridDim.x * wpb) {
        const run *r = a.n_runs + a.n_off[y];
        const float *sm = a.n_sums + a.n_off[y];
        int n = a.n_len[y];
        int first_x = n ? r[0].x : 0x7fffffff, last_x = n ? r[n - 1].x : -1;
        for (int x = lane; x < a.W; x += 32) {
            float v = 0.0f;
            if (x >= first_x && x <= last_x) v = lo(fabsf(sum_at(r, sm, n, x)), 1.0f);
            a.n_vis[static_cast<size_t>(y) * a.W + x] = v;
        }
    }
}

// ---------------------------------------------------------------- shadows
struct shadow_rect { int left, right, top, bottom, width, height; };

// Working rectangle of render_shadow (hpp:2409-2426) from the exact bounds of
// the padded scan conversion, including the reference's quirk that the
// first run after sorting is kept even when its delta is zero.
__global__ void k_shadow_rect(const cover_box *box, int W, int H, int border, shadow_rect *out) {
    int ext_w = W + 2 * border, ext_h = H + 2 * border;
    int left = ext_w, right = 0, top = ext_h, bottom = 0;
    cover_box b = *box;
    if (b.x0 <= b.x1) {
        left = min(left, b.x0); right = max(right, b.x1);
        top = min(top, b.y0); bottom = max(bottom, b.y1);
    }
    if (b.first_key != 0x7fffffffffffffffll) {
        int fx = static_cast<int>(b.first_key & 0xffffffffll), fy = static_cast<int>(b.first_key >> 32);
        left = min(left, fx); right = max(right, fx);
        top = min(top, fy); bottom = max(bottom, fy);
    }
    left = max(left - border, 0);
    right = min(right + border, ext_w) + 1;
    top = max(top - border, 0);
    bottom = min(bottom + border, ext_h);
    shadow_rect r;
    r.left = left; r.right = right; r.top = top; r.bottom = bottom;
    r.width = max(right - left, 0);
    r.height = max(bottom - top, 0);
    *out = r;
}

// Alpha raster of the shadow (hpp:2430-2452), warp per working row: pixels
// between the row's first and last run get coverage times paint alpha.
__global__ void k_shadow_raster(const command *cmd, paint_src src, row_view rv, int row_base,
                                const shadow_rect *rect, float *__restrict__ out) {
    int lane = threadIdx.x & 31;
    const command &c = *cmd;
    const shadow_rect rc = *rect;
    for (int y = rc.top + warp_id_global(); y < rc.bottom; y += warps_total()) {
        int row = row_base + y;
        int n = rv.row_len[row];
        const run *r = rv.runs + rv.row_off[row];
        const float *sm = rv.sums + rv.row_off[row];
        int first = n ? r[0].x : 0x7fffffff, last = n ? r[n - 1].x : -1;
        for (int x = rc.left + lane; x < rc.right; x += 32) {
            float val = 0.0f;
            if (x >= first && x <= last) {
                float cov = cover_of(sum_at(r, sm, n, x), c.fill_rule);
                if (cov >= kVisible) {
                    float px = (static_cast<float>(x) + 0.5f) - c.sh_offx;
                    float py = (static_cast<float>(y) + 0.5f) - c.sh_offy;
                    val = cov * paint_at(c, src, px, py).w;
                }
            }
            out[static_cast<size_t>(y - rc.top) * rc.width + (x - rc.left)] = val;
        }
    }
}

// The reference's extended box blur (Gwosdek et al., hpp:2453-2503): three
// running-sum passes along each row, then along each column, with the same
// float operation order (one thread per row, then per column).  `tmp` holds
// one working copy per row/column.
__global__ void k_blur_rows(float *s, float *tmp, const shadow_rect *rect, int radius, float w1, float w2) {
    const shadow_rect rc = *rect;
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= rc.height) return;
    size_t width = rc.width, r = radius;
    float *row = s + static_cast<size_t>(y) * width;
    float *t = tmp + static_cast<size_t>(y) * width;
    for (int pass = 0; pass < 3; ++pass) {
        for (size_t x = 0; x < width; ++x) t[x] = row[x];
        float run = r + 1 < width ? w1 * t[r + 1] : 0.0f;
        for (size_t x = 0; x <= r && x < width; ++x) run += (w1 + w2) * t[x];
        row[0] = run;
        for (size_t x = 1; x < width; ++x) {
            if (x >= r + 1) run -= w2 * t[x - r - 1];
            if (x >= r + 2) run -= w1 * t[x - r - 2];
            if (x + r < width) run += w2 * t[x + r];
            if (x + r + 1 < width) run += w1 * t[x + r + 1];
            row[x] = run;
        }
    }
}

__global__ void k_blur_cols(float *s, float *tmp, const shadow_rect *rect, int radius, float w1, float w2) {
    const shadow_rect rc = *rect;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= rc.width) return;
    size_t width = rc.width, height = rc.height, r = radius;
    for (int pass = 0; pass < 3; ++pass) {
        for (size_t y = 0; y < height; ++y) tmp[y * width + x] = s[y * width + x];
        float run = r + 1 < height ? w1 * tmp[(r + 1) * width + x] : 0.0f;
        for (size_t y = 0; y <= r && y < height; ++y) run += (w1 + w2) * tmp[y * width + x];
        if (height > 0) s[x] = run;
        for (size_t y = 1; y < height; ++y) {
            if (y >= r + 1) run -= w2 * tmp[(y - r - 1) * width + x];
            if (y >= r + 2) run -= w1 * tmp[(y - r - 2) * width + x];
            if (y + r < height) run += w2 * tmp[(y + r) * width + x];
            if (y + r + 1 < height) run += w1 * tmp[(y + r + 1) * width + x];
            s[y * width + x] = run;
        }
    }
}

// Shadow composite through the clip visibility (hpp:2504-2538); nothing is
// cleared outside the working rectangle.
__global__ void k_shadow_composite(const command *cmd, float4 *bitmap, int W, int H, const float *visp,
                                   const shadow_rect *rect, const float *__restrict__ sh) {
    const command &c = *cmd;
    const shadow_rect r = *rect;
    if (r.width <= 0 || r.height <= 0) return;
    int b = c.sh_border;
    int x0 = max(0, r.left - b), x1 = min(W, r.right - b);
    int y0 = max(0, r.top - b), y1 = min(H, r.bottom - b);
    int x = x0 + blockIdx.x * blockDim.x + threadIdx.x;
    int y = y0 + blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= x1 || y >= y1) return;
    float vis = visp ? visp[static_cast<size_t>(y) * W + x] : 1.0f;
    if (vis < kVisible) return;
    float s = sh[static_cast<size_t>(y + b - r.top) * r.width + (x + b - r.left)];
    float k = c.alpha * s;
    float4 fore = make_float4(c.sh_color[0] * k, c.sh_color[1] * k, c.sh_color[2] * k, c.sh_color[3] * k);
    float4 *px = bitmap + static_cast<size_t>(y) * W + x;
    *px = blend(*px, fore, c.op, vis);
}

// ------------------------------------------------------------ pixel I/O
// put_image_data (hpp:3383-3408).
__global__ void k_put(const command *cmd, const uint8_t *__restrict__ pixels, float4 *__restrict__ bitmap, int W,
                      int H, const float *__restrict__ lut) {
    const command &c = *cmd;
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= c.put_w || iy >= c.put_h) return;
    int cx = c.put_x + ix, cy = c.put_y + iy;
    if (cx < 0 || W <= cx || cy < 0 || H <= cy) return;
    const uint8_t *p = pixels + c.put_first + (static_cast<size_t>(iy) * c.put_w + ix) * 4;
    float a = static_cast<float>(p[3]) / 255.0f;
    bitmap[static_cast<size_t>(cy) * W + cx] = make_float4(lut[p[0]] * a, lut[p[1]] * a, lut[p[2]] * a, a);
}

// get_image_data (hpp:3348-3381) into a compact w x h RGBA8 buffer.
__global__ void k_get(const float4 *__restrict__ bitmap, int W, int H, uchar4 *__restrict__ out, int w, int h,
                      int x0, int y0) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= w || iy >= h) return;
    int cx = x0 + ix, cy = y0 + iy;
    float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (0 <= cx && cx < W && 0 <= cy && cy < H) c = bitmap[static_cast<size_t>(cy) * W + cx];
    out[static_cast<size_t>(iy) * w + ix] = to_srgb8(c, cx, cy);
}

}  // namespace cyg

#endif
