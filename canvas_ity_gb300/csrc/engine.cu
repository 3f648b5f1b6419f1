// engine.cu -- the GB300 render engine behind include/cy_gpu.h and
// include/cy_batch.h.
//
// A context owns one canvas: the premultiplied linear float RGBA bitmap
// (the reference's `bitmap`, hpp:1171) and its clip masks.  Calls queue
// commands on the host.  A frame executes the queued commands of one or many
// contexts:
//   prepare  pack every queued geometry/paint buffer into one arena and copy
//            it up, flatten all Bezier paths, size every buffer (two small
//            read-backs of counts), then run once;
//   run      device work only, in stream order: flattening, batched scan
//            conversion of every draw / shadow / clip, clip masks level by
//            level, shadow images, then either the strip kernel (tile engine)
//            or per-draw paint launches (plain engine);
//   finish   copy get_image_data results out, release resources.
// After the first run, `run` issues no host synchronisation, so a prepared
// frame can be re-run (the benchmark times exactly that).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <atomic>
#include <chrono>
#include <vector>

#include "../../include/cy_gpu.h"
#include "engine_types.h"
#include "kernels.cuh"
#include "strips.cuh"
#include "stroke.cuh"
#include "encode.hpp"

using namespace cyg;

namespace {

thread_local int g_engine = 0;          // 0 tile (strip) engine, 1 plain per-draw engine
thread_local int g_deferred = 0;        // contexts created now queue their reads
thread_local int g_thread_status = 0;   // first failure in this thread since the last take
int g_strip_pixels = 4096;              // strip size of the tile engine (autotuned)
int g_strip_threads = 256;
// Coverage of the tile engine's draws: 0 binned (fixed-point accumulation in
// shared memory, within the parity tolerance), 1 exact (row-sorted runs, the
// reference's float sums bit for bit).  Read when a frame is prepared.
std::atomic<int> g_coverage{0};
// Binned strips keep 20 B per pixel in shared memory (float4 pixels and an
// int32 accumulation image): at most this many pixels per strip.
constexpr int kBinnedMaxStrip = 9216;
constexpr size_t kMaxStripSmem = 226 * 1024;   // dynamic shared memory of one strip block (of 227 KiB)
// Rows per bin band of a binned canvas W pixels wide: about 2048 pixels.
inline int band_rows(int W) { return std::max(1, 2048 / std::max(1, W)); }

void note_thread_status(int rc) {
    if (rc && g_thread_status == 0) g_thread_status = rc;
}

struct dbuf {
    void *p = nullptr;
    size_t cap = 0;
    // Grow to at least `bytes`; contents are not preserved.
    bool ensure(size_t bytes) {
        if (bytes <= cap && p) return true;
        size_t n = std::max(std::max(bytes, static_cast<size_t>(256)), cap + cap / 2);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, n) != cudaSuccess) { cudaGetLastError(); return false; }
        cap = n;
        return true;
    }
    // Grow to at least `bytes`, keeping the first `keep` bytes (copied on
    // stream s, which is waited for before the old buffer is freed).
    bool grow_keep(size_t bytes, size_t keep, cudaStream_t s) {
        if (bytes <= cap && p) return true;
        size_t n = std::max(std::max(bytes, static_cast<size_t>(256)), cap + cap / 2);
        void *q = nullptr;
        if (cudaMalloc(&q, n) != cudaSuccess) { cudaGetLastError(); return false; }
        if (p && keep && (cudaMemcpyAsync(q, p, std::min(keep, cap), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
                          cudaStreamSynchronize(s) != cudaSuccess)) {
            cudaGetLastError();
            cudaFree(q);
            return false;
        }
        if (p) cudaFree(p);
        p = q;
        cap = n;
        return true;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

struct hbuf {
    void *p = nullptr;
    size_t cap = 0;
    bool ensure(size_t bytes) {
        if (bytes <= cap && p) return true;
        size_t n = std::max(std::max(bytes, static_cast<size_t>(4096)), cap + cap / 2);
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaMallocHost(&p, n) != cudaSuccess) { cudaGetLastError(); return false; }
        cap = n;
        return true;
    }
    void release() { if (p) cudaFreeHost(p); p = nullptr; cap = 0; }
};

// A clip mask: the reference's sparse runs per row plus the dense visibility
// they imply.  Created by a queued clip; its content is made when the frame
// that holds the clip runs.
struct mask_slot {
    float *vis = nullptr;       // W*H
    int32_t *off = nullptr;     // H+1
    int32_t *len = nullptr;     // H+1
    cyg::run *runs = nullptr;
    float *sums = nullptr;
    int *last_row = nullptr;    // device int: last row holding runs
    int64_t cap = 0;            // run capacity (0 until sized)
    int refs = 0;
    void free_all() {
        cudaFree(vis); cudaFree(off); cudaFree(len); cudaFree(runs); cudaFree(sums); cudaFree(last_row);
        vis = nullptr; off = nullptr; len = nullptr; runs = nullptr; sums = nullptr; last_row = nullptr;
        cap = 0;
    }
};

const float *linear_lut_host() {
    // linearized(i / 255) of the reference (hpp:1273-1278), with host powf.
    static float lut[256];
    static std::once_flag once;
    std::call_once(once, [] {
        for (int i = 0; i < 256; ++i) {
            float v = static_cast<float>(i) / 255.0f;
            lut[i] = v < 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
        }
    });
    return lut;
}

// get_image_data's colour byte (hpp:3348-3381, delinearized at hpp:1287-1289)
// for clamped value u under Bayer threshold t, with host powf.
int srgb_byte_host(float u, float t) {
    float s = u < 0.0031308f ? 12.92f * u : 1.055f * powf(u, 1.0f / 2.4f) - 0.055f;
    return static_cast<int>(t + 255.0f * s);
}

// thr[d][q]: the least u in [0, 1] whose byte under Bayer cell d is >= q
// (+inf when none), found by bisection over the float bit patterns; the
// byte only grows with u, so the byte of u is the count of q >= 1 with
// thr[d][q] <= u.
const float *srgb_thresholds_host() {
    static float thr[16][256];
    static std::once_flag once;
    std::call_once(once, [] {
        static const float bayer[16] = {0.03125f, 0.53125f, 0.15625f, 0.65625f, 0.78125f, 0.28125f,
                                        0.90625f, 0.40625f, 0.21875f, 0.71875f, 0.09375f, 0.59375f,
                                        0.96875f, 0.46875f, 0.84375f, 0.34375f};
        for (int d = 0; d < 16; ++d) {
            thr[d][0] = 0.0f;
            for (int q = 1; q < 256; ++q) {
                uint32_t lo_b = 0, hi_b = 0x3f800000u;   // bit patterns of 0 and 1
                float one = 1.0f;
                if (srgb_byte_host(one, bayer[d]) < q) {
                    thr[d][q] = INFINITY;
                    continue;
                }
                while (lo_b < hi_b) {   // least pattern whose byte reaches q
                    uint32_t mid = lo_b + (hi_b - lo_b) / 2;
                    float u;
                    std::memcpy(&u, &mid, 4);
                    if (srgb_byte_host(u, bayer[d]) >= q) hi_b = mid; else lo_b = mid + 1;
                }
                std::memcpy(&thr[d][q], &lo_b, 4);
            }
        }
    });
    return &thr[0][0];
}

// Upload the threshold table to the current device once.
int ensure_srgb_table() {
    static std::mutex lock;
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return CY_ENODEV; }
    std::lock_guard<std::mutex> hold(lock);
    if (done[dev]) return CY_OK;
    if (cudaMemcpyToSymbol(g_srgb_thr, srgb_thresholds_host(), sizeof(float) * 16 * 256) != cudaSuccess) {
        cudaGetLastError();
        return CY_ECUDA;
    }
    done[dev] = true;
    return CY_OK;
}

inline size_t align256(size_t v) { return (v + 255) & ~static_cast<size_t>(255); }

// Run fn(i) for i < n on up to 16 host threads (inline for small n).
template <class Fn>
void parallel_for(size_t n, Fn fn) {
    int threads = static_cast<int>(std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 16));
    if (n < 64 || threads <= 1) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<size_t> next(0);
    auto work = [&]() {
        for (size_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) fn(i);
    };
    std::vector<std::thread> pool;
    try {
        for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    } catch (...) {
    }
    work();
    for (std::thread &t : pool) t.join();
}

// Canvas buffers are recycled through a per-device pool of size classes
// (steps of 1/4 of a power of two), so replaying canvases does not call
// cudaMalloc/cudaFree (which synchronises the device) for each of them.
struct canvas_pool {
    std::mutex m;
    std::vector<std::pair<size_t, void *>> free;   // (class bytes, buffer)
    size_t pooled = 0;
};
constexpr size_t kPoolCap = size_t(16) << 30;
canvas_pool g_pools[64];

size_t pool_class(size_t bytes) {
    size_t c = 256;
    while (c < bytes) c <<= 1;
    size_t q = c / 8;   // candidates 5/8, 6/8, 7/8, 8/8 of the power of two
    for (size_t k = 5; k <= 8; ++k)
        if (q * k >= bytes) return q * k;
    return c;
}

void *pool_get(size_t bytes, size_t *got) {
    int dev = 0;
    cudaGetDevice(&dev);
    size_t cls = pool_class(bytes);
    *got = cls;
    if (dev >= 0 && dev < 64) {
        canvas_pool &p = g_pools[dev];
        std::lock_guard<std::mutex> hold(p.m);
        for (size_t i = 0; i < p.free.size(); ++i)
            if (p.free[i].first == cls) {
                void *b = p.free[i].second;
                p.free[i] = p.free.back();
                p.free.pop_back();
                p.pooled -= cls;
                return b;
            }
    }
    void *b = nullptr;
    if (cudaMalloc(&b, cls) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return b;
}

void pool_put(void *b, size_t cls) {
    if (!b) return;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64) {
        canvas_pool &p = g_pools[dev];
        std::lock_guard<std::mutex> hold(p.m);
        if (p.pooled + cls <= kPoolCap) {
            p.free.emplace_back(cls, b);
            p.pooled += cls;
            return;
        }
    }
    cudaFree(b);
}

// Host-side queue of one context.
struct queue {
    std::vector<command> cmds;
    std::vector<int32_t> mask_ids;  // per command: mask_in id, mask_out id
    std::vector<float2> host_pts;
    std::vector<int32_t> host_prev;
    std::vector<float2> bez_pts;
    std::vector<flat_item> items;
    std::vector<stroke_group> groups;   // stroked subpaths (device stroke expansion)
    std::vector<stroke_style> styles;
    std::vector<float> dash;
    std::vector<float> stop_off;
    std::vector<float4> stop_col;
    std::vector<uchar4> texels;
    std::vector<uint8_t> put_px;
    std::vector<unsigned char *> get_dst;   // per read: host destination (null: deferred)
    std::vector<int32_t> get_stride;
    size_t bytes = 0;
    int64_t rows = 0;
    int64_t get_bytes = 0;
    bool empty() const { return cmds.empty(); }
    void clear() {
        cmds.clear(); mask_ids.clear(); host_pts.clear(); host_prev.clear(); bez_pts.clear(); items.clear();
        groups.clear(); styles.clear(); dash.clear();
        stop_off.clear(); stop_col.clear(); texels.clear(); put_px.clear(); get_dst.clear(); get_stride.clear();
        bytes = 0; rows = 0; get_bytes = 0;
    }
};

}  // namespace

struct cy_ctx {
    int W = 0, H = 0;
    int device = 0;             // the device the canvas and its stream live on
    int status = 0;
    int engine = 0;
    bool deferred = false;
    bool has_content = false;   // bitmap holds more than transparent black
    bool transient = false;     // destroyed right after its frame: the tile engine keeps no float pixels
    cudaStream_t stream = nullptr;
    float4 *bitmap = nullptr;
    size_t bitmap_bytes = 0;        // size class of the pooled buffer
    std::vector<mask_slot> masks;   // id 0 unused (whole canvas)
    std::vector<mask_slot> dead;    // released masks, freed at the next frame
    queue q;
    std::vector<uint8_t> deferred_out;   // results of deferred reads
    void *cached_frame = nullptr;        // frame reused by this context's flushes
    int fail(int rc, int line = 0) {
        if (status == 0) {
            status = rc;
            if (std::getenv("CY_DEBUG")) std::fprintf(stderr, "canvas_ity_gb300: frame failed with %d (engine.cu:%d)\n", rc, line);
        }
        note_thread_status(rc);
        return rc;
    }
};

// ------------------------------------------------------------------ frame
struct frame {
    cudaStream_t stream = nullptr;
    int engine = 0;
    int status = 0;
    std::vector<cy_ctx *> cvs;
    // combined host data
    queue all;                 // commands and reads of all contexts (geometry stays in their queues)
    struct ctx_base { int32_t hpts, bez, items, stop, tex, groups, styles, dash; int64_t put; };
    std::vector<ctx_base> bases;   // where each context's geometry lands in the arena
    std::vector<int64_t> get_base; // where each context's reads start in the read-back buffer
    bool keep_reads = false;       // finish leaves deferred reads in get_host
    int64_t n_hpts = 0, n_bez = 0, n_items_all = 0, n_stop = 0, n_tex = 0, n_put = 0;
    int64_t n_groups = 0, n_styles = 0, n_dash = 0;
    // Device stroke expansion: flattened centre lines occupy flat_pts[0,
    // nflat), the outlines follow at nflat; dashed centre lines are apart.
    int64_t nflat = 0, n_outline = 0, n_dashed = 0, n_pieces = 0, n_chunks = 0, n_jpos = 0;
    bool any_dash = false;
    // The sizing in prepare() flattened the centre lines and ran every stroke
    // pass up to the outline counts; the first run then only writes the
    // outlines (later runs redo everything).
    bool geometry_ready = false;
    int stroke_write();
    std::vector<int32_t> cmd_cv;
    int64_t get_total = 0;
    std::vector<scan_job> jobs;
    std::vector<int32_t> main_job, shadow_job;
    std::vector<cyg::shadow_job> sjobs;
    int64_t shadow_floats = 0;
    std::vector<strip_cmd> ext;
    std::vector<strip_canvas> scv;
    std::vector<int2> items_host;
    struct clip_op { int cmd; int cv; int in_id, out_id; int level; };
    std::vector<clip_op> clips;
    int max_level = -1;
    int64_t total_rows = 0, total_segs = 0;
    // Run jobs scanned straight from their polylines (tab_nc), binned jobs
    // (tab_bn, every segment clipped on its own) and run jobs that go through
    // the clip passes first (tab_cl): (first point, job index).
    std::vector<int2> tab_nc, tab_bn, tab_cl;
    std::vector<int32_t> bn_idx;   // tab_bn's block index (job_entry)
    int64_t nc_segs = 0, bn_segs = 0, cl_points = 0;
    int64_t pass_n[5] = {};    // clip pass sizes (input of pass 0 .. output of pass 3)
    int n_items = 0;
    int strip_pixels = 4096;
    // Binned coverage (tile engine): draws' segments go to row-band bins.
    bool binned = false;
    int64_t n_bins = 0, n_bin_entries = 0;
    // device
    dbuf arena, flat_pts, flat_prev, item_cnt, item_off, pat_f4, jobs_dev, boxes;
    dbuf row_cnt, row_off, row_cur, row_len, row_meta, long_rows, n_long, runs, sums;
    dbuf bin_cnt, bin_cur, bin_off, bin_seg, clip_dev;
    dbuf tabs_dev, cp_cnt, cp_off, cp_pts[2], cp_prev[2], cp_job[2];
    dbuf sj_dev, sh_img, sh_scratch, rects, scv_dev, items_dev, ext_dev, counter, get_dev, lut_dev;
    dbuf dash_cnt, dash_off, dash_pts, dash_subs, dash_nsub, dash_st, st_err, pc_cnt, pc_base, pc_list, wk_cnt, wk_base,
        wk_chunks, jn_cnt, jn_alpha, jn_sum, jn_off, jn_pbase, jn_pchunk, st_goff;
    hbuf staging, offs_host, rowoff_host, get_host, stoff_host, binoff_host;
    char *d = nullptr;
    size_t o_cmd = 0, o_hpts = 0, o_hprev = 0, o_bez = 0, o_items = 0, o_soff = 0, o_scol = 0, o_tex = 0, o_put = 0;
    size_t o_groups = 0, o_styles = 0, o_dash = 0;
    stroke_in stroke_args() const;
    int stroke_passes(bool sizing);
    bool sized = false;        // run store and masks sized by the first run
    int64_t n_runs = 0, main_runs = 0, main_rows = 0, h2d_bytes = 0;
    int launches = 0;          // kernel launches of the last run
    bool profiling = false;
    cudaEvent_t ev[8] = {};
    int n_ev = 0;
    void mark() {
        if (profiling && n_ev < 8) cudaEventRecord(ev[n_ev++], stream);
    }
    bool ext_built = false;
    bool strips_built = false;
    bool clips_built = false;                 // clip_dev holds the clip masks' arguments
    std::vector<clip_args> clip_host;
    std::vector<int> level_first, level_max_h;   // clips of each nesting level in clip_host
    int strip_threads = 256;
    cudaGraphExec_t graph_exec = nullptr;   // captured device-only run (after sizing)
    // inputs of the strip launch, kept by run() so the paint stage can be
    // launched again on its own (autotuning)
    row_view last_rv;
    paint_src last_src;
    const command *last_cmds = nullptr;
    const uint8_t *last_put = nullptr;
    const float *last_lut = nullptr;
    int launch_strips();
    int build_strips();
    // The strip kernel instance for the frame's coverage and block size, and
    // its shared memory: 16 B per pixel, 24 B when binned.
    using strip_fn = void (*)(strip_params);
    strip_fn strip_kernel() const {
        if (binned)
            return strip_threads == 128 ? k_strips<128, true> : strip_threads == 512 ? k_strips<512, true>
                                                                                      : k_strips<256, true>;
        return strip_threads == 128 ? k_strips<128, false> : strip_threads == 512 ? k_strips<512, false>
                                                                                   : k_strips<256, false>;
    }
    // Shared memory of a strip: 16 B per pixel; binned adds an int32 per
    // pixel and a chunk mask per row.
    int strip_cap = 0, strip_words = 0;   // pixels of the largest strip, words of its chunk marks
    size_t strip_smem() const {
        if (!binned) return static_cast<size_t>(strip_cap) * sizeof(float4);
        return static_cast<size_t>(strip_cap) * (sizeof(float4) + sizeof(int32_t)) +
               static_cast<size_t>(strip_words) * sizeof(uint32_t);
    }
    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
    }

    // Forget the previous frame's commands but keep its device buffers.
    void reset() {
        drop_graph();
        status = 0;
        cvs.clear();
        all.clear();
        bases.clear();
        get_base.clear();
        keep_reads = false;
        n_hpts = n_bez = n_items_all = n_stop = n_tex = n_put = 0;
        n_groups = n_styles = n_dash = 0;
        nflat = n_outline = n_dashed = n_pieces = n_chunks = n_jpos = 0;
        any_dash = false;
        geometry_ready = false;
        cmd_cv.clear();
        get_total = 0;
        jobs.clear();
        main_job.clear();
        shadow_job.clear();
        sjobs.clear();
        shadow_floats = 0;
        ext.clear();
        scv.clear();
        items_host.clear();
        clips.clear();
        max_level = -1;
        total_rows = total_segs = 0;
        tab_nc.clear();
        tab_bn.clear();
        tab_cl.clear();
        nc_segs = bn_segs = cl_points = 0;
        for (int64_t &v : pass_n) v = 0;
        n_items = 0;
        binned = false;
        n_bins = n_bin_entries = 0;
        sized = ext_built = strips_built = clips_built = false;
        n_runs = main_runs = main_rows = h2d_bytes = 0;
    }

    ~frame() {
        drop_graph();
        for (cudaEvent_t e : ev) if (e) cudaEventDestroy(e);
        dbuf *b[] = {&arena, &flat_pts, &flat_prev, &item_cnt, &item_off, &pat_f4, &jobs_dev, &boxes, &row_cnt,
                     &row_off, &row_cur, &row_len, &row_meta, &long_rows, &n_long, &runs, &sums, &tabs_dev, &cp_cnt, &cp_off,
                     &cp_pts[0], &cp_pts[1], &cp_prev[0], &cp_prev[1], &cp_job[0], &cp_job[1], &sj_dev, &sh_img, &sh_scratch, &rects,
                     &scv_dev, &items_dev, &ext_dev, &counter, &get_dev, &lut_dev, &dash_cnt, &dash_off, &dash_pts,
                     &dash_subs, &dash_nsub, &dash_st, &st_err, &pc_cnt, &pc_base, &pc_list, &wk_cnt, &wk_base, &wk_chunks, &jn_cnt,
                     &jn_alpha, &jn_sum, &jn_off, &jn_pbase, &jn_pchunk, &st_goff, &bin_cnt, &bin_cur, &bin_off, &bin_seg, &clip_dev};
        for (dbuf *x : b) x->release();
        staging.release();
        stoff_host.release();
        binoff_host.release();
        offs_host.release();
        rowoff_host.release();
        get_host.release();
    }
    int fail(int rc, int line = 0) {
        if (status == 0) {
            status = rc;
            if (std::getenv("CY_DEBUG")) std::fprintf(stderr, "canvas_ity_gb300: frame failed with %d (engine.cu:%d)\n", rc, line);
        }
        for (cy_ctx *c : cvs) c->fail(rc);
        note_thread_status(rc);
        return rc;
    }
    bool ok(cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        if (std::getenv("CY_DEBUG")) std::fprintf(stderr, "canvas_ity_gb300: CUDA error %s\n", cudaGetErrorString(e));
        fail(e == cudaErrorMemoryAllocation ? CY_ENOMEM : CY_ECUDA);
        return false;
    }
    int scan(const int32_t *in, int32_t *out, int n);
    template <class In> int scan64(const In *in, int64_t *out, int n);
    int clip_passes(job_tables &t);
    void gather();
    void stage(char *h);
    int prepare();
    int run();
    int finish();
};

int frame::scan(const int32_t *in, int32_t *out, int n) {
    // Exclusive scan with recursion over tile sums.
    int tiles = (n + 4095) / 4096;
    if (tiles <= 0) return CY_OK;
    if (tiles == 1) {
        k_scan_tiles<<<1, 1024, 0, stream>>>(in, out, n, nullptr);
        return ok(cudaGetLastError()) ? CY_OK : status;
    }
    int32_t *sums_p = nullptr, *offs_p = nullptr;
    if (!ok(cudaMallocAsync(reinterpret_cast<void **>(&sums_p), static_cast<size_t>(tiles) * 4, stream)) ||
        !ok(cudaMallocAsync(reinterpret_cast<void **>(&offs_p), static_cast<size_t>(tiles) * 4, stream)))
        return status;
    k_scan_tiles<<<tiles, 1024, 0, stream>>>(in, out, n, sums_p);
    int rc = scan(sums_p, offs_p, tiles);
    if (rc == CY_OK) k_scan_add<<<(n + 255) / 256, 256, 0, stream>>>(out, n, offs_p);
    cudaFreeAsync(sums_p, stream);
    cudaFreeAsync(offs_p, stream);
    if (rc == CY_OK && !ok(cudaGetLastError())) rc = status;
    return rc;
}

// Kernels one tiled scan of n entries launches (4096 entries per tile).
static int scan_launch_count(int64_t n) {
    int c = 1;
    while (n > 4096) {
        n = (n + 4095) / 4096;
        c += 2;
    }
    return c;
}

// The reference's Sutherland-Hodgman clip of the jobs that need it
// (hpp:2204-2235): four passes over the polygons of all such jobs, each a
// count, a scan and an emit.  The first run reads every pass's size back to
// size the buffers; later runs of the same frame reuse them.
int frame::clip_passes(job_tables &t) {
    if (pass_n[0] <= 0) {
        pass_n[4] = 0;
        return CY_OK;
    }
    clip_pass P;
    std::memset(&P, 0, sizeof(P));
    P.jobs = jobs_dev.as<scan_job>();
    P.tab = tabs_dev.as<int2>() + tab_nc.size() + tab_bn.size();
    P.n_tab = static_cast<int>(tab_cl.size());
    P.src_pts[0] = t.pts[0];
    P.src_pts[1] = t.pts[1];
    P.src_prev[0] = t.prev[0];
    P.src_prev[1] = t.prev[1];
    for (int e = 0; e < 4; ++e) {
        int64_t n = pass_n[e];
        if (n > INT32_MAX / 2) return fail(CY_ENOMEM, __LINE__);
        P.n = static_cast<int>(n);
        P.edge = e;
        if (!sized && (!cp_cnt.ensure(static_cast<size_t>(n + 1) * 4) || !cp_off.ensure(static_cast<size_t>(n + 1) * 4)))
            return fail(CY_ENOMEM, __LINE__);
        P.cnt = cp_cnt.as<int32_t>();
        P.off = cp_off.as<int32_t>();
        if (e > 0) {
            int in = (e - 1) & 1;
            P.in_pts = cp_pts[in].as<float2>();
            P.in_prev = cp_prev[in].as<int32_t>();
            P.in_job = cp_job[in].as<int32_t>();
        }
        int grid = std::max(1, static_cast<int>(std::min<int64_t>((n + 1 + 255) / 256, 152 * 32)));
        if (n > 0) {
            if (e == 0) k_clip_count<true><<<grid, 256, 0, stream>>>(P);
            else k_clip_count<false><<<grid, 256, 0, stream>>>(P);
            int rc = scan(P.cnt, cp_off.as<int32_t>(), static_cast<int>(n) + 1);
            if (rc) return rc;
            launches += 1 + scan_launch_count(n + 1);
        }
        if (!sized) {
            int32_t total = 0;
            if (n > 0 && (!ok(cudaMemcpyAsync(&total, cp_off.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, stream)) ||
                          !ok(cudaStreamSynchronize(stream))))
                return status;
            if (total < 0 || total > INT32_MAX / 2) return fail(CY_ENOMEM, __LINE__);
            pass_n[e + 1] = total;
            int out = e & 1;
            size_t m = static_cast<size_t>(total) + 1;
            if (!cp_pts[out].ensure(m * sizeof(float2)) || !cp_prev[out].ensure(m * 4) || !cp_job[out].ensure(m * 4))
                return fail(CY_ENOMEM, __LINE__);
        }
        int out = e & 1;
        P.out_pts = cp_pts[out].as<float2>();
        P.out_prev = cp_prev[out].as<int32_t>();
        P.out_job = cp_job[out].as<int32_t>();
        if (n > 0) {
            if (e == 0) {
                k_clip_emit<true><<<grid, 256, 0, stream>>>(P);
                k_clip_link<true><<<grid, 256, 0, stream>>>(P);
            } else {
                k_clip_emit<false><<<grid, 256, 0, stream>>>(P);
                k_clip_link<false><<<grid, 256, 0, stream>>>(P);
            }
            launches += 2;
        }
    }
    t.cl_pts = cp_pts[1].as<float2>();
    t.cl_prev = cp_prev[1].as<int32_t>();
    t.cl_job = cp_job[1].as<int32_t>();
    return ok(cudaGetLastError()) ? CY_OK : status;
}

template <class In>
int frame::scan64(const In *in, int64_t *out, int n) {
    // Exclusive scan of counts into int64 offsets, recursing over tile sums.
    int tiles = (n + 4095) / 4096;
    if (tiles <= 0) return CY_OK;
    if (tiles == 1) {
        k_scan_tiles64<In><<<1, 1024, 0, stream>>>(in, out, n, nullptr);
        return ok(cudaGetLastError()) ? CY_OK : status;
    }
    int64_t *sums_p = nullptr, *offs_p = nullptr;
    if (!ok(cudaMallocAsync(reinterpret_cast<void **>(&sums_p), static_cast<size_t>(tiles) * 8, stream)) ||
        !ok(cudaMallocAsync(reinterpret_cast<void **>(&offs_p), static_cast<size_t>(tiles) * 8, stream)))
        return status;
    k_scan_tiles64<In><<<tiles, 1024, 0, stream>>>(in, out, n, sums_p);
    int rc = scan64<int64_t>(sums_p, offs_p, tiles);
    if (rc == CY_OK) k_scan_add64<<<(n + 255) / 256, 256, 0, stream>>>(out, n, offs_p);
    cudaFreeAsync(sums_p, stream);
    cudaFreeAsync(offs_p, stream);
    if (rc == CY_OK && !ok(cudaGetLastError())) rc = status;
    return rc;
}

// Concatenate the queues of every canvas of the frame, rebasing indices.
void frame::gather() {
    bases.resize(cvs.size());
    for (size_t ci = 0; ci < cvs.size(); ++ci) {
        queue &q = cvs[ci]->q;
        ctx_base &b = bases[ci];
        b.hpts = static_cast<int32_t>(n_hpts);
        b.bez = static_cast<int32_t>(n_bez);
        b.items = static_cast<int32_t>(n_items_all);
        b.stop = static_cast<int32_t>(n_stop);
        b.tex = static_cast<int32_t>(n_tex);
        b.put = n_put;
        b.groups = static_cast<int32_t>(n_groups);
        b.styles = static_cast<int32_t>(n_styles);
        b.dash = static_cast<int32_t>(n_dash);
        n_groups += static_cast<int64_t>(q.groups.size());
        n_styles += static_cast<int64_t>(q.styles.size());
        n_dash += static_cast<int64_t>(q.dash.size());
        n_hpts += static_cast<int64_t>(q.host_pts.size());
        n_bez += static_cast<int64_t>(q.bez_pts.size());
        n_items_all += static_cast<int64_t>(q.items.size());
        n_stop += static_cast<int64_t>(q.stop_off.size());
        n_tex += static_cast<int64_t>(q.texels.size());
        n_put += static_cast<int64_t>(q.put_px.size());
        for (size_t k = 0; k < q.cmds.size(); ++k) {
            command c = q.cmds[k];
            if (c.kind == CMD_FILL || c.kind == CMD_CLIP) {
                c.first += c.geom == 0 ? b.hpts : c.geom == 1 ? b.items : b.groups;
                c.stop_first += b.stop;
                if (!c.pat_ptr) c.pat_first += b.tex;
            } else if (c.kind == CMD_PUT) {
                c.put_first += b.put;
            } else if (c.kind == CMD_GET) {
                c.get_out += get_total;
            }
            all.cmds.push_back(c);
            cmd_cv.push_back(static_cast<int32_t>(ci));
            all.mask_ids.push_back(q.mask_ids[2 * k]);
            all.mask_ids.push_back(q.mask_ids[2 * k + 1]);
        }
        all.get_dst.insert(all.get_dst.end(), q.get_dst.begin(), q.get_dst.end());
        all.get_stride.insert(all.get_stride.end(), q.get_stride.begin(), q.get_stride.end());
        get_base.push_back(get_total);
        get_total += q.get_bytes;
    }
}

// Copy every context's geometry, stops, texels and put pixels into the
// staging buffer at its place in the arena, contexts spread over host threads.
void frame::stage(char *h) {
    auto copy_ctx = [&](size_t ci) {
        const queue &q = cvs[ci]->q;
        const ctx_base &b = bases[ci];
        if (!q.host_pts.empty())
            std::memcpy(h + o_hpts + static_cast<size_t>(b.hpts) * sizeof(float2), q.host_pts.data(),
                        q.host_pts.size() * sizeof(float2));
        int32_t *prev = reinterpret_cast<int32_t *>(h + o_hprev) + b.hpts;
        for (size_t k = 0; k < q.host_prev.size(); ++k) prev[k] = q.host_prev[k] + b.hpts;
        if (!q.bez_pts.empty())
            std::memcpy(h + o_bez + static_cast<size_t>(b.bez) * sizeof(float2), q.bez_pts.data(),
                        q.bez_pts.size() * sizeof(float2));
        flat_item *items = reinterpret_cast<flat_item *>(h + o_items) + b.items;
        for (size_t k = 0; k < q.items.size(); ++k) {
            flat_item it = q.items[k];
            it.pt += b.bez;
            if (it.sub_end >= 0) it.sub_end += b.items;
            items[k] = it;
        }
        stroke_group *groups = reinterpret_cast<stroke_group *>(h + o_groups) + b.groups;
        for (size_t k = 0; k < q.groups.size(); ++k) {
            stroke_group g = q.groups[k];
            g.head += b.items;
            g.end += b.items;
            g.style += b.styles;
            groups[k] = g;
        }
        stroke_style *styles = reinterpret_cast<stroke_style *>(h + o_styles) + b.styles;
        for (size_t k = 0; k < q.styles.size(); ++k) {
            stroke_style st = q.styles[k];
            st.dash_first += b.dash;
            styles[k] = st;
        }
        if (!q.dash.empty())
            std::memcpy(h + o_dash + static_cast<size_t>(b.dash) * sizeof(float), q.dash.data(),
                        q.dash.size() * sizeof(float));
        if (!q.stop_off.empty()) {
            std::memcpy(h + o_soff + static_cast<size_t>(b.stop) * sizeof(float), q.stop_off.data(),
                        q.stop_off.size() * sizeof(float));
            std::memcpy(h + o_scol + static_cast<size_t>(b.stop) * sizeof(float4), q.stop_col.data(),
                        q.stop_col.size() * sizeof(float4));
        }
        if (!q.texels.empty())
            std::memcpy(h + o_tex + static_cast<size_t>(b.tex) * sizeof(uchar4), q.texels.data(),
                        q.texels.size() * sizeof(uchar4));
        if (!q.put_px.empty())
            std::memcpy(h + o_put + static_cast<size_t>(b.put), q.put_px.data(), q.put_px.size());
    };
    parallel_for(cvs.size(), copy_ctx);
}

// Whether a job's points (command bounds moved by the job's offset) can fall
// outside [0, wd] x [0, ht].  Inside, the reference's Sutherland-Hodgman
// pass returns the polygon unchanged, so the clip passes are skipped; the one
// pixel margin covers the rounding of flattening and of adding the offset.
static bool needs_clip(const command &c, float wd, float ht, float ox, float oy) {
    if (c.gx0 <= -1000000000 || c.gy0 <= -1000000000 || c.gx1 >= 1000000000 || c.gy1 >= 1000000000) return true;
    double x0 = static_cast<double>(c.gx0) + ox, x1 = static_cast<double>(c.gx1) + ox;
    double y0 = static_cast<double>(c.gy0) + oy, y1 = static_cast<double>(c.gy1) + oy;
    return !(x0 >= 1.0 && y0 >= 1.0 && x1 <= static_cast<double>(wd) - 1.0 && y1 <= static_cast<double>(ht) - 1.0);
}

stroke_in frame::stroke_args() const {
    stroke_in si;
    si.flat = flat_pts.as<float2>();
    si.item_off = item_off.as<int32_t>();
    si.groups = reinterpret_cast<const stroke_group *>(d + o_groups);
    si.styles = reinterpret_cast<const stroke_style *>(d + o_styles);
    si.dash = reinterpret_cast<const float *>(d + o_dash);
    si.dash_pts = dash_pts.as<float2>();
    si.dash_subs = dash_subs.as<int2>();
    si.dash_off = dash_off.as<int32_t>();
    si.dash_nsub = dash_nsub.as<int32_t>();
    si.dash_state_at = dash_st.as<dash_state>();
    si.nflat = static_cast<int32_t>(nflat);
    si.n = static_cast<int>(n_groups);
    si.error = st_err.as<int32_t>();
    return si;
}

// Stroke expansion: dash (count, scan, write), walks (count, scan, write),
// joins (count, scan, write).  Every run does all of it from the centre
// lines; the first run (`sizing`) reads the sizes back between the steps to
// allocate, and stops before writing the outlines (flat_pts may move).
int frame::stroke_passes(bool sizing) {
    const int ng = static_cast<int>(n_groups);
    const int sgrid = (ng + kStrokeWarps - 1) / kStrokeWarps;
    const size_t gn = static_cast<size_t>(ng) + 2;
    int32_t *hb = static_cast<int32_t *>(stoff_host.p);
    if (sizing) {
        if (!st_err.ensure(4) || !dash_cnt.ensure(gn * 4) || !dash_off.ensure(gn * 4) || !dash_nsub.ensure(gn * 4) ||
            !pc_cnt.ensure(gn * 4) || !pc_base.ensure(gn * 4) || !st_goff.ensure(gn * 8) ||
            !stoff_host.ensure(gn * 8) || !dash_pts.ensure(256) || !dash_subs.ensure(256))
            return fail(CY_ENOMEM, __LINE__);
        hb = static_cast<int32_t *>(stoff_host.p);
        any_dash = false;
        for (cy_ctx *cv : cvs)
            for (const stroke_style &st : cv->q.styles) any_dash = any_dash || st.dash_n > 0;
        // the dash walk's state at every centre-line point (k_dash)
        if (any_dash && !dash_st.ensure(static_cast<size_t>(nflat + 1) * sizeof(dash_state)))
            return fail(CY_ENOMEM, __LINE__);
        if (!ok(cudaMemsetAsync(st_err.p, 0, 4, stream))) return status;
    }
    auto read_back = [&](void *dst, const void *src, size_t bytes) {
        return ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream)) &&
               ok(cudaStreamSynchronize(stream));
    };
    if (any_dash) {
        k_dash<false><<<sgrid, kStrokeWarps * 32, 0, stream>>>(stroke_args(), dash_cnt.as<int32_t>());
        if (!ok(cudaMemsetAsync(dash_cnt.as<int32_t>() + ng, 0, 4, stream))) return status;
        if (int rc = scan(dash_cnt.as<int32_t>(), dash_off.as<int32_t>(), ng + 1)) return rc;
        if (sizing) {
            if (!ok(cudaMemcpyAsync(hb + 1, st_err.p, 4, cudaMemcpyDeviceToHost, stream)) ||
                !read_back(hb, dash_off.as<int32_t>() + ng, 4))
                return status;
            n_dashed = hb[0];
            if (hb[1] != 0 || n_dashed < 0 || nflat + n_dashed > (static_cast<int64_t>(1) << 30))
                return fail(CY_ENOMEM, __LINE__);
            if (!dash_pts.ensure(static_cast<size_t>(n_dashed + 1) * sizeof(float2)) ||
                !dash_subs.ensure(static_cast<size_t>(n_dashed + 1) * sizeof(int2)))
                return fail(CY_ENOMEM, __LINE__);
        }
        k_dash<true><<<sgrid, kStrokeWarps * 32, 0, stream>>>(stroke_args(), nullptr);
        launches += 3 + scan_launch_count(ng + 1);
    }
    // pieces (subpaths after dashing), then their walks' chunks
    const int g256 = (ng + 255) / 256;
    k_piece_count<<<g256, 256, 0, stream>>>(stroke_args(), pc_cnt.as<int32_t>());
    if (!ok(cudaMemsetAsync(pc_cnt.as<int32_t>() + ng, 0, 4, stream))) return status;
    if (int rc = scan(pc_cnt.as<int32_t>(), pc_base.as<int32_t>(), ng + 1)) return rc;
    if (sizing) {
        if (!read_back(hb, pc_base.as<int32_t>() + ng, 4)) return status;
        n_pieces = hb[0];
        if (n_pieces < 0 || n_pieces > (static_cast<int64_t>(1) << 30)) return fail(CY_ENOMEM, __LINE__);
        size_t np1 = static_cast<size_t>(n_pieces) + 1;
        if (!pc_list.ensure(np1 * sizeof(stroke_piece)) || !wk_cnt.ensure(np1 * 4) || !wk_base.ensure(np1 * 4))
            return fail(CY_ENOMEM, __LINE__);
    }
    const int npc = static_cast<int>(n_pieces);
    k_pieces<<<g256, 256, 0, stream>>>(stroke_args(), pc_base.as<int32_t>(), pc_list.as<stroke_piece>());
    k_piece_chunks<<<std::max(1, (npc + 255) / 256), 256, 0, stream>>>(stroke_args(), pc_list.as<stroke_piece>(), npc,
                                                                     wk_cnt.as<int32_t>());
    if (!ok(cudaMemsetAsync(wk_cnt.as<int32_t>() + npc, 0, 4, stream))) return status;
    if (int rc = scan(wk_cnt.as<int32_t>(), wk_base.as<int32_t>(), npc + 1)) return rc;
    if (sizing) {
        if (!read_back(hb, wk_base.as<int32_t>() + npc, 4)) return status;
        n_chunks = hb[0];
        // below 2^26 chunks, their packed walk positions (at most 32 each) fit an int32
        if (n_chunks < 0 || n_chunks >= (static_cast<int64_t>(1) << 26)) return fail(CY_ENOMEM, __LINE__);
        size_t nc = static_cast<size_t>(n_chunks) + 1;
        if (!wk_chunks.ensure(nc * sizeof(walk_chunk)) || !jn_sum.ensure(nc * 4) || !jn_pbase.ensure(nc * 4))
            return fail(CY_ENOMEM, __LINE__);
    }
    k_walk<<<std::max(1, (npc + kStrokeWarps - 1) / kStrokeWarps), kStrokeWarps * 32, 0, stream>>>(
        stroke_args(), pc_list.as<stroke_piece>(), npc, wk_base.as<int32_t>(), wk_chunks.as<walk_chunk>());
    const int nch = static_cast<int>(n_chunks);
    // the chunks' walk positions, packed (k_chunk_positions)
    k_chunk_lanes<<<std::max(1, (nch + 255) / 256), 256, 0, stream>>>(wk_chunks.as<walk_chunk>(), nch,
                                                                     jn_sum.as<int32_t>());
    if (!ok(cudaMemsetAsync(jn_sum.as<int32_t>() + nch, 0, 4, stream))) return status;
    if (int rc = scan(jn_sum.as<int32_t>(), jn_pbase.as<int32_t>(), nch + 1)) return rc;
    if (sizing) {
        if (!read_back(hb, jn_pbase.as<int32_t>() + nch, 4)) return status;
        n_jpos = hb[0];
        if (n_jpos < 0 || n_jpos > static_cast<int64_t>(n_chunks) * 32) return fail(CY_ENOMEM, __LINE__);
        size_t np1 = static_cast<size_t>(n_jpos) + 1;
        if (!jn_pchunk.ensure(np1 * 4) || !jn_cnt.ensure(np1 * 4) || !jn_alpha.ensure(np1 * 4) ||
            !jn_off.ensure(np1 * 8))
            return fail(CY_ENOMEM, __LINE__);
    }
    const int njp = static_cast<int>(n_jpos);
    k_chunk_positions<<<std::max(1, (nch + 7) / 8), 256, 0, stream>>>(wk_chunks.as<walk_chunk>(), nch,
                                                                    jn_pbase.as<int32_t>(), jn_pchunk.as<int32_t>());
    const int jgrid = std::max(1, (njp + kStrokeWarps * 32 - 1) / (kStrokeWarps * 32));
    k_join<false><<<jgrid, kStrokeWarps * 32, 0, stream>>>(stroke_args(), wk_chunks.as<walk_chunk>(),
                                                           jn_pbase.as<int32_t>(), jn_pchunk.as<int32_t>(), njp,
                                                           jn_cnt.as<int32_t>(), jn_alpha.as<float>(), nullptr,
                                                           nullptr, nullptr, 0, 0);
    if (!ok(cudaMemsetAsync(jn_cnt.as<int32_t>() + njp, 0, 4, stream))) return status;
    if (int rc = scan64(jn_cnt.as<int32_t>(), jn_off.as<int64_t>(), njp + 1)) return rc;
    k_group_off<<<(ng + 1 + 255) / 256, 256, 0, stream>>>(pc_base.as<int32_t>(), wk_base.as<int32_t>(),
                                                         jn_pbase.as<int32_t>(), jn_off.as<int64_t>(), ng,
                                                         st_goff.as<int64_t>());
    launches += 8 + scan_launch_count(ng + 1) + scan_launch_count(npc + 1) + scan_launch_count(nch + 1) +
                scan_launch_count(njp + 1);
    if (sizing) {
        int64_t *g64 = static_cast<int64_t *>(stoff_host.p);
        int32_t *errp = reinterpret_cast<int32_t *>(g64 + ng + 1);
        if (!ok(cudaMemcpyAsync(errp, st_err.p, 4, cudaMemcpyDeviceToHost, stream)) ||
            !read_back(g64, st_goff.p, static_cast<size_t>(ng + 1) * 8))
            return status;
        int err = *errp;
        n_outline = g64[ng];
        if (err != 0 || n_outline < 0 || nflat + n_outline > (static_cast<int64_t>(1) << 30))
            return fail(CY_ENOMEM, __LINE__);
        // the outlines go after the centre lines, which are kept
        if (!flat_pts.grow_keep(static_cast<size_t>(nflat + n_outline + 1) * sizeof(float2),
                                static_cast<size_t>(nflat) * sizeof(float2), stream) ||
            !flat_prev.grow_keep(static_cast<size_t>(nflat + n_outline + 1) * 4, static_cast<size_t>(nflat) * 4,
                                 stream))
            return fail(CY_ENOMEM, __LINE__);
        geometry_ready = true;
        return ok(cudaGetLastError()) ? CY_OK : status;
    }
    return stroke_write();
}

// The outlines from the counted joins (k_join's write pass).
int frame::stroke_write() {
    const int njp = static_cast<int>(n_jpos);
    const int jgrid = std::max(1, (njp + kStrokeWarps * 32 - 1) / (kStrokeWarps * 32));
    k_join<true><<<jgrid, kStrokeWarps * 32, 0, stream>>>(stroke_args(), wk_chunks.as<walk_chunk>(),
                                                          jn_pbase.as<int32_t>(), jn_pchunk.as<int32_t>(), njp,
                                                          jn_cnt.as<int32_t>(), jn_alpha.as<float>(),
                                                          jn_off.as<int64_t>(),
                                                          flat_pts.as<float2>() + nflat, flat_prev.as<int32_t>() + nflat,
                                                          static_cast<int32_t>(nflat), n_outline);
    ++launches;
    return ok(cudaGetLastError()) ? CY_OK : status;
}

int frame::prepare() {
    if (int rc = ensure_srgb_table()) return fail(rc);
    const bool timing = std::getenv("CY_DEBUG") != nullptr;
    auto t_begin = std::chrono::steady_clock::now();
    auto since = [&](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
    };
    gather();
    std::vector<command> &cmds = all.cmds;
    binned = engine == 0 && g_coverage.load() == 0;
    for (cy_ctx *c : cvs)
        if (c->W > kBinnedMaxStrip) binned = false;   // its strips would not fit in shared memory
    for (cy_ctx *c : cvs) {
        for (auto &m : c->dead) m.free_all();
        c->dead.clear();
    }
    // Arena: everything queued goes up in one copy.
    o_cmd = 0;
    o_hpts = align256(o_cmd + cmds.size() * sizeof(command));
    o_hprev = align256(o_hpts + static_cast<size_t>(n_hpts) * sizeof(float2));
    o_bez = align256(o_hprev + static_cast<size_t>(n_hpts) * sizeof(int32_t));
    o_items = align256(o_bez + static_cast<size_t>(n_bez) * sizeof(float2));
    o_groups = align256(o_items + static_cast<size_t>(n_items_all) * sizeof(flat_item));
    o_styles = align256(o_groups + static_cast<size_t>(n_groups) * sizeof(stroke_group));
    o_dash = align256(o_styles + static_cast<size_t>(n_styles) * sizeof(stroke_style));
    o_soff = align256(o_dash + static_cast<size_t>(n_dash) * sizeof(float));
    o_scol = align256(o_soff + static_cast<size_t>(n_stop) * sizeof(float));
    o_tex = align256(o_scol + static_cast<size_t>(n_stop) * sizeof(float4));
    o_put = align256(o_tex + static_cast<size_t>(n_tex) * sizeof(uchar4));
    size_t total = align256(o_put + static_cast<size_t>(n_put));
    if (n_hpts > INT32_MAX / 2 || n_bez > INT32_MAX / 2 || n_items_all > INT32_MAX / 2 || n_stop > INT32_MAX / 2 ||
        n_tex > INT32_MAX / 2 || n_groups > INT32_MAX / 2 || n_styles > INT32_MAX / 2 || n_dash > INT32_MAX / 2)
        return fail(CY_ENOMEM, __LINE__);
    if (!arena.ensure(total) || !staging.ensure(total)) return fail(CY_ENOMEM, __LINE__);
    char *h = static_cast<char *>(staging.p);
    stage(h);
    d = static_cast<char *>(arena.p);
    if (total > o_hpts && !ok(cudaMemcpyAsync(d + o_hpts, h + o_hpts, total - o_hpts, cudaMemcpyHostToDevice, stream)))
        return status;
    h2d_bytes = static_cast<int64_t>(total);
    if (!lut_dev.ensure(256 * sizeof(float))) return fail(CY_ENOMEM, __LINE__);
    if (!ok(cudaMemcpyAsync(lut_dev.p, linear_lut_host(), 256 * sizeof(float), cudaMemcpyHostToDevice, stream)))
        return status;
    double t_staged = timing ? since(t_begin) : 0.0;
    // Flattening counts size the polyline store (one read-back).
    int n_items = static_cast<int>(n_items_all);
    const int32_t *offs_h = nullptr;
    if (n_items > 0) {
        if (!item_cnt.ensure(static_cast<size_t>(n_items + 1) * 4) ||
            !item_off.ensure(static_cast<size_t>(n_items + 1) * 4) ||
            !offs_host.ensure(static_cast<size_t>(n_items + 1) * 4))
            return fail(CY_ENOMEM, __LINE__);
        const float2 *d_bez = reinterpret_cast<const float2 *>(d + o_bez);
        const flat_item *d_items = reinterpret_cast<const flat_item *>(d + o_items);
        k_flat_count<<<(n_items + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items, item_cnt.as<int32_t>());
        if (!ok(cudaMemsetAsync(item_cnt.as<int32_t>() + n_items, 0, 4, stream))) return status;
        int rc = scan(item_cnt.as<int32_t>(), item_off.as<int32_t>(), n_items + 1);
        if (rc) return rc;
        if (!ok(cudaMemcpyAsync(offs_host.p, item_off.p, static_cast<size_t>(n_items + 1) * 4,
                                cudaMemcpyDeviceToHost, stream)) ||
            !ok(cudaStreamSynchronize(stream)))
            return status;
        offs_h = static_cast<const int32_t *>(offs_host.p);
        nflat = offs_h[n_items];
        if (nflat < 0 || nflat > (static_cast<int64_t>(1) << 30)) return fail(CY_ENOMEM, __LINE__);
        if (!flat_pts.ensure(static_cast<size_t>(nflat + 1) * sizeof(float2)) ||
            !flat_prev.ensure(static_cast<size_t>(nflat + 1) * 4))
            return fail(CY_ENOMEM, __LINE__);
        if (n_groups > 0) {
            // the stroke passes read the centre lines: flatten them now
            const float2 *d_bez = reinterpret_cast<const float2 *>(d + o_bez);
            const flat_item *d_items = reinterpret_cast<const flat_item *>(d + o_items);
            k_flat_emit<<<(n_items + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items, item_off.as<int32_t>(),
                                                                    flat_pts.as<float2>(), flat_prev.as<int32_t>(),
                                                                    nflat);
            if (int rc = stroke_passes(true)) return rc;
        }
    }
    const int64_t *stoff_h = static_cast<const int64_t *>(stoff_host.p);
    for (command &c : cmds) {
        if (c.kind != CMD_FILL && c.kind != CMD_CLIP) continue;
        if (c.geom == 0) {
            c.line_first = c.first;
            c.line_count = c.count;
        } else if (c.geom == 2) {
            c.line_first = c.count > 0 ? static_cast<int32_t>(nflat + stoff_h[c.first]) : 0;
            c.line_count = c.count > 0 ? static_cast<int32_t>(stoff_h[c.first + c.count] - stoff_h[c.first]) : 0;
        } else if (c.count == 0 || !offs_h) {
            c.line_first = 0;
            c.line_count = 0;
        } else {
            c.line_first = offs_h[c.first];
            c.line_count = offs_h[c.first + c.count] - c.line_first;
        }
    }
    if (!cmds.empty()) {
        std::memcpy(h + o_cmd, cmds.data(), cmds.size() * sizeof(command));
        if (!ok(cudaMemcpyAsync(d + o_cmd, h + o_cmd, cmds.size() * sizeof(command), cudaMemcpyHostToDevice,
                                stream)))
            return status;
    }
    // Scan-conversion jobs: shadow pass (padded canvas) and main pass of each
    // draw, and the path of each clip.
    // A binned job (a draw's own coverage on the tile engine) gets row-band
    // bins instead of rows of runs.
    auto add_job = [&](const command &c, int rows_n, int cols_n, float wd, float ht, float ox, float oy,
                       bool to_bins = false) {
        scan_job j;
        std::memset(&j, 0, sizeof(j));
        j.geom = c.geom;
        j.line_first = c.line_first;
        j.seg_count = c.line_count;
        // binned coverage clips each segment on its own in k_bin: no
        // polygon passes
        j.clip = !to_bins && needs_clip(c, wd, ht, ox, oy) ? 1 : 0;
        j.rows = rows_n;
        j.cols = cols_n;
        j.width = wd;
        j.height = ht;
        j.offx = ox;
        j.offy = oy;
        if (to_bins) {
            j.binned = 1;
            j.band_h = band_rows(cols_n - 2);
            j.bin_base = static_cast<int32_t>(n_bins);
            n_bins += (rows_n + j.band_h - 1) / j.band_h;
        } else {
            j.row_base = static_cast<int32_t>(total_rows);
            total_rows += rows_n;
        }
        total_segs += c.line_count;
        jobs.push_back(j);
        return static_cast<int>(jobs.size()) - 1;
    };
    main_job.assign(cmds.size(), -1);
    shadow_job.assign(cmds.size(), -1);
    std::vector<int> level_of_cv(cvs.size(), 0);
    for (size_t i = 0; i < cmds.size(); ++i) {
        const command &c = cmds[i];
        const cy_ctx *cv = cvs[cmd_cv[i]];
        int W = cv->W, H = cv->H;
        if (c.kind == CMD_FILL && c.shadow) {
            int b = c.sh_border;
            int ew = W + 2 * b, eh = H + 2 * b;
            shadow_job[i] = add_job(c, eh, ew + 2, static_cast<float>(ew), static_cast<float>(eh), c.sh_offx,
                                    c.sh_offy);
            jobs[shadow_job[i]].need_box = 1;
            cyg::shadow_job s;
            std::memset(&s, 0, sizeof(s));
            s.cmd = static_cast<int32_t>(i);
            s.job = shadow_job[i];
            s.row_base = jobs[shadow_job[i]].row_base;
            s.W = W;
            s.H = H;
            s.border = b;
            s.img = shadow_floats;
            s.radius = c.sh_radius;
            s.w1 = c.sh_w1;
            s.w2 = c.sh_w2;
            shadow_floats += static_cast<int64_t>(ew + 1) * eh;
            sjobs.push_back(s);
        }
        if (c.kind == CMD_FILL || c.kind == CMD_CLIP)
            main_job[i] = add_job(c, H, W + 2, static_cast<float>(W), static_cast<float>(H), 0.0f, 0.0f,
                                  binned && c.kind == CMD_FILL);
        if (c.kind == CMD_CLIP) jobs[main_job[i]].need_box = 1;
        if (c.kind == CMD_CLIP) {
            int lv = level_of_cv[cmd_cv[i]]++;
            clips.push_back(clip_op{static_cast<int>(i), cmd_cv[i], all.mask_ids[2 * i], all.mask_ids[2 * i + 1], lv});
            max_level = std::max(max_level, lv);
        }
    }
    if (total_rows > INT32_MAX / 2 || total_segs > INT32_MAX / 2 || n_bins > INT32_MAX / 2)
        return fail(CY_ENOMEM, __LINE__);
    for (size_t ji = 0; ji < jobs.size(); ++ji) {
        const scan_job &j = jobs[ji];
        if (j.seg_count <= 0) continue;
        if (j.clip) {
            tab_cl.push_back(make_int2(static_cast<int>(cl_points), static_cast<int>(ji)));
            cl_points += j.seg_count;
        } else if (j.binned) {
            tab_bn.push_back(make_int2(static_cast<int>(bn_segs), static_cast<int>(ji)));
            bn_segs += j.seg_count;
        } else {
            tab_nc.push_back(make_int2(static_cast<int>(nc_segs), static_cast<int>(ji)));
            nc_segs += j.seg_count;
        }
    }
    pass_n[0] = cl_points;
    // Block index of the binned table: entry holding segment b << kTabShift
    // for every block b, and one more.
    bn_idx.clear();
    if (!tab_bn.empty()) {
        const int64_t nblk = (bn_segs >> cyg::kTabShift) + 2;
        bn_idx.resize(static_cast<size_t>(nblk));
        size_t e = 0;
        for (int64_t b = 0; b < nblk; ++b) {
            const int64_t target = std::min<int64_t>(b << cyg::kTabShift, bn_segs - 1);
            while (e + 1 < tab_bn.size() && tab_bn[e + 1].x <= target) ++e;
            bn_idx[static_cast<size_t>(b)] = static_cast<int32_t>(e);
        }
    }
    if (!tab_nc.empty() || !tab_bn.empty() || !tab_cl.empty()) {
        size_t nt = tab_nc.size() + tab_bn.size() + tab_cl.size();
        if (!tabs_dev.ensure(nt * sizeof(int2) + bn_idx.size() * sizeof(int32_t))) return fail(CY_ENOMEM, __LINE__);
        std::vector<int2> all_tabs(tab_nc);
        all_tabs.insert(all_tabs.end(), tab_bn.begin(), tab_bn.end());
        all_tabs.insert(all_tabs.end(), tab_cl.begin(), tab_cl.end());
        if (!ok(cudaMemcpyAsync(tabs_dev.p, all_tabs.data(), nt * sizeof(int2), cudaMemcpyHostToDevice, stream)) ||
            (!bn_idx.empty() && !ok(cudaMemcpyAsync(tabs_dev.as<int2>() + nt, bn_idx.data(),
                                                     bn_idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                                     stream))) ||
            !ok(cudaStreamSynchronize(stream)))
            return status;
    }
    size_t nr = static_cast<size_t>(total_rows);
    if (!jobs.empty()) {
        if (!jobs_dev.ensure(jobs.size() * sizeof(scan_job)) || !row_cnt.ensure((nr + 1) * 4) ||
            !row_off.ensure((nr + 2) * 8) || !row_cur.ensure((nr + 1) * 4) || !row_len.ensure((nr + 1) * 4) ||
            !boxes.ensure(jobs.size() * sizeof(cover_box)) || !rowoff_host.ensure((nr + 1) * 8) ||
            !long_rows.ensure((nr + 1) * 4) || !n_long.ensure(4) || !row_meta.ensure((nr + 1) * sizeof(int4)))
            return fail(CY_ENOMEM, __LINE__);
        if (!ok(cudaMemcpyAsync(jobs_dev.p, jobs.data(), jobs.size() * sizeof(scan_job), cudaMemcpyHostToDevice,
                                stream)) ||
            !ok(cudaMemsetAsync(row_cnt.p, 0, (nr + 1) * 4, stream)) ||
            !ok(cudaMemsetAsync(row_cur.p, 0, (nr + 1) * 4, stream)))
            return status;
    }
    if (n_bins > 0) {
        size_t nb = static_cast<size_t>(n_bins);
        if (!bin_cnt.ensure((nb + 1) * 4) || !bin_cur.ensure((nb + 1) * 4) || !bin_off.ensure((nb + 2) * 8) ||
            !binoff_host.ensure(8))
            return fail(CY_ENOMEM, __LINE__);
    }
    if (!sjobs.empty()) {
        if (!sj_dev.ensure(sjobs.size() * sizeof(cyg::shadow_job)) ||
            !sh_img.ensure(static_cast<size_t>(shadow_floats) * 4) ||
            !sh_scratch.ensure(static_cast<size_t>(shadow_floats) * 4))
            return fail(CY_ENOMEM, __LINE__);
        if (!ok(cudaMemcpyAsync(sj_dev.p, sjobs.data(), sjobs.size() * sizeof(cyg::shadow_job),
                                cudaMemcpyHostToDevice, stream)))
            return status;
    }
    if (!rects.ensure(std::max<size_t>(cmds.size(), 1) * sizeof(shadow_rect))) return fail(CY_ENOMEM, __LINE__);
    if (!get_dev.ensure(static_cast<size_t>(std::max<int64_t>(get_total, 16))) ||
        !get_host.ensure(static_cast<size_t>(std::max<int64_t>(get_total, 16))))
        return fail(CY_ENOMEM, __LINE__);
    if (!ok(cudaFuncSetAttribute(k_rows_long, cudaFuncAttributeMaxDynamicSharedMemorySize, kLongSmem))) return status;
    double t_sized = timing ? since(t_begin) : 0.0;
    // The first run also sizes the run store and the clip masks.
    int rc = run();
    if (timing)
        std::fprintf(stderr, "frame prepare: staged %.1f ms, geometry sized %.1f ms, first run queued %.1f ms\n",
                     t_staged, t_sized, since(t_begin));
    return rc;
}

int frame::run() {
    if (status) return status;
    n_ev = 0;
    launches = 0;
    mark();   // 0: start
    std::vector<command> &cmds = all.cmds;
    const float2 *d_hpts = reinterpret_cast<const float2 *>(d + o_hpts);
    const int32_t *d_hprev = reinterpret_cast<const int32_t *>(d + o_hprev);
    const float2 *d_bez = reinterpret_cast<const float2 *>(d + o_bez);
    const flat_item *d_items = reinterpret_cast<const flat_item *>(d + o_items);
    const command *d_cmds = reinterpret_cast<const command *>(d + o_cmd);
    const float *lut = lut_dev.as<float>();
    paint_src src;
    src.stop_off = reinterpret_cast<const float *>(d + o_soff);
    src.stop_col = reinterpret_cast<const float4 *>(d + o_scol);
    src.texels = nullptr;
    if (n_tex > 0) {
        if (!pat_f4.ensure(static_cast<size_t>(n_tex) * sizeof(float4))) return fail(CY_ENOMEM, __LINE__);
        int n = static_cast<int>(n_tex);
        k_pattern_prep<<<(n + 255) / 256, 256, 0, stream>>>(reinterpret_cast<const uchar4 *>(d + o_tex),
                                                            pat_f4.as<float4>(), n, lut);
        src.texels = pat_f4.as<float4>();
    }
    int n_items_flat = static_cast<int>(n_items_all);
    const bool reuse = geometry_ready;   // first run after the sizing: centre lines and counts are in place
    geometry_ready = false;
    if (n_items_flat > 0 && !reuse) {
        // flattening counts and offsets, then the points (the first run's
        // read-back only sized the store)
        k_flat_count<<<(n_items_flat + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items_flat,
                                                                    item_cnt.as<int32_t>());
        if (!ok(cudaMemsetAsync(item_cnt.as<int32_t>() + n_items_flat, 0, 4, stream))) return status;
        if (int rc = scan(item_cnt.as<int32_t>(), item_off.as<int32_t>(), n_items_flat + 1)) return rc;
        k_flat_emit<<<(n_items_flat + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items_flat,
                                                                    item_off.as<int32_t>(), flat_pts.as<float2>(),
                                                                    flat_prev.as<int32_t>(), nflat);
        launches += 2 + scan_launch_count(n_items_flat + 1);
    }
    if (n_tex > 0) ++launches;
    if (n_groups > 0 && n_outline > 0) {
        if (int rc = reuse ? stroke_write() : stroke_passes(false)) return rc;
    }
    mark();   // 1: patterns and flattening done
    size_t nr = static_cast<size_t>(total_rows);
    int n_jobs = static_cast<int>(jobs.size());
    row_view rv;
    rv.row_off = row_off.as<int64_t>();
    rv.row_len = row_len.as<int32_t>();
    rv.meta = row_meta.as<int4>();
    rv.runs = runs.as<cyg::run>();
    rv.sums = sums.as<float>();
    if (n_jobs > 0) {
        job_tables t;
        std::memset(&t, 0, sizeof(t));
        k_box_init<<<(n_jobs + 255) / 256, 256, 0, stream>>>(boxes.as<cover_box>(), n_jobs);
        t.jobs = jobs_dev.as<scan_job>();
        t.tab = tabs_dev.as<int2>();
        t.n_tab = static_cast<int>(tab_nc.size());
        t.pts[0] = d_hpts;
        t.prev[0] = d_hprev;
        t.pts[1] = flat_pts.p ? flat_pts.as<float2>() : d_hpts;
        t.prev[1] = flat_prev.p ? flat_prev.as<int32_t>() : d_hprev;
        t.boxes = boxes.as<cover_box>();
        t.row_cnt = row_cnt.as<int32_t>();
        t.row_cur = row_cur.as<int32_t>();
        int rc = clip_passes(t);
        if (rc) return rc;
        int segs_nc = static_cast<int>(nc_segs), segs_bn = static_cast<int>(bn_segs),
            segs_cl = static_cast<int>(pass_n[4]);
        // the binned jobs' own table
        job_tables tb = t;
        tb.tab = tabs_dev.as<int2>() + tab_nc.size();
        tb.n_tab = static_cast<int>(tab_bn.size());
        tb.tab_idx = bn_idx.empty() ? nullptr
                                    : reinterpret_cast<const int32_t *>(tabs_dev.as<int2>() + tab_nc.size() +
                                                                         tab_bn.size() + tab_cl.size());
        // Segments per warp round: halved while that leaves fewer than 48
        // warps per SM of work.
        auto per_warp = [](int segs) {
            int s = 32;
            while (s > 2 && segs / s < 152 * 48) s >>= 1;
            return s;
        };
        const int spw_nc = per_warp(segs_nc), spw_cl = per_warp(segs_cl);
        auto grid_for = [](int segs, int spw) {
            int per_block = kRunsWarps * spw;
            return std::max(1, std::min((segs + per_block - 1) / per_block, 152 * 16));
        };
        int grid_nc = grid_for(segs_nc, spw_nc), grid_cl = grid_for(segs_cl, spw_cl);
        if (segs_nc > 0) k_runs<false, false><<<grid_nc, kRunsWarps * 32, 0, stream>>>(t, segs_nc, spw_nc);
        if (segs_cl > 0) k_runs<false, true><<<grid_cl, kRunsWarps * 32, 0, stream>>>(t, segs_cl, spw_cl);
        rc = scan64(row_cnt.as<int32_t>(), row_off.as<int64_t>(), static_cast<int>(nr) + 1);
        if (rc) return rc;
        // Binned draws: count each bin's segments, then place the bins.
        bin_tables bt;
        std::memset(&bt, 0, sizeof(bt));
        const size_t nb = static_cast<size_t>(n_bins);
        const int bin_blocks = std::max(1, std::min((segs_bn + 255) / 256, 152 * 8));
        if (nb > 0) {
            bt.cnt = bin_cnt.as<int32_t>();
            bt.cur = bin_cur.as<int32_t>();
            bt.off = bin_off.as<int64_t>();
            if (!ok(cudaMemsetAsync(bin_cnt.p, 0, (nb + 1) * 4, stream)) ||
                !ok(cudaMemsetAsync(bin_cur.p, 0, (nb + 1) * 4, stream)))
                return status;
            if (segs_bn > 0) k_bin<false><<<bin_blocks, 256, 0, stream>>>(tb, bt, segs_bn);
            rc = scan64(bin_cnt.as<int32_t>(), bin_off.as<int64_t>(), static_cast<int>(nb) + 1);
            if (rc) return rc;
            launches += 2 + (segs_bn > 0 ? 2 : 0) + scan_launch_count(static_cast<int64_t>(nb) + 1);
        }
        if (!sized) {
            sized = true;
            // First run: size the run store, the bins and the new clip masks from the counts.
            if (!ok(cudaMemcpyAsync(rowoff_host.p, row_off.p, (nr + 1) * 8, cudaMemcpyDeviceToHost, stream)) ||
                (nb > 0 && !ok(cudaMemcpyAsync(binoff_host.p, bin_off.as<int64_t>() + nb, 8, cudaMemcpyDeviceToHost,
                                               stream))) ||
                !ok(cudaStreamSynchronize(stream)))
                return status;
            if (nb > 0) {
                n_bin_entries = *static_cast<const int64_t *>(binoff_host.p);
                if (n_bin_entries < 0) return fail(CY_ENOMEM, __LINE__);
                if (!bin_seg.ensure(static_cast<size_t>(n_bin_entries + 1) * sizeof(float4)))
                    return fail(CY_ENOMEM, __LINE__);
            }
            const int64_t *rowoff_h = static_cast<const int64_t *>(rowoff_host.p);
            int64_t nruns = rowoff_h[nr];
            if (nruns < 0) return fail(CY_ENOMEM, __LINE__);
            n_runs = nruns;
            for (size_t i = 0; i < cmds.size(); ++i) {
                if (cmds[i].kind != CMD_FILL || main_job[i] < 0 || jobs[main_job[i]].binned) continue;
                const scan_job &mj = jobs[main_job[i]];
                main_runs += rowoff_h[mj.row_base + mj.rows] - rowoff_h[mj.row_base];
                main_rows += mj.rows;
            }
            if (!runs.ensure(static_cast<size_t>(nruns + 1) * sizeof(cyg::run)) ||
                !sums.ensure(static_cast<size_t>(nruns + 1) * sizeof(float)))
                return fail(CY_ENOMEM, __LINE__);
            rv.runs = runs.as<cyg::run>();
            rv.sums = sums.as<float>();
            for (const clip_op &op : clips) {
                cy_ctx *cv = cvs[op.cv];
                mask_slot &nm = cv->masks[op.out_id];
                const scan_job &j = jobs[main_job[op.cmd]];
                int64_t path_runs = rowoff_h[j.row_base + j.rows] - rowoff_h[j.row_base];
                int64_t old_cap = op.in_id > 0 ? cv->masks[op.in_id].cap : 2 * static_cast<int64_t>(cv->H);
                nm.cap = std::max<int64_t>(path_runs + old_cap, 1);
                if (nm.cap > INT32_MAX) return fail(CY_ENOMEM, __LINE__);
                if (!ok(cudaMalloc(&nm.runs, static_cast<size_t>(nm.cap) * sizeof(cyg::run))) ||
                    !ok(cudaMalloc(&nm.sums, static_cast<size_t>(nm.cap) * sizeof(float))))
                    return status;
            }
        }
        t.row_off = row_off.as<int64_t>();
        t.runs = runs.as<cyg::run>();
        if (segs_nc > 0) k_runs<true, false><<<grid_nc, kRunsWarps * 32, 0, stream>>>(t, segs_nc, spw_nc);
        if (segs_cl > 0) k_runs<true, true><<<grid_cl, kRunsWarps * 32, 0, stream>>>(t, segs_cl, spw_cl);
        if (nb > 0) {
            bt.seg = bin_seg.as<float4>();
            if (segs_bn > 0) k_bin<true><<<bin_blocks, 256, 0, stream>>>(tb, bt, segs_bn);
        }
        int rgrid = static_cast<int>(std::min<size_t>((nr + kRowsWarps - 1) / kRowsWarps, 152 * 32));
        if (!ok(cudaMemsetAsync(n_long.p, 0, 4, stream))) return status;
        k_rows<<<std::max(rgrid, 1), kRowsWarps * 32, 0, stream>>>(
            row_off.as<int64_t>(), row_cnt.as<int32_t>(), row_cur.as<int32_t>(), row_len.as<int32_t>(),
            runs.as<cyg::run>(), sums.as<float>(), static_cast<int>(nr), long_rows.as<int32_t>(),
            n_long.as<int32_t>(), row_meta.as<int4>());
        k_rows_long<<<152 * 2, kLongThreads, kLongSmem, stream>>>(
            row_off.as<int64_t>(), row_cnt.as<int32_t>(), row_cur.as<int32_t>(), row_len.as<int32_t>(),
            runs.as<cyg::run>(), sums.as<float>(), long_rows.as<int32_t>(), n_long.as<int32_t>(),
            row_meta.as<int4>());
        if (!ok(cudaGetLastError())) return status;
        launches += (segs_nc > 0 ? 2 : 0) + (segs_cl > 0 ? 2 : 0) + 2 + scan_launch_count(static_cast<int64_t>(nr) + 1);
    }
    mark();   // 2: scan conversion done
    // Clip masks, level by level (a clip depends on the previous mask); all
    // clips of a level together, four launches.
    if (!clips.empty()) {
        if (!clips_built) {
            clips_built = true;
            clip_host.clear();
            level_first.assign(static_cast<size_t>(max_level) + 2, 0);
            level_max_h.assign(static_cast<size_t>(max_level) + 1, 0);
            for (int lv = 0; lv <= max_level; ++lv) {
                level_first[lv] = static_cast<int>(clip_host.size());
                for (const clip_op &op : clips) {
                    if (op.level != lv) continue;
                    cy_ctx *cv = cvs[op.cv];
                    mask_slot &nm = cv->masks[op.out_id];
                    const mask_slot *om = op.in_id > 0 ? &cv->masks[op.in_id] : nullptr;
                    const scan_job &j = jobs[main_job[op.cmd]];
                    clip_args a;
                    a.p_off = row_off.as<int64_t>();
                    a.p_len = row_len.as<int32_t>();
                    a.p_runs = runs.as<cyg::run>();
                    a.p_base = j.row_base;
                    a.p_box = boxes.as<cover_box>() + main_job[op.cmd];
                    a.o_off = om ? om->off : nullptr;
                    a.o_len = om ? om->len : nullptr;
                    a.o_runs = om ? om->runs : nullptr;
                    a.o_last_row = om ? om->last_row : nullptr;
                    a.n_off = nm.off;
                    a.n_len = nm.len;
                    a.n_runs = nm.runs;
                    a.n_sums = nm.sums;
                    a.n_vis = nm.vis;
                    a.n_last_row = nm.last_row;
                    a.W = cv->W;
                    a.H = cv->H;
                    a.rule = cmds[op.cmd].fill_rule;
                    clip_host.push_back(a);
                    level_max_h[lv] = std::max(level_max_h[lv], cv->H);
                }
            }
            level_first[max_level + 1] = static_cast<int>(clip_host.size());
            if (!clip_dev.ensure(clip_host.size() * sizeof(clip_args)) ||
                !ok(cudaMemcpyAsync(clip_dev.p, clip_host.data(), clip_host.size() * sizeof(clip_args),
                                    cudaMemcpyHostToDevice, stream)))
                return status;
        }
        const clip_args *ca = clip_dev.as<clip_args>();
        for (int lv = 0; lv <= max_level; ++lv) {
            int first = level_first[lv], n = level_first[lv + 1] - first, H = level_max_h[lv];
            if (n == 0) continue;
            k_clip_caps_all<<<dim3((H + 1 + 255) / 256, n), 256, 0, stream>>>(ca, first);
            k_clip_scan_all<<<dim3(1, n), 1024, 0, stream>>>(ca, first);
            k_clip_rows_all<<<dim3((H + 127) / 128, n), 128, 0, stream>>>(ca, first);
            k_mask_fill_all<<<dim3(std::max(1, std::min((H + 7) / 8, 64)), n), 256, 0, stream>>>(ca, first);
            if (!ok(cudaGetLastError())) return status;
            launches += 4;
        }
    }
    // Shadow images of every shadowed draw.
    if (!sjobs.empty()) {
        int ns = static_cast<int>(sjobs.size());
        int max_w = 0, max_h = 0;
        for (const auto &s : sjobs) {
            max_w = std::max(max_w, s.W + 2 * s.border + 1);
            max_h = std::max(max_h, s.H + 2 * s.border);
        }
        const cyg::shadow_job *dsj = sj_dev.as<cyg::shadow_job>();
        k_shadow_rects<<<(ns + 127) / 128, 128, 0, stream>>>(dsj, ns, boxes.as<cover_box>(), rects.as<shadow_rect>());
        dim3 rg(std::max(1, std::min((max_h + 7) / 8, 64)), ns);
        k_shadow_raster_all<<<rg, 256, 0, stream>>>(dsj, d_cmds, src, rv, rects.as<shadow_rect>(), sh_img.as<float>());
        dim3 bg((max_h + 127) / 128, ns), cg((max_w + 127) / 128, ns);
        dim3 tg((max_w + 31) / 32, (max_h + 31) / 32, ns), tb(32, 8);
        // raster (column-major) -> row blur in place -> transpose into the
        // scratch image -> column blur in place there: the final image.
        k_blur_rows_all<<<bg, 128, 0, stream>>>(dsj, rects.as<shadow_rect>(), sh_img.as<float>(),
                                                 sh_scratch.as<float>());
        k_transpose_all<<<tg, tb, 0, stream>>>(dsj, rects.as<shadow_rect>(), sh_img.as<float>(),
                                               sh_scratch.as<float>());
        k_blur_cols_all<<<cg, 128, 0, stream>>>(dsj, rects.as<shadow_rect>(), sh_scratch.as<float>(),
                                                 sh_img.as<float>());
        if (!ok(cudaGetLastError())) return status;
        launches += 5;
    }
    mark();   // 3: masks and shadows done
    if (get_total > 0 && !ok(cudaMemsetAsync(get_dev.p, 0, static_cast<size_t>(get_total), stream))) return status;
    const uint8_t *d_put = reinterpret_cast<const uint8_t *>(d + o_put);
    // Per-command extras.
    if (!ext_built) {
        ext_built = true;
        ext.assign(cmds.size(), strip_cmd());
        for (size_t i = 0; i < cmds.size(); ++i) {
            strip_cmd &e = ext[i];
            std::memset(&e, 0, sizeof(e));
            const command &c = cmds[i];
            cy_ctx *cv = cvs[cmd_cv[i]];
            e.main_row_base = main_job[i] >= 0 ? jobs[main_job[i]].row_base : 0;
            e.bin_base = main_job[i] >= 0 ? jobs[main_job[i]].bin_base : 0;
            e.band_h = main_job[i] >= 0 && jobs[main_job[i]].band_h > 0 ? jobs[main_job[i]].band_h : 1;
            e.has_shadow = shadow_job[i] >= 0;
            e.shadow_img = 0;
            if (e.has_shadow)
                for (const auto &s : sjobs)
                    if (s.cmd == static_cast<int32_t>(i)) e.shadow_img = s.img;
            int in_id = all.mask_ids[2 * i];
            e.vis = in_id > 0 ? cv->masks[in_id].vis : nullptr;
            if (c.kind == CMD_GET) {
                e.get_out = c.get_out;
                e.get_x = c.get_x; e.get_y = c.get_y; e.get_w = c.get_w; e.get_h = c.get_h;
            }
        }
    }
    if (engine == 1) {
        // Plain engine: per-draw launches over each canvas's float bitmap.
        // A fresh deferred canvas starts blank on every run, so running the
        // frame again (timing, graph replay) gives the same pixels.
        for (cy_ctx *cv : cvs)
            if (cv->deferred && !cv->has_content &&
                !ok(cudaMemsetAsync(cv->bitmap, 0, static_cast<size_t>(cv->W) * cv->H * sizeof(float4), stream)))
                return status;
        for (size_t i = 0; i < cmds.size(); ++i) {
            const command &c = cmds[i];
            cy_ctx *cv = cvs[cmd_cv[i]];
            int W = cv->W, H = cv->H;
            const strip_cmd &e = ext[i];
            if (c.kind == CMD_CLIP) continue;
            if (c.kind == CMD_PUT) {
                dim3 blk(32, 8), grd((c.put_w + 31) / 32, (c.put_h + 7) / 8);
                k_put<<<grd, blk, 0, stream>>>(d_cmds + i, d_put, cv->bitmap, W, H, lut);
                ++launches;
                continue;
            }
            if (c.kind == CMD_GET) {
                dim3 blk(32, 8), grd((c.get_w + 31) / 32, (c.get_h + 7) / 8);
                k_get<<<grd, blk, 0, stream>>>(cv->bitmap, W, H,
                                               reinterpret_cast<uchar4 *>(get_dev.as<uint8_t>() + c.get_out),
                                               c.get_w, c.get_h, c.get_x, c.get_y);
                ++launches;
                continue;
            }
            if (e.has_shadow) {
                dim3 blk(32, 8), cgrd((W + 31) / 32, (H + 7) / 8);
                k_shadow_composite<<<cgrd, blk, 0, stream>>>(d_cmds + i, cv->bitmap, W, H, e.vis,
                                                             rects.as<shadow_rect>() + i,
                                                             sh_scratch.as<float>() + e.shadow_img);
            }
            bool clearing = !(c.op & 8);
            int y0 = clearing ? 0 : std::max(0, std::min(H, c.gy0));
            int y1 = clearing ? H : std::max(0, std::min(H, c.gy1 + 1));
            if (y1 > y0) {
                paint_args pa;
                pa.cmd = d_cmds + i;
                pa.bitmap = cv->bitmap;
                pa.W = W;
                pa.H = H;
                pa.rv = rv;
                pa.row_base = e.main_row_base;
                pa.vis = e.vis;
                pa.y_begin = y0;
                pa.y_end = y1;
                pa.src = src;
                k_paint<<<std::max(1, (y1 - y0 + 7) / 8), 256, 0, stream>>>(pa);
                ++launches;
            }
            if (e.has_shadow) ++launches;
        }
        mark();   // 4: paint done
        return ok(cudaGetLastError()) ? CY_OK : status;
    }
    // Tile engine: one persistent launch over (canvas, strip) work items.
    if (!strips_built) {
        int rc = build_strips();
        if (rc) return rc;
    }
    last_rv = rv;
    last_src = src;
    last_cmds = d_cmds;
    last_put = d_put;
    last_lut = lut;
    int rc = launch_strips();
    mark();   // 4: paint done
    return rc;
}

// Strip layout of the frame for the current strip configuration: per
// canvas its strip height, work items (canvas, first row) in decreasing
// cost, uploaded with the per-command extras.
int frame::build_strips() {
    strips_built = true;
    strip_pixels = g_strip_pixels;
    if (binned) strip_pixels = std::min(strip_pixels, kBinnedMaxStrip);
    strip_threads = g_strip_threads;
    strip_cap = 0;
    strip_words = 0;
    const int nwarps = (strip_threads == 128 || strip_threads == 512 ? strip_threads : 256) / 32;
    scv.resize(cvs.size());
    std::vector<std::pair<int64_t, int2>> work;
    int cursor = 0;
    for (size_t ci = 0; ci < cvs.size(); ++ci) {
        cy_ctx *cv = cvs[ci];
        if (cv->W > strip_pixels) return fail(CY_EINVAL);   // a row must fit in one strip
        strip_canvas &s = scv[ci];
        s.W = cv->W;
        s.H = cv->H;
        s.TH = std::max(1, std::min(cv->H, strip_pixels / std::max(1, cv->W)));
        if (binned && s.TH > nwarps && s.TH < cv->H) {
            // a multiple of the warps, so each warp owns whole rows (when that
            // costs at most a quarter of the strip)
            int th = s.TH - s.TH % nwarps;
            if (4 * th >= 3 * s.TH) s.TH = th;
        }
        strip_cap = std::max(strip_cap, s.TH * s.W);
        strip_words = std::max(strip_words, (s.TH * ((s.W + 31) / 32) + 31) / 32);
        s.cmd_first = cursor;
        s.cmd_count = static_cast<int32_t>(cv->q.cmds.size());
        cursor += s.cmd_count;
        // canvases keep their pixels for later frames, unless their owner
        // destroys them after this one
        s.flags = (cv->has_content ? 1 : 0) | (cv->transient ? 0 : 2);
        s.bitmap = cv->bitmap;
        int64_t cost = static_cast<int64_t>(s.TH) * s.W * (s.cmd_count + 1);
        for (int y = 0; y < s.H; y += s.TH) work.push_back({cost, make_int2(static_cast<int>(ci), y)});
    }
    std::stable_sort(work.begin(), work.end(),
                     [](const std::pair<int64_t, int2> &a, const std::pair<int64_t, int2> &b) {
                         return a.first > b.first;
                     });
    items_host.resize(work.size());
    for (size_t k = 0; k < work.size(); ++k) items_host[k] = work[k].second;
    n_items = static_cast<int>(items_host.size());
    if (!scv_dev.ensure(scv.size() * sizeof(strip_canvas)) ||
        !items_dev.ensure(std::max<size_t>(items_host.size(), 1) * sizeof(int2)) ||
        !ext_dev.ensure(std::max<size_t>(ext.size(), 1) * sizeof(strip_cmd)) || !counter.ensure(4))
        return fail(CY_ENOMEM, __LINE__);
    if (!ok(cudaMemcpyAsync(scv_dev.p, scv.data(), scv.size() * sizeof(strip_canvas), cudaMemcpyHostToDevice,
                            stream)))
        return status;
    if (n_items > 0 && !ok(cudaMemcpyAsync(items_dev.p, items_host.data(), items_host.size() * sizeof(int2),
                                           cudaMemcpyHostToDevice, stream)))
        return status;
    if (!ext.empty() && !ok(cudaMemcpyAsync(ext_dev.p, ext.data(), ext.size() * sizeof(strip_cmd),
                                            cudaMemcpyHostToDevice, stream)))
        return status;
    // The attribute is per kernel, shared by every frame in every thread:
    // always the largest strip any frame may launch (a launch uses its own).
    if (strip_smem() > kMaxStripSmem) return fail(CY_EINVAL, __LINE__);
    if (!ok(cudaFuncSetAttribute(strip_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kMaxStripSmem))))
        return status;
    return CY_OK;
}

// The persistent strip kernel over all (canvas, strip) items, with the
// inputs of the last run.
int frame::launch_strips() {
    if (n_items == 0) return CY_OK;
    size_t smem = strip_smem();
    if (!ok(cudaMemsetAsync(counter.p, 0, 4, stream))) return status;
    strip_params P;
    P.canvases = scv_dev.as<strip_canvas>();
    P.items = items_dev.as<int2>();
    P.n_items = n_items;
    P.counter = counter.as<int>();
    P.cmds = last_cmds;
    P.ext = ext_dev.as<strip_cmd>();
    P.rv = last_rv;
    P.src = last_src;
    P.rects = rects.as<shadow_rect>();
    P.shadow_imgs = sh_scratch.as<float>();
    P.put_px = last_put;
    P.lut = last_lut;
    P.get_buf = get_dev.as<uint8_t>();
    P.strip_pixels = strip_cap;
    P.strip_words = strip_words;
    P.bin_off = bin_off.p ? bin_off.as<int64_t>() : nullptr;
    P.bin_seg = bin_seg.p ? bin_seg.as<float4>() : nullptr;
    int per_sm = 0, dev = 0, sms = 152;
    auto kern = strip_kernel();
    int threads = strip_threads == 128 || strip_threads == 512 ? strip_threads : 256;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = std::max(1, std::min(n_items, sms * std::max(per_sm, 1)));
    kern<<<grid, threads, smem, stream>>>(P);
    ++launches;
    return ok(cudaGetLastError()) ? CY_OK : status;
}

int frame::finish() {
    if (status) return status;
    if (get_total > 0 && !ok(cudaMemcpyAsync(get_host.p, get_dev.p, static_cast<size_t>(get_total),
                                             cudaMemcpyDeviceToHost, stream)))
        return status;
    if (!ok(cudaStreamSynchronize(stream))) return status;
    // Deliver reads: to the caller's buffer, or keep them for deferred
    // readers; contexts in parallel, each context's reads in call order.
    std::vector<std::vector<std::pair<int, int>>> gets(cvs.size());   // (command, read index)
    {
        int g = 0;
        for (size_t i = 0; i < all.cmds.size(); ++i)
            if (all.cmds[i].kind == CMD_GET) gets[cmd_cv[i]].emplace_back(static_cast<int>(i), g++);
    }
    auto deliver = [&](size_t ci) {
        cy_ctx *cv = cvs[ci];
        size_t add = 0;
        for (auto &p : gets[ci]) {
            const command &c = all.cmds[p.first];
            if (!all.get_dst[p.second]) add += static_cast<size_t>(c.get_w) * c.get_h * 4;
        }
        cv->deferred_out.reserve(cv->deferred_out.size() + add);
        for (auto &p : gets[ci]) {
            const command &c = all.cmds[p.first];
            const uint8_t *src = static_cast<const uint8_t *>(get_host.p) + c.get_out;
            unsigned char *dst = all.get_dst[p.second];
            int stride = all.get_stride[p.second];
            if (dst) {
                for (int row = 0; row < c.get_h; ++row)
                    std::memcpy(dst + static_cast<ptrdiff_t>(row) * stride,
                                src + static_cast<size_t>(row) * c.get_w * 4, static_cast<size_t>(c.get_w) * 4);
            } else if (!keep_reads) {
                cv->deferred_out.insert(cv->deferred_out.end(), src,
                                        src + static_cast<size_t>(c.get_w) * c.get_h * 4);
            }
        }
    };
    parallel_for(cvs.size(), deliver);
    for (cy_ctx *cv : cvs) {
        queue &q = cv->q;
        for (size_t i = 0; i < q.cmds.size(); ++i) {
            int in = q.mask_ids[2 * i], out = q.mask_ids[2 * i + 1];
            if (in > 0) cy_mask_release(cv, in);
            if (out > 0) cy_mask_release(cv, out);
            if (q.cmds[i].kind == CMD_FILL || q.cmds[i].kind == CMD_PUT) cv->has_content = true;
        }
        q.clear();
    }
    return CY_OK;
}

// ------------------------------------------------------------ host helpers
namespace {

void bounds_of(const float *xy, size_t n, command &c) {
    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    bool finite = true;
    for (size_t i = 0; i < n; ++i) {
        float x = xy[2 * i], y = xy[2 * i + 1];
        finite = finite && std::isfinite(x) && std::isfinite(y);
        if (x < x0) x0 = x;
        if (x > x1) x1 = x;
        if (y < y0) y0 = y;
        if (y > y1) y1 = y;
    }
    auto clampi = [](float v) {
        if (!(v == v)) return 0;
        if (v < -1.0e9f) return -1000000000;
        if (v > 1.0e9f) return 1000000000;
        return static_cast<int>(floorf(v));
    };
    // A non-finite coordinate makes the bounds unknown: the whole canvas,
    // and the polygon clip, which leaves such points out and joins their
    // neighbours as the reference's does (hpp:2218-2223); without the clip a
    // NaN point would leave its polygon open.  So does a coordinate of 2^20
    // or more: the clip's crossing with such a far point cancels
    // (hpp:2220-2221) and can land anywhere on the canvas, outside the
    // points' own bounds.
    bool bad = !finite || !(x0 <= x1) || !(y0 <= y1);
    if (!bad && std::max(std::max(std::fabs(x0), std::fabs(x1)), std::max(std::fabs(y0), std::fabs(y1))) >= 1048576.0f)
        bad = true;
    c.gx0 = bad ? -1000000000 : clampi(x0);
    c.gy0 = bad ? -1000000000 : clampi(y0);
    c.gx1 = bad ? 1000000000 : clampi(x1) + 1;
    c.gy1 = bad ? 1000000000 : clampi(y1) + 1;
}

// ---------------------------------------------------- device image cache
// Pattern and draw_image texels that recur -- the same image drawn on many
// canvases of a frame, or by many serving requests -- are kept on the device,
// already linearised and premultiplied (what k_pattern_prep makes of them,
// hpp:2841-2864), keyed by their size and bytes.  An image is cached the
// second time it is seen; the first time it goes up with its frame as
// usual.  The texels live in 32 MiB pool chunks that are never moved or
// freed while the process runs (frames and captured graphs hold pointers
// into them); the pool stops growing at 1 GiB per device, after which new
// images go up with their frames again.
namespace {

constexpr size_t kTexChunk = size_t(32) << 20;
constexpr size_t kTexCap = size_t(1) << 30;
constexpr int kTexDevices = 64;

struct tex_entry {
    int w = 0, h = 0;
    std::vector<uchar4> px;          // the source bytes (exact match on lookup)
    const float4 *dev = nullptr;
};

struct tex_cache {
    std::vector<void *> chunks;
    size_t used = 0;                 // bytes used in the last chunk
    size_t total = 0;                // bytes of all chunks
    std::unordered_map<uint64_t, std::vector<tex_entry>> map;
    std::unordered_map<uint64_t, int> seen;   // hash -> sightings of uncached images
    cudaStream_t stream = nullptr;
    void *stage = nullptr;           // device copy of the bytes being converted
    size_t stage_cap = 0;
    float *lut = nullptr;
    int64_t hits = 0, inserts = 0;
};

std::mutex g_tex_lock;
tex_cache g_tex[kTexDevices];

uint64_t image_hash(const uchar4 *px, size_t n, int w, int h) {
    // FNV-1a over the bytes, 8 at a time, seeded with the size.
    uint64_t x = 1469598103934665603ull ^ (static_cast<uint64_t>(w) << 32 | static_cast<uint32_t>(h));
    const unsigned char *b = reinterpret_cast<const unsigned char *>(px);
    size_t bytes = n * 4, i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t v;
        std::memcpy(&v, b + i, 8);
        x = (x ^ v) * 1099511628211ull;
    }
    for (; i < bytes; ++i) x = (x ^ b[i]) * 1099511628211ull;
    return x;
}

// The cached texels of a w x h RGBA8 image on device `dev`, or null when it
// is not (yet) cached.  Inserting converts the image on the cache's stream
// and waits for it, so the texels are ready before any frame refers to them.
const float4 *tex_cache_lookup(int dev, const uchar4 *px, int w, int h) {
    if (dev < 0 || dev >= kTexDevices) return nullptr;
    const size_t n = static_cast<size_t>(w) * static_cast<size_t>(h);
    const size_t need = (n * sizeof(float4) + 255) & ~static_cast<size_t>(255);
    if (need > kTexChunk) return nullptr;
    const uint64_t key = image_hash(px, n, w, h);
    std::lock_guard<std::mutex> hold(g_tex_lock);
    tex_cache &tc = g_tex[dev];
    auto it = tc.map.find(key);
    if (it != tc.map.end())
        for (const tex_entry &e : it->second)
            if (e.w == w && e.h == h && std::memcmp(e.px.data(), px, n * 4) == 0) {
                ++tc.hits;
                return e.dev;
            }
    if (tc.seen.size() > 65536) tc.seen.clear();
    if (++tc.seen[key] < 2) return nullptr;
    // second sighting: insert
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != dev) {
        cudaGetLastError();
        return nullptr;
    }
    if (tc.chunks.empty() || tc.used + need > kTexChunk) {
        if (tc.total + kTexChunk > kTexCap) return nullptr;
        void *chunk = nullptr;
        if (cudaMalloc(&chunk, kTexChunk) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        tc.chunks.push_back(chunk);
        tc.total += kTexChunk;
        tc.used = 0;
    }
    if (!tc.stream && cudaStreamCreateWithFlags(&tc.stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        tc.stream = nullptr;
        return nullptr;
    }
    if (!tc.lut) {
        if (cudaMalloc(&tc.lut, 256 * sizeof(float)) != cudaSuccess ||
            cudaMemcpy(tc.lut, linear_lut_host(), 256 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            if (tc.lut) cudaFree(tc.lut);
            tc.lut = nullptr;
            return nullptr;
        }
    }
    if (tc.stage_cap < n * 4) {
        if (tc.stage) cudaFree(tc.stage);
        tc.stage = nullptr;
        tc.stage_cap = 0;
        if (cudaMalloc(&tc.stage, n * 4) != cudaSuccess) {
            cudaGetLastError();
            tc.stage = nullptr;
            return nullptr;
        }
        tc.stage_cap = n * 4;
    }
    float4 *dst = reinterpret_cast<float4 *>(static_cast<char *>(tc.chunks.back()) + tc.used);
    int ni = static_cast<int>(n);
    if (cudaMemcpyAsync(tc.stage, px, n * 4, cudaMemcpyHostToDevice, tc.stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    k_pattern_prep<<<(ni + 255) / 256, 256, 0, tc.stream>>>(static_cast<const uchar4 *>(tc.stage), dst, ni, tc.lut);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(tc.stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    tc.used += need;
    tex_entry e;
    e.w = w;
    e.h = h;
    e.px.assign(px, px + n);
    e.dev = dst;
    tc.map[key].push_back(std::move(e));
    tc.seen.erase(key);
    ++tc.inserts;
    return dst;
}

}  // namespace

int fill_paint(queue &q, const cy_paint *p, command &c, int device) {
    c.paint = p->kind;
    c.clamp = p->clamp_edges;
    for (int i = 0; i < 6; ++i) c.inv[i] = p->inverse[i];
    for (int i = 0; i < 4; ++i) c.color[i] = p->color[i];
    c.p0x = p->start[0]; c.p0y = p->start[1]; c.p1x = p->end[0]; c.p1y = p->end[1];
    c.r0 = p->start_radius; c.r1 = p->end_radius;
    c.stop_first = c.stop_count = 0;
    c.pat_first = c.pat_w = c.pat_h = c.pat_rep = 0;
    c.pat_ptr = 0;
    if (p->kind == CY_PAINT_LINEAR || p->kind == CY_PAINT_RADIAL) {
        if (p->n_stops <= 0) { c.paint = CY_PAINT_NONE; return CY_OK; }
        if (!p->stop_offsets || !p->stop_colors) return CY_EINVAL;
        c.stop_first = static_cast<int32_t>(q.stop_off.size());
        c.stop_count = p->n_stops;
        for (int i = 0; i < p->n_stops; ++i) {
            q.stop_off.push_back(p->stop_offsets[i]);
            q.stop_col.push_back(make_float4(p->stop_colors[4 * i], p->stop_colors[4 * i + 1],
                                             p->stop_colors[4 * i + 2], p->stop_colors[4 * i + 3]));
        }
        q.bytes += static_cast<size_t>(p->n_stops) * 20;
    } else if (p->kind == CY_PAINT_PATTERN) {
        if (!p->pattern || p->pattern_width <= 0 || p->pattern_height <= 0) return CY_EINVAL;
        size_t n = static_cast<size_t>(p->pattern_width) * static_cast<size_t>(p->pattern_height);
        if (q.texels.size() + n > static_cast<size_t>(INT32_MAX)) return CY_EINVAL;
        c.pat_w = p->pattern_width;
        c.pat_h = p->pattern_height;
        c.pat_rep = p->repetition;
        const uchar4 *src = reinterpret_cast<const uchar4 *>(p->pattern);
        if (const float4 *cached = tex_cache_lookup(device, src, p->pattern_width, p->pattern_height)) {
            c.pat_ptr = static_cast<int64_t>(reinterpret_cast<uintptr_t>(cached));
            c.pat_first = 0;
        } else {
            c.pat_first = static_cast<int32_t>(q.texels.size());
            q.texels.insert(q.texels.end(), src, src + n);
            q.bytes += n * 4;
        }
    } else if (p->kind != CY_PAINT_NONE && p->kind != CY_PAINT_SOLID) {
        return CY_EINVAL;
    }
    return CY_OK;
}

void fill_state(const cy_draw_state *s, command &c) {
    c.op = s->operation;
    c.alpha = s->global_alpha;
    c.fill_rule = s->fill_rule == 1 ? 1 : 0;
    c.shadow = 0;
    // render_shadow runs only for a visible shadow colour that is blurred or
    // offset (hpp:2398-2401); its parameters follow hpp:2402-2408, 2453-2459.
    if (s->shadow_color[3] != 0.0f &&
        !(s->shadow_blur == 0.0f && s->shadow_offset_x == 0.0f && s->shadow_offset_y == 0.0f)) {
        float sigma2 = 0.25f * s->shadow_blur * s->shadow_blur;
        size_t radius = static_cast<size_t>(0.5f * sqrtf(4.0f * sigma2 + 1.0f) - 0.5f);
        if (radius > 4096) radius = 4096;
        int border = 3 * (static_cast<int>(radius) + 1);
        float alpha = static_cast<float>(2 * radius + 1) * (static_cast<float>(radius * (radius + 1)) - sigma2) /
                      (2.0f * sigma2 - static_cast<float>(6 * (radius + 1) * (radius + 1)));
        float divisor = 2.0f * (alpha + static_cast<float>(radius)) + 1.0f;
        c.shadow = 1;
        c.sh_radius = static_cast<int32_t>(radius);
        c.sh_border = border;
        for (int i = 0; i < 4; ++i) c.sh_color[i] = s->shadow_color[i];
        c.sh_w1 = alpha / divisor;
        c.sh_w2 = (1.0f - alpha) / divisor;
        c.sh_offx = static_cast<float>(border) + s->shadow_offset_x;
        c.sh_offy = static_cast<float>(border) + s->shadow_offset_y;
    }
}

bool valid_counts(const int *counts, int n, size_t &total) {
    total = 0;
    for (int i = 0; i < n; ++i) {
        if (counts[i] < 0) return false;
        total += static_cast<size_t>(counts[i]);
    }
    return total < (static_cast<size_t>(1) << 30);
}

// The rectangles a command's geometry is scanned against: the canvas, and
// for a shadow the padded canvas with the points moved by the shadow offset.
// keep_left: a polygon wholly left of the canvas is kept, for a draw whose
// coverage may be binned -- clipped segment by segment, its projection onto
// x = 0 adds pieces whose rounded sums need not cancel to zero as the
// polygon clip's empty result does.
struct cull_rects {
    float w, h;
    bool shadow;
    float sw, sh, sx, sy;
    bool keep_left;
};

// Whether the Sutherland-Hodgman clip (hpp:2204-2235) leaves nothing of a
// polygon in every rectangle of the command.  The clip's passes run in the
// order x >= 0, y >= 0, x <= w, y <= h: a polygon wholly beyond the edge of
// a pass loses all its points there, provided every earlier pass returned it
// unchanged (wholly inside its edge; a crossing would add points whose
// rounding is not bounded by the polygon's).  The comparisons are the
// clip's own; `margin` widens them for control polygons, whose flattened
// points may stray from the hull by rounding.
bool culled(const float2 *p, int n, const cull_rects &r, float margin) {
    auto empty = [&](float ox, float oy, float w, float h) {
        for (int e = 0; e < 4; ++e) {
            bool out = true, in = true;
            for (int k = 0; k < n && (out || in); ++k) {
                float x = ox + p[k].x, y = oy + p[k].y;
                float d = e == 0 ? x : e == 1 ? y : e == 2 ? w - x : h - y;
                out = out && d < -margin;
                in = in && d >= margin;
            }
            if (out) return !(e == 0 && r.keep_left);
            if (!in) return false;
        }
        return false;
    };
    if (n <= 0) return true;
    if (!empty(0.0f, 0.0f, r.w, r.h)) return false;
    return !r.shadow || empty(r.sx, r.sy, r.sw, r.sh);
}

int queue_geometry(queue &q, const float *points, const int *counts, int n_sub, bool bezier, command &cmd,
                   const cull_rects &rects) {
    size_t total = 0;
    if (n_sub < 0 || (n_sub > 0 && (!counts || !points)) || !valid_counts(counts, n_sub, total))
        return CY_EINVAL;
    bounds_of(points, total, cmd);
    const float2 *p = reinterpret_cast<const float2 *>(points);
    if (!bezier) {
        cmd.geom = 0;
        cmd.first = static_cast<int32_t>(q.host_pts.size());
        size_t at = 0, kept = 0;
        for (int s = 0; s < n_sub; ++s) {
            int32_t base = static_cast<int32_t>(q.host_pts.size());
            int n = counts[s];
            if (!culled(p + at, n, rects, 0.0f)) {
                for (int k = 0; k < n; ++k) {
                    q.host_pts.push_back(p[at + k]);
                    q.host_prev.push_back(k == 0 ? base + n - 1 : base + k - 1);
                }
                kept += n;
            }
            at += n;
        }
        cmd.count = static_cast<int32_t>(kept);
        q.bytes += kept * 12;
        return CY_OK;
    }
    // Bezier path: one flattening item per subpath start and per cubic.
    for (int s = 0; s < n_sub; ++s)
        if (counts[s] != 0 && (counts[s] - 1) % 3 != 0) return CY_EINVAL;
    cmd.geom = 1;
    cmd.first = static_cast<int32_t>(q.items.size());
    int32_t pbase = static_cast<int32_t>(q.bez_pts.size());
    q.bez_pts.insert(q.bez_pts.end(), p, p + total);
    size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s];
        if (n == 0) continue;
        float big = 0.0f;
        for (int k = 0; k < n; ++k) big = std::max(big, std::max(std::fabs(p[at + k].x), std::fabs(p[at + k].y)));
        if (culled(p + at, n, rects, 1.0f + 1.0e-5f * big)) {
            at += n;
            continue;
        }
        int32_t start = static_cast<int32_t>(q.items.size());
        flat_item head = {pbase + static_cast<int32_t>(at), 0, -1.0f};
        q.items.push_back(head);
        for (int k = 1; k < n; k += 3) {
            flat_item cub = {pbase + static_cast<int32_t>(at + k - 1), -1, -1.0f};
            q.items.push_back(cub);
        }
        q.items[start].sub_end = static_cast<int32_t>(q.items.size());
        at += n;
    }
    cmd.count = static_cast<int32_t>(q.items.size()) - cmd.first;
    q.bytes += total * 8 + static_cast<size_t>(cmd.count) * 8;
    return CY_OK;
}

int flush_ctx(cy_ctx *c) {
    if (c->status) return c->status;
    if (c->q.empty()) return CY_OK;
    if (!c->cached_frame) c->cached_frame = new (std::nothrow) frame();
    frame *f = static_cast<frame *>(c->cached_frame);
    if (!f) return c->fail(CY_ENOMEM, __LINE__);
    f->reset();
    f->stream = c->stream;
    f->engine = c->engine;
    f->cvs.push_back(c);
    int rc = f->prepare();
    if (rc == CY_OK) rc = f->finish();
    f->cvs.clear();
    return rc;
}

int maybe_flush(cy_ctx *c) {
    queue &q = c->q;
    if (q.bytes > (static_cast<size_t>(256) << 20) || q.cmds.size() >= 65536 ||
        q.rows > (static_cast<int64_t>(16) << 20))
        return c->deferred ? CY_OK : flush_ctx(c);
    return CY_OK;
}

int queue_draw(cy_ctx *c, const float *points, const int *counts, int n_sub, bool bezier, const cy_paint *paint,
               const cy_draw_state *state) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!paint || !state) return CY_EINVAL;
    if (state->mask < 0 || state->mask >= static_cast<int>(c->masks.size()) ||
        (state->mask > 0 && c->masks[state->mask].refs <= 0))
        return CY_EINVAL;
    queue &q = c->q;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_FILL;
    size_t stops = q.stop_off.size(), tex = q.texels.size();
    fill_state(state, cmd);
    cull_rects rects = {static_cast<float>(c->W), static_cast<float>(c->H), cmd.shadow != 0,
                        static_cast<float>(c->W + 2 * cmd.sh_border), static_cast<float>(c->H + 2 * cmd.sh_border),
                        cmd.sh_offx, cmd.sh_offy, true};
    int rc = fill_paint(q, paint, cmd, c->device);
    if (rc == CY_OK) rc = queue_geometry(q, points, counts, n_sub, bezier, cmd, rects);
    if (rc != CY_OK) {
        q.stop_off.resize(stops);
        q.stop_col.resize(stops);
        q.texels.resize(tex);
        return rc;
    }
    q.rows += c->H + (cmd.shadow ? c->H + 2 * cmd.sh_border : 0);
    q.cmds.push_back(cmd);
    q.mask_ids.push_back(state->mask);
    q.mask_ids.push_back(0);
    if (state->mask > 0) c->masks[state->mask].refs++;   // held until the frame finishes
    return maybe_flush(c);
}

std::atomic<int> g_device_stroke(1);

// Bounds of a stroke outline from its path's control points: the outline
// stays within half * max(2, miter limit if mitred) of the centre line in
// user space (joins, caps and their control points included), mapped by the
// forward transform, plus a margin for the rounding of the round trip
// through user space.
void stroke_bounds(const float *xy, size_t n, const stroke_style &st, command &c) {
    bounds_of(xy, n, c);
    if (c.gx0 <= -1000000000 || c.gy0 <= -1000000000 || c.gx1 >= 1000000000 || c.gy1 >= 1000000000) return;
    const float *f = st.fwd, *iv = st.inv;
    double lin = std::sqrt(static_cast<double>(f[0]) * f[0] + static_cast<double>(f[1]) * f[1] +
                           static_cast<double>(f[2]) * f[2] + static_cast<double>(f[3]) * f[3]);
    double ilin = std::sqrt(static_cast<double>(iv[0]) * iv[0] + static_cast<double>(iv[1]) * iv[1] +
                            static_cast<double>(iv[2]) * iv[2] + static_cast<double>(iv[3]) * iv[3]);
    double r = 2.0 * std::fabs(static_cast<double>(st.half));
    if (st.join == 0) r = std::max(r, std::sqrt(std::fabs(static_cast<double>(st.ratio))));
    double big = std::max(std::max(std::fabs(static_cast<double>(c.gx0)), std::fabs(static_cast<double>(c.gx1))),
                          std::max(std::fabs(static_cast<double>(c.gy0)), std::fabs(static_cast<double>(c.gy1))));
    double user = ilin * big + std::fabs(static_cast<double>(iv[4])) + std::fabs(static_cast<double>(iv[5]));
    double margin = r * lin + 2.0 +
                    1.0e-5 * (big + lin * user + std::fabs(static_cast<double>(f[4])) + std::fabs(static_cast<double>(f[5])));
    if (!(margin < 1.0e9)) {
        c.gx0 = c.gy0 = -1000000000;
        c.gx1 = c.gy1 = 1000000000;
        return;
    }
    auto grow = [&](int32_t &v, double by) {
        double x = static_cast<double>(v) + by;
        v = x < -1.0e9 ? -1000000000 : x > 1.0e9 ? 1000000000 : static_cast<int32_t>(std::floor(x));
    };
    grow(c.gx0, -margin);
    grow(c.gy0, -margin);
    grow(c.gx1, margin + 1.0);
    grow(c.gy1, margin + 1.0);
}

// stroke(): the path's cubics are flattened with the stroking angle limit,
// then dashed and expanded on the device (k_dash, k_stroke).  The dash
// phase at the start of each subpath is computed here, as in hpp:1867-1876.
int queue_stroke(cy_ctx *c, const float *points, const int *counts, const int *closed, int n_sub,
                 const cy_stroke_style *style, const cy_paint *paint, const cy_draw_state *state) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!paint || !state || !style) return CY_EINVAL;
    if (state->mask < 0 || state->mask >= static_cast<int>(c->masks.size()) ||
        (state->mask > 0 && c->masks[state->mask].refs <= 0))
        return CY_EINVAL;
    size_t total = 0;
    if (n_sub < 0 || (n_sub > 0 && (!counts || !points || !closed)) || !valid_counts(counts, n_sub, total))
        return CY_EINVAL;
    for (int i = 0; i < n_sub; ++i)
        if (counts[i] != 0 && (counts[i] - 1) % 3 != 0) return CY_EINVAL;
    if (style->n_dash < 0 || (style->n_dash > 0 && !style->dash) || style->n_dash > (1 << 20) ||
        style->line_join < 0 || style->line_join > 2 || style->line_cap < 0 || style->line_cap > 2)
        return CY_EINVAL;
    const float *fw = style->forward;
    // stroke_lines and render_main draw nothing under a singular transform.
    if (fw[0] * fw[3] - fw[1] * fw[2] == 0.0f) return CY_OK;
    stroke_style st;
    std::memset(&st, 0, sizeof(st));
    st.half = style->line_width * 0.5f;
    st.ratio = style->miter_limit * style->miter_limit * st.half * st.half;
    st.join = style->line_join;
    st.cap = style->line_cap;
    for (int i = 0; i < 6; ++i) {
        st.fwd[i] = style->forward[i];
        st.inv[i] = style->inverse[i];
    }
    if (style->n_dash > 0) {
        const float *dash = style->dash;
        int nd = style->n_dash;
        float sum = 0.0f;
        for (int i = 0; i < nd; ++i) sum = sum + dash[i];
        float offset = fmodf(style->dash_offset, sum);
        if (offset < 0.0f) offset += sum;
        int start = 0, steps = 0;
        while (offset >= dash[start]) {
            offset -= dash[start];
            start = start + 1 < nd ? start + 1 : 0;
            if (++steps > 4 * nd + 8) return CY_EINVAL;   // offset within two periods of the pattern
        }
        st.dash_n = nd;
        st.dash_start = start;
        st.dash_next = dash[start] - offset;
    }
    float tol = 0.125f;
    float ratio = tol / (0.5f * style->line_width < tol ? tol : 0.5f * style->line_width);
    float angular = (ratio - 2.0f) * ratio * 2.0f + 1.0f;   // hpp:1498-1500
    queue &q = c->q;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_FILL;
    size_t stops = q.stop_off.size(), tex = q.texels.size();
    fill_state(state, cmd);
    cmd.fill_rule = 0;   // render_main fills the outline nonzero
    int rc = fill_paint(q, paint, cmd, c->device);
    if (rc != CY_OK) {
        q.stop_off.resize(stops);
        q.stop_col.resize(stops);
        q.texels.resize(tex);
        return rc;
    }
    stroke_bounds(points, total, st, cmd);
    cmd.geom = 2;
    cmd.first = static_cast<int32_t>(q.groups.size());
    int32_t style_id = static_cast<int32_t>(q.styles.size());
    st.dash_first = static_cast<int32_t>(q.dash.size());
    q.dash.insert(q.dash.end(), style->dash, style->dash + style->n_dash);
    q.styles.push_back(st);
    const float2 *p = reinterpret_cast<const float2 *>(points);
    int32_t pbase = static_cast<int32_t>(q.bez_pts.size());
    q.bez_pts.insert(q.bez_pts.end(), p, p + total);
    size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s];
        if (n == 0) continue;
        stroke_group g;
        g.head = static_cast<int32_t>(q.items.size());
        g.closed = closed[s] ? 1 : 0;
        g.style = style_id;
        flat_item head = {pbase + static_cast<int32_t>(at), 0, angular};
        q.items.push_back(head);
        for (int k = 1; k < n; k += 3) {
            flat_item cub = {pbase + static_cast<int32_t>(at + k - 1), -1, angular};
            q.items.push_back(cub);
        }
        g.end = static_cast<int32_t>(q.items.size());
        q.items[g.head].sub_end = g.end;
        q.groups.push_back(g);
        at += n;
    }
    cmd.count = static_cast<int32_t>(q.groups.size()) - cmd.first;
    q.bytes += total * 8 + (total / 3 + static_cast<size_t>(n_sub)) * 12 + static_cast<size_t>(cmd.count) * 16 +
               sizeof(stroke_style) + static_cast<size_t>(style->n_dash) * 4;
    q.rows += c->H + (cmd.shadow ? c->H + 2 * cmd.sh_border : 0);
    q.cmds.push_back(cmd);
    q.mask_ids.push_back(state->mask);
    q.mask_ids.push_back(0);
    if (state->mask > 0) c->masks[state->mask].refs++;
    return maybe_flush(c);
}

}  // namespace

// ------------------------------------------------------------- public ABI
extern "C" {

void cy_set_engine(int engine) { g_engine = engine; }
// Internal (the batch and serving paths): the context will be destroyed
// right after its next frame finishes, so the tile engine need not store
// its float pixels back (its reads are still written).
void cy_ctx_set_transient(cy_ctx *c, int transient) {
    if (c) c->transient = transient != 0;
}
void cy_set_coverage(int exact) { g_coverage.store(exact ? 1 : 0); }

int cy_image_cache_stats(long long *stats, int n) {
    if (!stats) return CY_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kTexDevices) {
        cudaGetLastError();
        return CY_ENODEV;
    }
    std::lock_guard<std::mutex> hold(g_tex_lock);
    const tex_cache &tc = g_tex[dev];
    long long entries = 0, texels = 0;
    for (const auto &kv : tc.map)
        for (const tex_entry &e : kv.second) {
            ++entries;
            texels += static_cast<long long>(e.w) * e.h;
        }
    long long v[] = {tc.hits, tc.inserts, entries, texels * 16, static_cast<long long>(tc.total)};
    int m = static_cast<int>(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) stats[i] = v[i];
    return m;
}
int cy_get_coverage(void) { return g_coverage.load(); }
void cy_set_deferred(int deferred) { g_deferred = deferred; }
void cy_set_strip_config(int pixels, int threads) {
    if (pixels >= 256 && pixels <= 12288) g_strip_pixels = pixels;
    if (threads == 128 || threads == 256 || threads == 512) g_strip_threads = threads;
}

// Internal: first engine failure raised in this thread since the last call.
int cy_take_thread_status(void) {
    int rc = g_thread_status;
    g_thread_status = 0;
    return rc;
}

int cy_ctx_create(int width, int height, cy_ctx **out) {
    if (!out) return CY_EINVAL;
    *out = nullptr;
    if (width < 1 || height < 1 || width > 32768 || height > 32768) return CY_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return CY_ENODEV;
    }
    cy_ctx *c = new (std::nothrow) cy_ctx();
    if (!c) return CY_ENOMEM;
    c->W = width;
    c->H = height;
    c->engine = g_engine;
    c->deferred = g_deferred != 0;
    // Canvases wider than a strip use the per-draw engine.
    if (width > g_strip_pixels) c->engine = 1;
    c->masks.resize(1);
    if (cudaGetDevice(&c->device) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return CY_ENODEV;
    }
    size_t npx = static_cast<size_t>(width) * static_cast<size_t>(height);
    auto okc = [&](cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        c->fail(e == cudaErrorMemoryAllocation ? CY_ENOMEM : CY_ECUDA);
        return false;
    };
    bool good = okc(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    if (good) {
        c->bitmap = static_cast<float4 *>(pool_get(npx * sizeof(float4), &c->bitmap_bytes));
        if (!c->bitmap) good = okc(cudaErrorMemoryAllocation);
    }
    // A deferred canvas is painted by frames that treat it as blank until it
    // has content, so only an immediate one starts from a cleared buffer.
    if (good && !c->deferred)
        good = okc(cudaMemsetAsync(c->bitmap, 0, npx * sizeof(float4), c->stream)) &&
               okc(cudaStreamSynchronize(c->stream));
    if (!good) {
        int rc = c->status;
        cy_ctx_destroy(c);
        return rc ? rc : CY_ECUDA;
    }
    *out = c;
    return CY_OK;
}

void cy_ctx_destroy(cy_ctx *c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    delete static_cast<frame *>(c->cached_frame);
    for (auto &m : c->masks) m.free_all();
    for (auto &m : c->dead) m.free_all();
    if (c->bitmap) pool_put(c->bitmap, c->bitmap_bytes);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int cy_ctx_status(const cy_ctx *c) { return c ? c->status : CY_EINVAL; }

int cy_fill_path(cy_ctx *c, const float *points, const int *counts, int n_sub, const cy_paint *paint,
                 const cy_draw_state *state) {
    return queue_draw(c, points, counts, n_sub, true, paint, state);
}

int cy_fill_lines(cy_ctx *c, const float *points, const int *counts, int n_sub, const cy_paint *paint,
                  const cy_draw_state *state) {
    return queue_draw(c, points, counts, n_sub, false, paint, state);
}

int cy_points_in_path(const float *points, const int *counts, int n_sub, const float *queries, int n_queries,
                      int fill_rule, unsigned char *inside) {
    if (n_sub < 0 || n_queries < 0 || (n_sub > 0 && (!points || !counts)) ||
        (n_queries > 0 && (!queries || !inside)))
        return CY_EINVAL;
    size_t total = 0;
    if (!valid_counts(counts, n_sub, total)) return CY_EINVAL;
    for (int s = 0; s < n_sub; ++s)
        if (counts[s] != 0 && (counts[s] - 1) % 3 != 0) return CY_EINVAL;
    if (n_queries == 0) return CY_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return CY_ENODEV;
    }
    // flattening items as for a fill, every subpath kept (path_to_lines(false))
    std::vector<flat_item> items;
    size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s];
        if (n == 0) continue;
        int32_t head = static_cast<int32_t>(items.size());
        items.push_back(flat_item{static_cast<int32_t>(at), 0, -1.0f});
        for (int k = 1; k < n; k += 3) items.push_back(flat_item{static_cast<int32_t>(at + k - 1), -1, -1.0f});
        items[head].sub_end = static_cast<int32_t>(items.size());
        at += static_cast<size_t>(n);
    }
    if (items.empty()) {
        std::memset(inside, 0, static_cast<size_t>(n_queries));
        return CY_OK;
    }
    const int ni = static_cast<int>(items.size());
    cudaStream_t st = nullptr;
    void *d_bez = nullptr, *d_items = nullptr, *d_cnt = nullptr, *d_off = nullptr, *d_pts = nullptr, *d_prev = nullptr,
         *d_q = nullptr, *d_in = nullptr;
    int rc = CY_OK;
    auto check = [&](cudaError_t e) {
        if (e == cudaSuccess || rc != CY_OK) return rc == CY_OK;
        cudaGetLastError();
        rc = e == cudaErrorMemoryAllocation ? CY_ENOMEM : CY_ECUDA;
        return false;
    };
    std::vector<int32_t> off(static_cast<size_t>(ni) + 1);
    if (check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) &&
        check(cudaMalloc(&d_bez, total * sizeof(float2))) && check(cudaMalloc(&d_items, items.size() * sizeof(flat_item))) &&
        check(cudaMalloc(&d_cnt, off.size() * 4)) && check(cudaMalloc(&d_off, off.size() * 4)) &&
        check(cudaMemcpyAsync(d_bez, points, total * sizeof(float2), cudaMemcpyHostToDevice, st)) &&
        check(cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(flat_item), cudaMemcpyHostToDevice, st))) {
        k_flat_count<<<(ni + 255) / 256, 256, 0, st>>>(static_cast<const float2 *>(d_bez),
                                                      static_cast<const flat_item *>(d_items), ni,
                                                      static_cast<int32_t *>(d_cnt));
        if (check(cudaGetLastError()) &&
            check(cudaMemcpyAsync(off.data(), d_cnt, static_cast<size_t>(ni) * 4, cudaMemcpyDeviceToHost, st)) &&
            check(cudaStreamSynchronize(st))) {
            // exclusive scan of the point counts on the host
            int64_t sum = 0;
            for (int i = 0; i < ni; ++i) {
                int32_t c = off[i];
                off[i] = static_cast<int32_t>(sum);
                sum += c;
            }
            if (sum <= 0 || sum > (static_cast<int64_t>(1) << 30)) rc = CY_ENOMEM;
            off[ni] = static_cast<int32_t>(sum);
            const size_t np = static_cast<size_t>(sum);
            if (rc == CY_OK && check(cudaMalloc(&d_pts, np * sizeof(float2))) && check(cudaMalloc(&d_prev, np * 4)) &&
                check(cudaMalloc(&d_q, static_cast<size_t>(n_queries) * sizeof(float2))) &&
                check(cudaMalloc(&d_in, static_cast<size_t>(n_queries))) &&
                check(cudaMemcpyAsync(d_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st)) &&
                check(cudaMemcpyAsync(d_q, queries, static_cast<size_t>(n_queries) * sizeof(float2),
                                      cudaMemcpyHostToDevice, st))) {
                k_flat_emit<<<(ni + 255) / 256, 256, 0, st>>>(static_cast<const float2 *>(d_bez),
                                                             static_cast<const flat_item *>(d_items), ni,
                                                             static_cast<const int32_t *>(d_off),
                                                             static_cast<float2 *>(d_pts), static_cast<int32_t *>(d_prev),
                                                             static_cast<int64_t>(np));
                k_points_in_path<<<(n_queries + 255) / 256, 256, 0, st>>>(
                    static_cast<const float2 *>(d_pts), static_cast<const int32_t *>(d_prev), static_cast<int>(np),
                    static_cast<const float2 *>(d_q), n_queries, fill_rule == 1 ? 1 : 0,
                    static_cast<unsigned char *>(d_in));
                if (check(cudaGetLastError()) &&
                    check(cudaMemcpyAsync(inside, d_in, static_cast<size_t>(n_queries), cudaMemcpyDeviceToHost, st)))
                    check(cudaStreamSynchronize(st));
            }
        }
    }
    if (st) cudaStreamSynchronize(st);
    for (void *p : {d_bez, d_items, d_cnt, d_off, d_pts, d_prev, d_q, d_in})
        if (p) cudaFree(p);
    if (st) cudaStreamDestroy(st);
    cudaGetLastError();
    return rc;
}

int cy_stroke_path(cy_ctx *c, const float *points, const int *counts, const int *closed, int n_sub,
                   const cy_stroke_style *style, const cy_paint *paint, const cy_draw_state *state) {
    return queue_stroke(c, points, counts, closed, n_sub, style, paint, state);
}

void cy_set_device_stroke(int on) { g_device_stroke.store(on ? 1 : 0); }
int cy_device_stroke(void) { return g_device_stroke.load(); }

int cy_mask_retain(cy_ctx *c, int mask) {
    if (!c || mask <= 0 || mask >= static_cast<int>(c->masks.size()) || c->masks[mask].refs <= 0)
        return CY_EINVAL;
    c->masks[mask].refs++;
    return CY_OK;
}

int cy_mask_release(cy_ctx *c, int mask) {
    if (!c || mask <= 0 || mask >= static_cast<int>(c->masks.size()) || c->masks[mask].refs <= 0)
        return CY_EINVAL;
    if (--c->masks[mask].refs == 0) {
        c->dead.push_back(c->masks[mask]);
        c->masks[mask] = mask_slot();
    }
    return CY_OK;
}

int cy_clip_path(cy_ctx *c, const float *points, const int *counts, int n_sub, int mask_in, int fill_rule,
                 int *mask_out) {
    if (!c || !mask_out) return CY_EINVAL;
    if (c->status) return c->status;
    if (mask_in < 0 || mask_in >= static_cast<int>(c->masks.size()) ||
        (mask_in > 0 && c->masks[mask_in].refs <= 0))
        return CY_EINVAL;
    queue &q = c->q;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_CLIP;
    cmd.fill_rule = fill_rule == 1 ? 1 : 0;
    cull_rects rects = {static_cast<float>(c->W), static_cast<float>(c->H), false, 0.0f, 0.0f, 0.0f, 0.0f, false};
    int rc = queue_geometry(q, points, counts, n_sub, true, cmd, rects);
    if (rc != CY_OK) return rc;
    int id = 0;
    for (int i = 1; i < static_cast<int>(c->masks.size()); ++i)
        if (c->masks[i].refs == 0 && !c->masks[i].vis) { id = i; break; }
    if (id == 0) {
        id = static_cast<int>(c->masks.size());
        c->masks.emplace_back();
    }
    mask_slot &m = c->masks[id];
    size_t H1 = static_cast<size_t>(c->H) + 1;
    auto okc = [&](cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        c->fail(CY_ENOMEM, __LINE__);
        return false;
    };
    if (!okc(cudaMalloc(&m.vis, static_cast<size_t>(c->W) * c->H * sizeof(float))) ||
        !okc(cudaMalloc(&m.off, H1 * 4)) || !okc(cudaMalloc(&m.len, H1 * 4)) || !okc(cudaMalloc(&m.last_row, 4))) {
        // Give back what was allocated, so the slot can be taken again.
        m.free_all();
        m = mask_slot();
        return c->status;
    }
    m.refs = 2;   // the caller's reference plus the queued command's
    q.rows += c->H;
    q.cmds.push_back(cmd);
    q.mask_ids.push_back(mask_in);
    q.mask_ids.push_back(id);
    if (mask_in > 0) c->masks[mask_in].refs++;
    *mask_out = id;
    return maybe_flush(c);
}

int cy_put_image(cy_ctx *c, const unsigned char *image, int w, int h, int stride, int x, int y) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!image || w <= 0 || h <= 0) return CY_OK;
    queue &q = c->q;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_PUT;
    cmd.put_x = x; cmd.put_y = y; cmd.put_w = w; cmd.put_h = h;
    cmd.put_first = static_cast<int64_t>(q.put_px.size());
    for (int row = 0; row < h; ++row) {
        const unsigned char *src = image + static_cast<ptrdiff_t>(row) * stride;
        q.put_px.insert(q.put_px.end(), src, src + static_cast<size_t>(w) * 4);
    }
    q.cmds.push_back(cmd);
    q.mask_ids.push_back(0);
    q.mask_ids.push_back(0);
    q.bytes += static_cast<size_t>(w) * h * 4;
    return maybe_flush(c);
}

int cy_flush(cy_ctx *c) {
    if (!c) return CY_EINVAL;
    int rc = flush_ctx(c);
    if (rc) return rc;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        return c->fail(CY_ECUDA);
    }
    return CY_OK;
}

int cy_get_image(cy_ctx *c, unsigned char *image, int w, int h, int stride, int x, int y) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!image || w <= 0 || h <= 0) return CY_OK;
    queue &q = c->q;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_GET;
    cmd.get_x = x; cmd.get_y = y; cmd.get_w = w; cmd.get_h = h;
    cmd.get_out = q.get_bytes;
    q.get_bytes += static_cast<int64_t>(w) * h * 4;   // packed: a context's reads are one range
    q.cmds.push_back(cmd);
    q.mask_ids.push_back(0);
    q.mask_ids.push_back(0);
    q.get_dst.push_back(c->deferred ? nullptr : image);
    q.get_stride.push_back(stride);
    if (c->deferred) return CY_OK;
    return flush_ctx(c);
}

int cy_encode_image(cy_ctx *c, int format, int x, int y, int w, int h, unsigned char *out, size_t cap,
                    size_t *len) {
    if (!c || (format != encode::TGA && format != encode::PNG) || w <= 0 || h <= 0 || w > 65535 || h > 65535)
        return CY_EINVAL;
    if (format == encode::PNG && (w > 16383 || encode::png_size(w, h) > static_cast<size_t>(INT32_MAX)))
        return CY_EINVAL;   // one stored block per row, and the writer's int sizes
    const bool png = format == encode::PNG;
    const size_t size = png ? encode::png_size(w, h) : encode::tga_size(w, h);
    if (len) *len = size;
    if (!out || cap < size) return CY_ENOMEM;
    if (c->status) return c->status;
    if (int rc = flush_ctx(c)) return rc;
    if (int rc = ensure_srgb_table()) return rc;
    unsigned char *d_out = nullptr;
    uint32_t *d_sums = nullptr;
    std::vector<uint32_t> sums(png ? static_cast<size_t>(h) * 3 : 0);
    auto okc = [&](cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        return false;
    };
    int rc = CY_OK;
    if (!okc(cudaMalloc(&d_out, size)) || (png && !okc(cudaMalloc(&d_sums, sums.size() * 4)))) {
        rc = CY_ENOMEM;
    } else {
        dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8);
        k_encode<<<grd, blk, 0, c->stream>>>(c->bitmap, c->W, c->H, c->has_content ? 0 : 1, w, h, x, y, png ? 1 : 0,
                                             d_out);
        if (png)
            k_png_rows<<<(h + 127) / 128, 128, 0, c->stream>>>(d_out, w, h, d_sums, d_sums + h, d_sums + 2 * h);
        if (!okc(cudaGetLastError()) || !okc(cudaMemcpyAsync(out, d_out, size, cudaMemcpyDeviceToHost, c->stream)) ||
            (png && !okc(cudaMemcpyAsync(sums.data(), d_sums, sums.size() * 4, cudaMemcpyDeviceToHost, c->stream))) ||
            !okc(cudaStreamSynchronize(c->stream)))
            rc = c->fail(CY_ECUDA);
    }
    if (d_out) cudaFree(d_out);
    if (d_sums) cudaFree(d_sums);
    if (rc) return rc;
    if (png) encode::png_frame(out, w, h, sums.data(), sums.data() + h, sums.data() + 2 * static_cast<size_t>(h));
    else encode::tga_header(out, w, h);
    return CY_OK;
}

int cy_read_linear(cy_ctx *c, float *out) {
    if (!c || !out) return CY_EINVAL;
    int rc = flush_ctx(c);
    if (rc) return rc;
    size_t bytes = static_cast<size_t>(c->W) * c->H * sizeof(float4);
    if (!c->has_content) {   // never painted: transparent black (a deferred buffer is not cleared)
        std::memset(out, 0, bytes);
        return CY_OK;
    }
    if (cudaMemcpyAsync(out, c->bitmap, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        return c->fail(CY_ECUDA);
    }
    return CY_OK;
}

// ------------------------------------------- allocation-free image readback
// cy_get_image_noalloc: the RGBA8 conversion of cy_get_image with its device
// staging buffer replaced by one fixed array in this file, so the call makes
// no allocation of any kind.  The array lives in every GPU that loads this
// library, until the process exits.
static __device__ __align__(256) uchar4 g_noalloc_rgba[CY_GET_IMAGE_NOALLOC_MAX_PIXELS];

namespace {
std::mutex g_noalloc_lock;             // serialises the calls of this process
constexpr int kNoallocDevices = 64;
uchar4 *g_noalloc_addr[kNoallocDevices] = {};   // device address of the array, per device
}  // namespace

extern "C" int cy_get_image_noalloc(cy_ctx *c, unsigned char *image, int w, int h, int stride, int x, int y) {
    if (!c || !image || w <= 0 || h <= 0) return CY_EINVAL;
    if (static_cast<int64_t>(w) * h > CY_GET_IMAGE_NOALLOC_MAX_PIXELS) return CY_EINVAL;
    if (static_cast<int64_t>(stride) < static_cast<int64_t>(w) * 4) return CY_EINVAL;
    if (c->status) return c->status;
    // Queued draws would need a frame run, which allocates: flush them first.
    if (!c->q.cmds.empty()) return CY_EINVAL;
    if (!c->has_content) {   // never painted: every byte is zero (the buffer itself is not cleared)
        for (int row = 0; row < h; ++row) std::memset(image + static_cast<size_t>(row) * stride, 0, static_cast<size_t>(w) * 4);
        return CY_OK;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocDevices) {
        cudaGetLastError();
        return CY_ENODEV;
    }
    // The array used is the current device's: it must be the canvas's own
    // (a caller's mistake, answered without marking the context failed).
    if (dev != c->device) return CY_EINVAL;
    std::lock_guard<std::mutex> hold(g_noalloc_lock);
    if (!g_noalloc_addr[dev]) {
        // Set-up, once per device, with that device current: host code must
        // use the array's device address, not its host-side name.
        void *addr = nullptr;
        if (cudaGetSymbolAddress(&addr, g_noalloc_rgba) != cudaSuccess || !addr) {
            cudaGetLastError();
            return CY_ECUDA;
        }
        g_noalloc_addr[dev] = static_cast<uchar4 *>(addr);
    }
    uchar4 *staging = g_noalloc_addr[dev];
    // The colour conversion's threshold table (16 KiB, also a fixed array)
    // is uploaded to the device by its first use in this process.
    if (int rc = ensure_srgb_table()) return rc;
    // k_get writes every pixel of the w x h rectangle (zero outside the
    // canvas), so nothing in the array has to start at zero.
    dim3 blk(32, 32), grd((w + 31) / 32, (h + 31) / 32);
    k_get<<<grd, blk, 0, c->stream>>>(c->bitmap, c->W, c->H, staging, w, h, x, y);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy2DAsync(image, static_cast<size_t>(stride), staging, static_cast<size_t>(w) * 4,
                          static_cast<size_t>(w) * 4, static_cast<size_t>(h), cudaMemcpyDeviceToHost,
                          c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        return c->fail(CY_ECUDA);
    }
    return CY_OK;
}

// ------------------------------------------------------------ batched API
struct cy_frame {
    std::unique_ptr<frame> f;
    cudaStream_t stream = nullptr;
};

// Device workspaces of finished frames, a few per device: the next frames
// reuse their buffers instead of allocating them again.
namespace {
std::mutex g_ws_lock;
std::vector<std::pair<int, std::unique_ptr<frame>>> g_ws;

std::unique_ptr<frame> take_workspace() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    std::lock_guard<std::mutex> hold(g_ws_lock);
    for (auto &w : g_ws)
        if (w.first == dev && w.second) return std::move(w.second);
    return nullptr;
}

constexpr int kWorkspacesPerDevice = 4;   // concurrent frames (server workers) keep theirs

void give_workspace(std::unique_ptr<frame> f) {
    int dev = -1;
    if (!f || f->status || cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return; }
    f->reset();
    std::unique_ptr<frame> spare;
    {
        std::lock_guard<std::mutex> hold(g_ws_lock);
        int held = 0;
        for (auto &w : g_ws)
            if (w.first == dev) {
                if (!w.second) { w.second = std::move(f); return; }
                ++held;
            }
        if (held >= kWorkspacesPerDevice) spare = std::move(f);   // enough kept: free this one
        else g_ws.emplace_back(dev, std::move(f));
    }
}
}  // namespace

void cy_frame_destroy(cy_frame *fr) {
    if (!fr) return;
    if (fr->stream) cudaStreamSynchronize(fr->stream);
    give_workspace(std::move(fr->f));
    fr->f.reset();
    if (fr->stream) cudaStreamDestroy(fr->stream);
    delete fr;
}

void cy_frame_workspace_release(void) {
    std::vector<std::pair<int, std::unique_ptr<frame>>> all;
    {
        std::lock_guard<std::mutex> hold(g_ws_lock);
        all.swap(g_ws);
    }
    int dev = -1;
    cudaGetDevice(&dev);
    for (auto &w : all)
        if (w.second) {
            cudaSetDevice(w.first);
            w.second.reset();
        }
    if (dev >= 0) cudaSetDevice(dev);
    cudaGetLastError();
}

int cy_frame_create(cy_ctx *const *ctxs, int n, int engine, cy_frame **out) {
    if (!out || n < 0 || (n > 0 && !ctxs)) return CY_EINVAL;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i]) return CY_EINVAL;
        if (ctxs[i]->status) return ctxs[i]->status;
        if (engine == 0 && ctxs[i]->W > g_strip_pixels) return CY_EINVAL;
    }
    cy_frame *fr = new (std::nothrow) cy_frame();
    if (!fr) return CY_ENOMEM;
    fr->f = take_workspace();
    if (!fr->f) fr->f.reset(new frame());
    if (cudaStreamCreateWithFlags(&fr->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete fr;
        return CY_ECUDA;
    }
    fr->f->stream = fr->stream;
    fr->f->engine = engine;
    for (int i = 0; i < n; ++i) fr->f->cvs.push_back(ctxs[i]);
    int rc = fr->f->prepare();
    if (rc) {
        cy_frame_destroy(fr);
        return rc;
    }
    *out = fr;
    return CY_OK;
}

int cy_frame_run(cy_frame *fr) {
    if (!fr) return CY_EINVAL;
    frame &f = *fr->f;
    if (f.graph_exec && !f.profiling) {
        if (f.status) return f.status;
        if (cudaGraphLaunch(f.graph_exec, fr->stream) != cudaSuccess) {
            cudaGetLastError();
            return f.fail(CY_ECUDA);
        }
        return CY_OK;
    }
    return f.run();
}

int cy_frame_autotune(cy_frame *fr, int *best_pixels, int *best_threads, float *best_ms) {
    if (!fr) return CY_EINVAL;
    frame &f = *fr->f;
    if (f.status) return f.status;
    if (!f.sized || f.engine != 0) return CY_EINVAL;
    int max_w = 1;
    for (cy_ctx *cv : f.cvs) {
        if (!cv->deferred) return CY_EINVAL;   // the paint stage must be repeatable
        max_w = std::max(max_w, cv->W);
    }
    const int pixels[] = {2048, 4096, 8192, 12288};
    const int threads[] = {128, 256, 512};
    int keep_p = g_strip_pixels, keep_t = g_strip_threads;
    int bp = 0, bt = 0;
    float bms = 0.0f;
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        cudaGetLastError();
        if (a) cudaEventDestroy(a);
        return CY_ECUDA;
    }
    f.drop_graph();
    int rc = CY_OK;
    for (int px : pixels) {
        if (px < max_w || (f.binned && px > kBinnedMaxStrip)) continue;
        for (int th : threads) {
            g_strip_pixels = px;
            g_strip_threads = th;
            f.strips_built = false;
            rc = f.build_strips();
            if (rc == CY_OK) rc = f.launch_strips();   // warm-up
            float ms = 0.0f;
            for (int rep = 0; rep < 2 && rc == CY_OK; ++rep) {
                cudaEventRecord(a, fr->stream);
                rc = f.launch_strips();
                cudaEventRecord(b, fr->stream);
                float t = 0.0f;
                if (rc == CY_OK && (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&t, a, b) != cudaSuccess)) {
                    cudaGetLastError();
                    rc = f.fail(CY_ECUDA);
                }
                if (rep == 0 || t < ms) ms = t;
            }
            if (rc != CY_OK) break;
            if (bp == 0 || ms < bms) { bp = px; bt = th; bms = ms; }
        }
        if (rc != CY_OK) break;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    g_strip_pixels = bp ? bp : keep_p;
    g_strip_threads = bt ? bt : keep_t;
    if (rc != CY_OK) return rc;
    f.strips_built = false;
    rc = f.build_strips();
    if (rc != CY_OK) return rc;
    if (best_pixels) *best_pixels = bp;
    if (best_threads) *best_threads = bt;
    if (best_ms) *best_ms = bms;
    return bp ? CY_OK : CY_EINVAL;
}

int cy_frame_capture(cy_frame *fr) {
    if (!fr) return CY_EINVAL;
    frame &f = *fr->f;
    if (f.status) return f.status;
    if (!f.sized) return CY_EINVAL;   // the first run sizes the buffers with host read-backs
    f.drop_graph();
    bool was_profiling = f.profiling;
    f.profiling = false;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(fr->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        f.profiling = was_profiling;
        return CY_ECUDA;
    }
    int rc = f.run();
    cudaError_t e = cudaStreamEndCapture(fr->stream, &g);
    f.profiling = was_profiling;
    if (rc != CY_OK || e != cudaSuccess || !g) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        return rc != CY_OK ? rc : f.fail(CY_ECUDA);
    }
    cudaGraphExec_t x = nullptr;
    e = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return CY_ECUDA;
    }
    f.graph_exec = x;
    return CY_OK;
}

int cy_frame_finish(cy_frame *fr) { return fr ? fr->f->finish() : CY_EINVAL; }

int cy_frame_finish_views(cy_frame *fr, const unsigned char **data, size_t *offsets) {
    if (!fr || !data || !offsets) return CY_EINVAL;
    frame &f = *fr->f;
    f.keep_reads = true;
    int rc = f.finish();
    f.keep_reads = false;
    if (rc) return rc;
    size_t n = f.cvs.size();
    for (size_t i = 0; i < n; ++i) offsets[i] = static_cast<size_t>(f.get_base[i]);
    offsets[n] = static_cast<size_t>(f.get_total);
    *data = static_cast<const unsigned char *>(f.get_host.p);
    return CY_OK;
}

int cy_frame_sync(cy_frame *fr) {
    if (!fr) return CY_EINVAL;
    if (cudaStreamSynchronize(fr->stream) != cudaSuccess) {
        cudaGetLastError();
        return fr->f->fail(CY_ECUDA);
    }
    return fr->f->status;
}

void *cy_frame_stream(cy_frame *fr) { return fr ? static_cast<void *>(fr->stream) : nullptr; }

int cy_frame_set_profiling(cy_frame *fr, int on) {
    if (!fr) return CY_EINVAL;
    frame &f = *fr->f;
    if (on && !f.ev[0])
        for (cudaEvent_t &e : f.ev)
            if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return CY_ECUDA; }
    f.profiling = on != 0;
    return CY_OK;
}

int cy_frame_profile(cy_frame *fr, float *phase_ms, int n) {
    if (!fr || !phase_ms) return CY_EINVAL;
    frame &f = *fr->f;
    if (cudaStreamSynchronize(fr->stream) != cudaSuccess) { cudaGetLastError(); return CY_ECUDA; }
    for (int i = 0; i < n; ++i) phase_ms[i] = 0.0f;
    for (int i = 0; i + 1 < f.n_ev && i < n; ++i)
        if (cudaEventElapsedTime(&phase_ms[i], f.ev[i], f.ev[i + 1]) != cudaSuccess) cudaGetLastError();
    return f.n_ev > 0 ? f.n_ev - 1 : 0;
}

int cy_frame_stats(cy_frame *fr, long long *stats, int n) {
    if (!fr || !stats) return CY_EINVAL;
    frame &f = *fr->f;
    long long pixels = 0;
    for (cy_ctx *c : f.cvs) pixels += static_cast<long long>(c->W) * c->H;
    long long v[] = {pixels, static_cast<long long>(f.all.cmds.size()), f.nc_segs + f.bn_segs + f.pass_n[4], f.n_runs, f.total_rows,
                     f.main_runs, f.main_rows, f.shadow_floats, f.get_total, f.h2d_bytes, f.launches,
                     static_cast<long long>(f.sjobs.size()), static_cast<long long>(f.clips.size()),
                     f.n_bin_entries, f.binned ? 1LL : 0LL};
    int m = static_cast<int>(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) stats[i] = v[i];
    return m;
}

int cy_frame_collect(cy_frame *fr, unsigned char *out, size_t cap, size_t *offsets) {
    if (!fr || !offsets) return CY_EINVAL;
    frame &f = *fr->f;
    size_t n = f.cvs.size(), total = 0;
    for (size_t i = 0; i < n; ++i) {
        offsets[i] = total;
        total += f.cvs[i]->deferred_out.size();
    }
    offsets[n] = total;
    if (total > cap || (total && !out)) return -2;
    parallel_for(n, [&](size_t i) {
        std::vector<uint8_t> &d = f.cvs[i]->deferred_out;
        if (!d.empty()) std::memcpy(out + offsets[i], d.data(), d.size());
        std::vector<uint8_t>().swap(d);
    });
    return CY_OK;
}

int cy_ctx_take_reads(cy_ctx *c, unsigned char *out, size_t cap, size_t *len) {
    if (!c) return CY_EINVAL;
    if (len) *len = c->deferred_out.size();
    if (c->deferred_out.size() > cap) return -2;
    if (!c->deferred_out.empty()) std::memcpy(out, c->deferred_out.data(), c->deferred_out.size());
    c->deferred_out.clear();
    return CY_OK;
}

}  // extern "C"
