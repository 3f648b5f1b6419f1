// engine.cu -- the GB300 render engine behind include/cy_gpu.h.
//
// A context owns one canvas on the GPU: the premultiplied linear float RGBA
// bitmap (hpp:1171), a zeroed fixed-point delta plane for scan conversion,
// and the clip masks.  Calls queue commands on the host; a flush uploads all
// queued geometry and paint in one copy, flattens every Bezier path in one
// launch pair, then runs each command's kernels in call order on the
// context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/cy_gpu.h"
#include "engine_types.h"
#include "kernels.cuh"

using namespace cyg;

namespace {

thread_local int g_engine = 1;
thread_local int g_thread_status = 0;  // first failure in this thread since the last take

struct dbuf {
    void *p = nullptr;
    size_t cap = 0;
    // Grow to at least `bytes`; contents are not preserved.
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        size_t n = std::max(std::max(bytes, static_cast<size_t>(256)), cap + cap / 2);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, n) != cudaSuccess) { cudaGetLastError(); return false; }
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
        if (bytes <= cap) return true;
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

// A clip mask: the reference's sparse runs per row plus the dense
// visibility they imply.  Created by a queued clip, filled at the flush.
struct mask_slot {
    float *vis = nullptr;       // W*H
    int32_t *off = nullptr;     // H+1
    int32_t *len = nullptr;     // H
    run *runs = nullptr;
    float *sums = nullptr;
    int *last_row = nullptr;    // device int: last row holding runs
    int64_t cap = 0;            // run capacity
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

inline size_t align256(size_t v) { return (v + 255) & ~static_cast<size_t>(255); }

}  // namespace

struct cy_ctx {
    int W = 0, H = 0;
    int status = 0;
    cudaStream_t stream = nullptr;
    float4 *bitmap = nullptr;
    float *lut = nullptr;
    std::vector<mask_slot> masks;   // id 0 unused (whole canvas)
    std::vector<mask_slot> dead;    // released masks, freed after the next flush
    // queued work
    std::vector<command> cmds;
    std::vector<float2> host_pts;
    std::vector<int32_t> host_prev;
    std::vector<float2> bez_pts;
    std::vector<flat_item> items;
    std::vector<float> stop_off;
    std::vector<float4> stop_col;
    std::vector<uchar4> texels;
    std::vector<uint8_t> put_px;
    std::vector<int32_t> mask_ids;  // per command: mask_in id, mask_out id
    size_t queued_bytes = 0;
    int64_t queued_rows = 0;   // scan-conversion rows the queued commands need
    // per-flush device scratch
    dbuf arena, flat_pts, flat_prev, item_cnt, item_off, boxes, pat_f4;
    dbuf jobs_dev, row_cnt, row_off, row_cur, row_len, runs, sums;
    dbuf sh_a, sh_b, sh_rect, get_dev;
    hbuf staging, get_host, offs_host, rowoff_host;

    int fail(int rc) {
        if (status == 0) status = rc;
        if (g_thread_status == 0) g_thread_status = rc;
        return rc;
    }
    bool ok(cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        fail(e == cudaErrorMemoryAllocation ? CY_ENOMEM : CY_ECUDA);
        return false;
    }
    int flush();
    int scan(const int32_t *in, int32_t *out, int n);
    int clip_mask(const command &c, int mask_in, int mask_out, const scan_job &job, int job_index,
                  const int32_t *rowoff_h);
};

// ------------------------------------------------------------ host helpers
namespace {

void bounds_of(const float *xy, size_t n, command &c) {
    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (size_t i = 0; i < n; ++i) {
        float x = xy[2 * i], y = xy[2 * i + 1];
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
    // NaN coordinates make the bounds unknown: use the whole canvas.
    bool bad = !(x0 <= x1) || !(y0 <= y1);
    c.gx0 = bad ? -1000000000 : clampi(x0);
    c.gy0 = bad ? -1000000000 : clampi(y0);
    c.gx1 = bad ? 1000000000 : clampi(x1) + 1;
    c.gy1 = bad ? 1000000000 : clampi(y1) + 1;
}

int fill_paint(cy_ctx *ctx, const cy_paint *p, command &c) {
    c.paint = p->kind;
    c.clamp = p->clamp_edges;
    for (int i = 0; i < 6; ++i) c.inv[i] = p->inverse[i];
    for (int i = 0; i < 4; ++i) c.color[i] = p->color[i];
    c.p0x = p->start[0]; c.p0y = p->start[1]; c.p1x = p->end[0]; c.p1y = p->end[1];
    c.r0 = p->start_radius; c.r1 = p->end_radius;
    c.stop_first = c.stop_count = 0;
    c.pat_first = c.pat_w = c.pat_h = c.pat_rep = 0;
    if (p->kind == CY_PAINT_LINEAR || p->kind == CY_PAINT_RADIAL) {
        if (p->n_stops <= 0) { c.paint = CY_PAINT_NONE; return CY_OK; }
        if (!p->stop_offsets || !p->stop_colors) return CY_EINVAL;
        c.stop_first = static_cast<int32_t>(ctx->stop_off.size());
        c.stop_count = p->n_stops;
        for (int i = 0; i < p->n_stops; ++i) {
            ctx->stop_off.push_back(p->stop_offsets[i]);
            ctx->stop_col.push_back(make_float4(p->stop_colors[4 * i], p->stop_colors[4 * i + 1],
                                                p->stop_colors[4 * i + 2], p->stop_colors[4 * i + 3]));
        }
        ctx->queued_bytes += static_cast<size_t>(p->n_stops) * 20;
    } else if (p->kind == CY_PAINT_PATTERN) {
        if (!p->pattern || p->pattern_width <= 0 || p->pattern_height <= 0) return CY_EINVAL;
        size_t n = static_cast<size_t>(p->pattern_width) * static_cast<size_t>(p->pattern_height);
        if (ctx->texels.size() + n > static_cast<size_t>(INT32_MAX)) return CY_EINVAL;
        c.pat_first = static_cast<int32_t>(ctx->texels.size());
        c.pat_w = p->pattern_width;
        c.pat_h = p->pattern_height;
        c.pat_rep = p->repetition;
        const uchar4 *src = reinterpret_cast<const uchar4 *>(p->pattern);
        ctx->texels.insert(ctx->texels.end(), src, src + n);
        ctx->queued_bytes += n * 4;
    } else if (p->kind != CY_PAINT_NONE && p->kind != CY_PAINT_SOLID) {
        return CY_EINVAL;
    }
    return CY_OK;
}

void fill_state(const cy_draw_state *s, command &c) {
    c.op = s->operation;
    c.alpha = s->global_alpha;
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

}  // namespace

// ------------------------------------------------------------- public ABI
extern "C" {

void cy_set_engine(int engine) { g_engine = engine; }

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
    c->masks.resize(1);
    size_t npx = static_cast<size_t>(width) * static_cast<size_t>(height);
    bool ok = c->ok(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) &&
              c->ok(cudaMalloc(&c->bitmap, npx * sizeof(float4))) &&
              c->ok(cudaMalloc(&c->lut, 256 * sizeof(float))) &&
              c->ok(cudaMemsetAsync(c->bitmap, 0, npx * sizeof(float4), c->stream)) &&
              c->ok(cudaMemcpyAsync(c->lut, linear_lut_host(), 256 * sizeof(float), cudaMemcpyHostToDevice,
                                    c->stream)) &&
              c->ok(cudaStreamSynchronize(c->stream));
    if (!ok) {
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
    for (auto &m : c->masks) m.free_all();
    for (auto &m : c->dead) m.free_all();
    if (c->bitmap) cudaFree(c->bitmap);
    if (c->lut) cudaFree(c->lut);
    dbuf *bufs[] = {&c->arena, &c->flat_pts, &c->flat_prev, &c->item_cnt, &c->item_off, &c->boxes,
                    &c->pat_f4, &c->jobs_dev, &c->row_cnt, &c->row_off, &c->row_cur, &c->row_len,
                    &c->runs, &c->sums, &c->sh_a, &c->sh_b, &c->sh_rect, &c->get_dev};
    for (dbuf *b : bufs) b->release();
    c->staging.release();
    c->get_host.release();
    c->offs_host.release();
    c->rowoff_host.release();
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int cy_ctx_status(const cy_ctx *c) { return c ? c->status : CY_EINVAL; }

static int queue_geometry(cy_ctx *c, const float *points, const int *counts, int n_sub, bool bezier,
                          command &cmd) {
    size_t total = 0;
    if (n_sub < 0 || (n_sub > 0 && (!counts || !points)) || !valid_counts(counts, n_sub, total))
        return CY_EINVAL;
    bounds_of(points, total, cmd);
    const float2 *p = reinterpret_cast<const float2 *>(points);
    if (!bezier) {
        cmd.geom = 0;
        cmd.first = static_cast<int32_t>(c->host_pts.size());
        cmd.count = static_cast<int32_t>(total);
        size_t at = 0;
        for (int s = 0; s < n_sub; ++s) {
            int32_t base = static_cast<int32_t>(c->host_pts.size());
            int n = counts[s];
            for (int k = 0; k < n; ++k) {
                c->host_pts.push_back(p[at + k]);
                c->host_prev.push_back(k == 0 ? base + n - 1 : base + k - 1);
            }
            at += n;
        }
        c->queued_bytes += total * 12;
        return CY_OK;
    }
    // Bezier path: one flattening item per subpath start and per cubic.
    cmd.geom = 1;
    cmd.first = static_cast<int32_t>(c->items.size());
    int32_t pbase = static_cast<int32_t>(c->bez_pts.size());
    c->bez_pts.insert(c->bez_pts.end(), p, p + total);
    size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s];
        if (n == 0) continue;
        if ((n - 1) % 3 != 0) return CY_EINVAL;
        int32_t start = static_cast<int32_t>(c->items.size());
        flat_item head = {pbase + static_cast<int32_t>(at), 0};
        c->items.push_back(head);
        for (int k = 1; k < n; k += 3) {
            flat_item cub = {pbase + static_cast<int32_t>(at + k - 1), -1};
            c->items.push_back(cub);
        }
        c->items[start].sub_end = static_cast<int32_t>(c->items.size());
        at += n;
    }
    cmd.count = static_cast<int32_t>(c->items.size()) - cmd.first;
    c->queued_bytes += total * 8 + static_cast<size_t>(cmd.count) * 8;
    return CY_OK;
}

static int queue_draw(cy_ctx *c, const float *points, const int *counts, int n_sub, bool bezier,
                      const cy_paint *paint, const cy_draw_state *state) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!paint || !state) return CY_EINVAL;
    if (state->mask < 0 || state->mask >= static_cast<int>(c->masks.size()) ||
        (state->mask > 0 && c->masks[state->mask].refs <= 0))
        return CY_EINVAL;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_FILL;
    size_t stops = c->stop_off.size(), tex = c->texels.size();
    int rc = fill_paint(c, paint, cmd);
    if (rc == CY_OK) rc = queue_geometry(c, points, counts, n_sub, bezier, cmd);
    if (rc != CY_OK) {
        c->stop_off.resize(stops);
        c->stop_col.resize(stops);
        c->texels.resize(tex);
        return rc;
    }
    fill_state(state, cmd);
    c->queued_rows += c->H + (cmd.shadow ? c->H + 2 * cmd.sh_border : 0);
    c->cmds.push_back(cmd);
    c->mask_ids.push_back(state->mask);
    c->mask_ids.push_back(0);
    if (state->mask > 0) c->masks[state->mask].refs++;   // held until the flush
    if (c->queued_bytes > (static_cast<size_t>(256) << 20) || c->cmds.size() >= 65536 ||
        c->queued_rows > (static_cast<int64_t>(16) << 20))
        return c->flush();
    return CY_OK;
}

int cy_fill_path(cy_ctx *c, const float *points, const int *counts, int n_sub, const cy_paint *paint,
                 const cy_draw_state *state) {
    return queue_draw(c, points, counts, n_sub, true, paint, state);
}

int cy_fill_lines(cy_ctx *c, const float *points, const int *counts, int n_sub, const cy_paint *paint,
                  const cy_draw_state *state) {
    return queue_draw(c, points, counts, n_sub, false, paint, state);
}

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

int cy_clip_path(cy_ctx *c, const float *points, const int *counts, int n_sub, int mask_in, int *mask_out) {
    if (!c || !mask_out) return CY_EINVAL;
    if (c->status) return c->status;
    if (mask_in < 0 || mask_in >= static_cast<int>(c->masks.size()) ||
        (mask_in > 0 && c->masks[mask_in].refs <= 0))
        return CY_EINVAL;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_CLIP;
    int rc = queue_geometry(c, points, counts, n_sub, true, cmd);
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
    if (!c->ok(cudaMalloc(&m.vis, static_cast<size_t>(c->W) * c->H * sizeof(float))) ||
        !c->ok(cudaMalloc(&m.off, H1 * 4)) || !c->ok(cudaMalloc(&m.len, H1 * 4)) ||
        !c->ok(cudaMalloc(&m.last_row, 4)))
        return c->status;
    m.refs = 2;   // the caller's reference plus the queued command's
    c->queued_rows += c->H;
    c->cmds.push_back(cmd);
    c->mask_ids.push_back(mask_in);
    c->mask_ids.push_back(id);
    if (mask_in > 0) c->masks[mask_in].refs++;
    *mask_out = id;
    return CY_OK;
}

int cy_put_image(cy_ctx *c, const unsigned char *image, int w, int h, int stride, int x, int y) {
    if (!c) return CY_EINVAL;
    if (c->status) return c->status;
    if (!image || w <= 0 || h <= 0) return CY_OK;
    command cmd;
    std::memset(&cmd, 0, sizeof(cmd));
    cmd.kind = CMD_PUT;
    cmd.put_x = x; cmd.put_y = y; cmd.put_w = w; cmd.put_h = h;
    cmd.put_first = static_cast<int64_t>(c->put_px.size());
    for (int row = 0; row < h; ++row) {
        const unsigned char *src = image + static_cast<ptrdiff_t>(row) * stride;
        c->put_px.insert(c->put_px.end(), src, src + static_cast<size_t>(w) * 4);
    }
    c->cmds.push_back(cmd);
    c->mask_ids.push_back(0);
    c->mask_ids.push_back(0);
    c->queued_bytes += static_cast<size_t>(w) * h * 4;
    return CY_OK;
}

int cy_flush(cy_ctx *c) {
    if (!c) return CY_EINVAL;
    int rc = c->flush();
    if (rc) return rc;
    return c->ok(cudaStreamSynchronize(c->stream)) ? CY_OK : c->status;
}

int cy_get_image(cy_ctx *c, unsigned char *image, int w, int h, int stride, int x, int y) {
    if (!c) return CY_EINVAL;
    if (!image || w <= 0 || h <= 0) return CY_OK;
    int rc = c->flush();
    if (rc) return rc;
    size_t bytes = static_cast<size_t>(w) * h * 4;
    if (!c->get_dev.ensure(bytes)) return c->fail(CY_ENOMEM);
    if (!c->get_host.ensure(bytes)) return c->fail(CY_ENOMEM);
    dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8);
    k_get<<<grd, blk, 0, c->stream>>>(c->bitmap, c->W, c->H, c->get_dev.as<uchar4>(), w, h, x, y);
    if (!c->ok(cudaGetLastError())) return c->status;
    if (!c->ok(cudaMemcpyAsync(c->get_host.p, c->get_dev.p, bytes, cudaMemcpyDeviceToHost, c->stream)))
        return c->status;
    if (!c->ok(cudaStreamSynchronize(c->stream))) return c->status;
    const unsigned char *src = static_cast<const unsigned char *>(c->get_host.p);
    for (int row = 0; row < h; ++row)
        std::memcpy(image + static_cast<ptrdiff_t>(row) * stride, src + static_cast<size_t>(row) * w * 4,
                    static_cast<size_t>(w) * 4);
    return CY_OK;
}

int cy_read_linear(cy_ctx *c, float *out) {
    if (!c || !out) return CY_EINVAL;
    int rc = c->flush();
    if (rc) return rc;
    size_t bytes = static_cast<size_t>(c->W) * c->H * sizeof(float4);
    if (!c->ok(cudaMemcpyAsync(out, c->bitmap, bytes, cudaMemcpyDeviceToHost, c->stream)) ||
        !c->ok(cudaStreamSynchronize(c->stream)))
        return c->status;
    return CY_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ flush
int cy_ctx::scan(const int32_t *in, int32_t *out, int n) {
    // Exclusive scan with recursion over tile sums.
    int tiles = (n + 4095) / 4096;
    if (tiles <= 0) return CY_OK;
    if (tiles == 1) {
        k_scan_tiles<<<1, 1024, 0, stream>>>(in, out, n, nullptr);
        return ok(cudaGetLastError()) ? CY_OK : status;
    }
    dbuf sums, offs;
    if (!sums.ensure(static_cast<size_t>(tiles) * 4) || !offs.ensure(static_cast<size_t>(tiles) * 4))
        return fail(CY_ENOMEM);
    k_scan_tiles<<<tiles, 1024, 0, stream>>>(in, out, n, sums.as<int32_t>());
    int rc = scan(sums.as<int32_t>(), offs.as<int32_t>(), tiles);
    if (rc == CY_OK) {
        k_scan_add<<<(n + 255) / 256, 256, 0, stream>>>(out, n, offs.as<int32_t>());
        if (!ok(cudaGetLastError())) rc = status;
    }
    cudaStreamSynchronize(stream);
    sums.release();
    offs.release();
    return rc;
}

int cy_ctx::clip_mask(const command &c, int mask_in, int mask_out, const scan_job &job, int job_index,
                      const int32_t *rowoff_h) {
    (void)c;
    mask_slot &nm = masks[mask_out];
    const mask_slot *om = mask_in > 0 ? &masks[mask_in] : nullptr;
    int64_t path_runs = rowoff_h[job.row_base + job.rows] - rowoff_h[job.row_base];
    int64_t cap = path_runs + (om ? om->cap : 2 * static_cast<int64_t>(H));
    if (cap > INT32_MAX) return fail(CY_ENOMEM);
    if (!ok(cudaMalloc(&nm.runs, static_cast<size_t>(std::max<int64_t>(cap, 1)) * sizeof(run))) ||
        !ok(cudaMalloc(&nm.sums, static_cast<size_t>(std::max<int64_t>(cap, 1)) * sizeof(float))))
        return status;
    nm.cap = cap;
    // Row capacities: the path's raw runs plus the old mask's runs.
    k_clip_caps<<<(H + 255) / 256, 256, 0, stream>>>(row_off.as<int32_t>() + job.row_base, om ? om->off : nullptr,
                                                      H, nm.len);
    if (!ok(cudaMemsetAsync(nm.len + H, 0, 4, stream))) return status;
    int rc = scan(nm.len, nm.off, H + 1);
    if (rc) return rc;
    if (!ok(cudaMemsetAsync(nm.last_row, 0xff, 4, stream))) return status;
    clip_args a;
    a.p_off = row_off.as<int32_t>();
    a.p_len = row_len.as<int32_t>();
    a.p_runs = runs.as<run>();
    a.p_base = job.row_base;
    a.p_box = boxes.as<cover_box>() + job_index;
    a.o_off = om ? om->off : nullptr;
    a.o_len = om ? om->len : nullptr;
    a.o_runs = om ? om->runs : nullptr;
    a.o_last_row = om ? om->last_row : nullptr;
    a.n_off = nm.off;
    a.n_len = nm.len;
    a.n_runs = nm.runs;
    a.n_last_row = nm.last_row;
    a.W = W;
    a.H = H;
    k_clip_rows<<<(H + 127) / 128, 128, 0, stream>>>(a);
    k_mask_prefix<<<(H + 127) / 128, 128, 0, stream>>>(nm.off, nm.len, nm.runs, nm.sums, H);
    k_mask_fill<<<std::max(1, (H + 7) / 8), 256, 0, stream>>>(nm.off, nm.len, nm.runs, nm.sums, W, H, nm.vis);
    return ok(cudaGetLastError()) ? CY_OK : status;
}

int cy_ctx::flush() {
    if (status) return status;
    if (cmds.empty()) return CY_OK;
    if (!ok(cudaStreamSynchronize(stream))) return status;
    for (auto &m : dead) m.free_all();
    dead.clear();
    // Arena layout: everything queued goes up in one copy.
    size_t o_cmd = 0;
    size_t o_hpts = align256(o_cmd + cmds.size() * sizeof(command));
    size_t o_hprev = align256(o_hpts + host_pts.size() * sizeof(float2));
    size_t o_bez = align256(o_hprev + host_prev.size() * sizeof(int32_t));
    size_t o_items = align256(o_bez + bez_pts.size() * sizeof(float2));
    size_t o_soff = align256(o_items + items.size() * sizeof(flat_item));
    size_t o_scol = align256(o_soff + stop_off.size() * sizeof(float));
    size_t o_tex = align256(o_scol + stop_col.size() * sizeof(float4));
    size_t o_put = align256(o_tex + texels.size() * sizeof(uchar4));
    size_t total = align256(o_put + put_px.size());
    if (!arena.ensure(total) || !staging.ensure(total)) return fail(CY_ENOMEM);
    char *h = static_cast<char *>(staging.p);
    auto put = [&](size_t off, const void *src, size_t n) { if (n) std::memcpy(h + off, src, n); };
    put(o_hpts, host_pts.data(), host_pts.size() * sizeof(float2));
    put(o_hprev, host_prev.data(), host_prev.size() * sizeof(int32_t));
    put(o_bez, bez_pts.data(), bez_pts.size() * sizeof(float2));
    put(o_items, items.data(), items.size() * sizeof(flat_item));
    put(o_soff, stop_off.data(), stop_off.size() * sizeof(float));
    put(o_scol, stop_col.data(), stop_col.size() * sizeof(float4));
    put(o_tex, texels.data(), texels.size() * sizeof(uchar4));
    put(o_put, put_px.data(), put_px.size());
    char *d = static_cast<char *>(arena.p);
    if (total > o_hpts &&
        !ok(cudaMemcpyAsync(d + o_hpts, h + o_hpts, total - o_hpts, cudaMemcpyHostToDevice, stream)))
        return status;
    const float2 *d_hpts = reinterpret_cast<const float2 *>(d + o_hpts);
    const int32_t *d_hprev = reinterpret_cast<const int32_t *>(d + o_hprev);
    const float2 *d_bez = reinterpret_cast<const float2 *>(d + o_bez);
    const flat_item *d_items = reinterpret_cast<const flat_item *>(d + o_items);
    paint_src src;
    src.stop_off = reinterpret_cast<const float *>(d + o_soff);
    src.stop_col = reinterpret_cast<const float4 *>(d + o_scol);
    src.texels = nullptr;
    if (!texels.empty()) {
        if (!pat_f4.ensure(texels.size() * sizeof(float4))) return fail(CY_ENOMEM);
        int n = static_cast<int>(texels.size());
        k_pattern_prep<<<(n + 255) / 256, 256, 0, stream>>>(reinterpret_cast<const uchar4 *>(d + o_tex),
                                                            pat_f4.as<float4>(), n, lut);
        src.texels = pat_f4.as<float4>();
    }
    // Flatten every Bezier path of the flush (path_to_lines, hpp:1495-1524).
    int n_items = static_cast<int>(items.size());
    const int32_t *offs_h = nullptr;
    if (n_items > 0) {
        if (!item_cnt.ensure(static_cast<size_t>(n_items + 1) * 4) ||
            !item_off.ensure(static_cast<size_t>(n_items + 1) * 4) ||
            !offs_host.ensure(static_cast<size_t>(n_items + 1) * 4))
            return fail(CY_ENOMEM);
        k_flat_count<<<(n_items + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items, item_cnt.as<int32_t>());
        if (!ok(cudaMemsetAsync(item_cnt.as<int32_t>() + n_items, 0, 4, stream))) return status;
        int rc = scan(item_cnt.as<int32_t>(), item_off.as<int32_t>(), n_items + 1);
        if (rc) return rc;
        if (!ok(cudaMemcpyAsync(offs_host.p, item_off.p, static_cast<size_t>(n_items + 1) * 4,
                                cudaMemcpyDeviceToHost, stream)) ||
            !ok(cudaStreamSynchronize(stream)))
            return status;
        offs_h = static_cast<const int32_t *>(offs_host.p);
        int64_t nflat = offs_h[n_items];
        if (nflat < 0 || nflat > (static_cast<int64_t>(1) << 30)) return fail(CY_ENOMEM);
        if (!flat_pts.ensure(static_cast<size_t>(nflat + 1) * sizeof(float2)) ||
            !flat_prev.ensure(static_cast<size_t>(nflat + 1) * 4))
            return fail(CY_ENOMEM);
        k_flat_emit<<<(n_items + 255) / 256, 256, 0, stream>>>(d_bez, d_items, n_items, item_off.as<int32_t>(),
                                                               flat_pts.as<float2>(), flat_prev.as<int32_t>(),
                                                               nflat);
        if (!ok(cudaGetLastError())) return status;
    }
    for (command &c : cmds) {
        if (c.kind == CMD_PUT) continue;
        if (c.geom == 0) {
            c.line_first = c.first;
            c.line_count = c.count;
        } else if (c.count == 0 || !offs_h) {
            c.line_first = 0;
            c.line_count = 0;
        } else {
            c.line_first = offs_h[c.first];
            c.line_count = offs_h[c.first + c.count] - c.line_first;
        }
    }
    std::memcpy(h + o_cmd, cmds.data(), cmds.size() * sizeof(command));
    if (!ok(cudaMemcpyAsync(d + o_cmd, h + o_cmd, cmds.size() * sizeof(command), cudaMemcpyHostToDevice, stream)))
        return status;
    const command *d_cmds = reinterpret_cast<const command *>(d + o_cmd);
    // Scan-conversion jobs: the shadow pass (padded canvas) and the main pass
    // of each draw, and the path of each clip.
    std::vector<scan_job> jobs;
    std::vector<int> main_job(cmds.size(), -1), shadow_job(cmds.size(), -1);
    int64_t total_rows = 0, total_segs = 0;
    auto add_job = [&](const command &c, int rows_n, int cols_n, float wd, float ht, float ox, float oy) {
        scan_job j;
        std::memset(&j, 0, sizeof(j));
        j.geom = c.geom;
        j.line_first = c.line_first;
        j.seg_first = static_cast<int32_t>(total_segs);
        j.seg_count = c.line_count;
        j.row_base = static_cast<int32_t>(total_rows);
        j.rows = rows_n;
        j.cols = cols_n;
        j.width = wd;
        j.height = ht;
        j.offx = ox;
        j.offy = oy;
        total_rows += rows_n;
        total_segs += c.line_count;
        jobs.push_back(j);
        return static_cast<int>(jobs.size()) - 1;
    };
    for (size_t i = 0; i < cmds.size(); ++i) {
        const command &c = cmds[i];
        if (c.kind == CMD_PUT) continue;
        if (c.kind == CMD_FILL && c.shadow) {
            int b = c.sh_border;
            int ew = W + 2 * b, eh = H + 2 * b;
            shadow_job[i] = add_job(c, eh, ew + 2, static_cast<float>(ew), static_cast<float>(eh), c.sh_offx,
                                    c.sh_offy);
        }
        main_job[i] = add_job(c, H, W + 2, static_cast<float>(W), static_cast<float>(H), 0.0f, 0.0f);
    }
    if (total_rows > INT32_MAX / 2 || total_segs > INT32_MAX / 2) return fail(CY_ENOMEM);
    int n_jobs = static_cast<int>(jobs.size());
    const int32_t *rowoff_h = nullptr;
    job_tables t;
    std::memset(&t, 0, sizeof(t));
    if (n_jobs > 0) {
        size_t nr = static_cast<size_t>(total_rows);
        if (!jobs_dev.ensure(jobs.size() * sizeof(scan_job)) || !row_cnt.ensure((nr + 1) * 4) ||
            !row_off.ensure((nr + 2) * 4) || !row_cur.ensure((nr + 1) * 4) || !row_len.ensure((nr + 1) * 4) ||
            !boxes.ensure(jobs.size() * sizeof(cover_box)) || !rowoff_host.ensure((nr + 1) * 4))
            return fail(CY_ENOMEM);
        if (!ok(cudaMemcpyAsync(jobs_dev.p, jobs.data(), jobs.size() * sizeof(scan_job), cudaMemcpyHostToDevice,
                                stream)) ||
            !ok(cudaMemsetAsync(row_cnt.p, 0, (nr + 1) * 4, stream)) ||
            !ok(cudaMemsetAsync(row_cur.p, 0, (nr + 1) * 4, stream)))
            return status;
        k_box_init<<<(n_jobs + 255) / 256, 256, 0, stream>>>(boxes.as<cover_box>(), n_jobs);
        t.jobs = jobs_dev.as<scan_job>();
        t.n_jobs = n_jobs;
        t.pts[0] = d_hpts;
        t.prev[0] = d_hprev;
        t.pts[1] = flat_pts.p ? flat_pts.as<float2>() : d_hpts;
        t.prev[1] = flat_prev.p ? flat_prev.as<int32_t>() : d_hprev;
        t.boxes = boxes.as<cover_box>();
        t.row_cnt = row_cnt.as<int32_t>();
        t.row_cur = row_cur.as<int32_t>();
        int segs = static_cast<int>(total_segs);
        int grid = std::max(1, std::min((segs + 7) / 8, 152 * 32));
        if (segs > 0) k_runs<false><<<grid, 256, 0, stream>>>(t, segs);
        int rc = scan(row_cnt.as<int32_t>(), row_off.as<int32_t>(), static_cast<int>(nr) + 1);
        if (rc) return rc;
        if (!ok(cudaMemcpyAsync(rowoff_host.p, row_off.p, (nr + 1) * 4, cudaMemcpyDeviceToHost, stream)) ||
            !ok(cudaStreamSynchronize(stream)))
            return status;
        rowoff_h = static_cast<const int32_t *>(rowoff_host.p);
        int64_t nruns = rowoff_h[nr];
        if (nruns < 0) return fail(CY_ENOMEM);
        if (!runs.ensure(static_cast<size_t>(nruns + 1) * sizeof(run)) ||
            !sums.ensure(static_cast<size_t>(nruns + 1) * sizeof(float)))
            return fail(CY_ENOMEM);
        t.row_off = row_off.as<int32_t>();
        t.runs = runs.as<run>();
        if (segs > 0) k_runs<true><<<grid, 256, 0, stream>>>(t, segs);
        k_rows<<<static_cast<int>((nr + 127) / 128), 128, 0, stream>>>(
            row_off.as<int32_t>(), row_cnt.as<int32_t>(), row_cur.as<int32_t>(), row_len.as<int32_t>(),
            runs.as<run>(), sums.as<float>(), static_cast<int>(nr));
        if (!ok(cudaGetLastError())) return status;
    }
    row_view rv;
    rv.row_off = row_off.as<int32_t>();
    rv.row_len = row_len.as<int32_t>();
    rv.runs = runs.as<run>();
    rv.sums = sums.as<float>();
    const uint8_t *d_put = reinterpret_cast<const uint8_t *>(d + o_put);
    for (size_t i = 0; i < cmds.size(); ++i) {
        const command &c = cmds[i];
        int in_id = mask_ids[2 * i], out_id = mask_ids[2 * i + 1];
        if (c.kind == CMD_PUT) {
            dim3 blk(32, 8), grd((c.put_w + 31) / 32, (c.put_h + 7) / 8);
            k_put<<<grd, blk, 0, stream>>>(d_cmds + i, d_put, bitmap, W, H, lut);
            if (!ok(cudaGetLastError())) return status;
            continue;
        }
        if (c.kind == CMD_CLIP) {
            int rc = clip_mask(c, in_id, out_id, jobs[main_job[i]], main_job[i], rowoff_h);
            if (rc) return rc;
            continue;
        }
        const float *vis = in_id > 0 ? masks[in_id].vis : nullptr;
        if (c.shadow) {
            const scan_job &sj = jobs[shadow_job[i]];
            int b = c.sh_border;
            int ew = W + 2 * b, eh = H + 2 * b;
            size_t area = static_cast<size_t>(ew + 1) * eh;
            if (!sh_a.ensure(area * 4) || !sh_b.ensure(area * 4) || !sh_rect.ensure(sizeof(shadow_rect)))
                return fail(CY_ENOMEM);
            shadow_rect *rect = sh_rect.as<shadow_rect>();
            k_shadow_rect<<<1, 1, 0, stream>>>(boxes.as<cover_box>() + shadow_job[i], W, H, b, rect);
            k_shadow_raster<<<std::max(1, (eh + 7) / 8), 256, 0, stream>>>(d_cmds + i, src, rv, sj.row_base, rect,
                                                                           sh_a.as<float>());
            k_blur_rows<<<(eh + 127) / 128, 128, 0, stream>>>(sh_a.as<float>(), sh_b.as<float>(), rect,
                                                               c.sh_radius, c.sh_w1, c.sh_w2);
            k_blur_cols<<<(ew + 1 + 127) / 128, 128, 0, stream>>>(sh_a.as<float>(), sh_b.as<float>(), rect,
                                                                   c.sh_radius, c.sh_w1, c.sh_w2);
            dim3 blk(32, 8), cgrd((W + 31) / 32, (H + 7) / 8);
            k_shadow_composite<<<cgrd, blk, 0, stream>>>(d_cmds + i, bitmap, W, H, vis, rect, sh_a.as<float>());
            if (!ok(cudaGetLastError())) return status;
        }
        bool clearing = !(c.op & 8);
        int y0 = clearing ? 0 : std::max(0, std::min(H, c.gy0));
        int y1 = clearing ? H : std::max(0, std::min(H, c.gy1 + 1));
        if (y1 > y0) {
            paint_args pa;
            pa.cmd = d_cmds + i;
            pa.bitmap = bitmap;
            pa.W = W;
            pa.H = H;
            pa.rv = rv;
            pa.row_base = jobs[main_job[i]].row_base;
            pa.vis = vis;
            pa.y_begin = y0;
            pa.y_end = y1;
            pa.src = src;
            k_paint<<<std::max(1, (y1 - y0 + 7) / 8), 256, 0, stream>>>(pa);
            if (!ok(cudaGetLastError())) return status;
        }
    }
    // Release the references the queued commands held on clip masks.
    for (size_t i = 0; i < cmds.size(); ++i) {
        int in = mask_ids[2 * i], out = mask_ids[2 * i + 1];
        if (in > 0) cy_mask_release(this, in);
        if (out > 0) cy_mask_release(this, out);
    }
    cmds.clear();
    host_pts.clear();
    host_prev.clear();
    bez_pts.clear();
    items.clear();
    stop_off.clear();
    stop_col.clear();
    texels.clear();
    put_px.clear();
    mask_ids.clear();
    queued_bytes = 0;
    queued_rows = 0;
    return CY_OK;
}
