// capi.cpp -- flat C binding of canvas_ity::canvas and the call-list replay
// entry point (include/canvas_ity_c.h).
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "../../include/canvas_ity.hpp"
#include "../../include/canvas_ity_c.h"
#include "../../include/cy_replay.hpp"
#include "../../include/cy_batch.h"

using canvas_ity::canvas;

struct cy_canvas {
    std::unique_ptr<canvas> owned;
    canvas &get() { return *owned; }
};

namespace {
struct traits {
    typedef canvas canvas_type;
    typedef canvas_ity::brush_type brush_type;
    typedef canvas_ity::composite_operation composite_operation;
    typedef canvas_ity::cap_style cap_style;
    typedef canvas_ity::join_style join_style;
    typedef canvas_ity::repetition_style repetition_style;
    typedef canvas_ity::align_style align_style;
    typedef canvas_ity::baseline_style baseline_style;
    static std::unique_ptr<canvas> make(int w, int h) { return std::unique_ptr<canvas>(new canvas(w, h)); }
    static bool set_fill_rule(canvas &c, int rule) {
        if (rule != 0 && rule != 1) return false;
        c.set_fill_rule(rule ? canvas_ity::even_odd : canvas_ity::nonzero);
        return true;
    }
};
inline canvas_ity::brush_type bt(int t) { return static_cast<canvas_ity::brush_type>(t); }
}  // namespace

extern "C" {

cy_canvas *cy_canvas_new(int w, int h) {
    if (w < 1 || h < 1 || w > 32768 || h > 32768) return nullptr;
    cy_canvas *c = new (std::nothrow) cy_canvas();
    if (!c) return nullptr;
    c->owned.reset(new (std::nothrow) canvas(w, h));
    if (!c->owned) { delete c; return nullptr; }
    return c;
}
void cy_canvas_delete(cy_canvas *c) { delete c; }
int cy_canvas_status(const cy_canvas *c) { return c ? const_cast<cy_canvas *>(c)->get().gpu_status() : -1; }
void cy_canvas_scale(cy_canvas *c, float x, float y) { c->get().scale(x, y); }
void cy_canvas_rotate(cy_canvas *c, float a) { c->get().rotate(a); }
void cy_canvas_translate(cy_canvas *c, float x, float y) { c->get().translate(x, y); }
void cy_canvas_transform(cy_canvas *c, float a, float b, float cc, float d, float e, float f) {
    c->get().transform(a, b, cc, d, e, f);
}
void cy_canvas_set_transform(cy_canvas *c, float a, float b, float cc, float d, float e, float f) {
    c->get().set_transform(a, b, cc, d, e, f);
}
void cy_canvas_set_global_alpha(cy_canvas *c, float a) { c->get().set_global_alpha(a); }
void cy_canvas_set_global_composite_operation(cy_canvas *c, int op) {
    c->get().global_composite_operation = static_cast<canvas_ity::composite_operation>(op);
}
void cy_canvas_set_shadow_color(cy_canvas *c, float r, float g, float b, float a) {
    c->get().set_shadow_color(r, g, b, a);
}
void cy_canvas_set_shadow_offset_x(cy_canvas *c, float v) { c->get().shadow_offset_x = v; }
void cy_canvas_set_shadow_offset_y(cy_canvas *c, float v) { c->get().shadow_offset_y = v; }
void cy_canvas_set_shadow_blur(cy_canvas *c, float v) { c->get().set_shadow_blur(v); }
void cy_canvas_set_line_width(cy_canvas *c, float v) { c->get().set_line_width(v); }
void cy_canvas_set_line_cap(cy_canvas *c, int v) { c->get().line_cap = static_cast<canvas_ity::cap_style>(v); }
void cy_canvas_set_line_join(cy_canvas *c, int v) { c->get().line_join = static_cast<canvas_ity::join_style>(v); }
void cy_canvas_set_miter_limit(cy_canvas *c, float v) { c->get().set_miter_limit(v); }
void cy_canvas_set_line_dash_offset(cy_canvas *c, float v) { c->get().line_dash_offset = v; }
void cy_canvas_set_line_dash(cy_canvas *c, const float *s, int n) { c->get().set_line_dash(s, n); }
void cy_canvas_set_color(cy_canvas *c, int t, float r, float g, float b, float a) {
    c->get().set_color(bt(t), r, g, b, a);
}
void cy_canvas_set_linear_gradient(cy_canvas *c, int t, float x0, float y0, float x1, float y1) {
    c->get().set_linear_gradient(bt(t), x0, y0, x1, y1);
}
void cy_canvas_set_radial_gradient(cy_canvas *c, int t, float x0, float y0, float r0, float x1, float y1,
                                   float r1) {
    c->get().set_radial_gradient(bt(t), x0, y0, r0, x1, y1, r1);
}
void cy_canvas_add_color_stop(cy_canvas *c, int t, float o, float r, float g, float b, float a) {
    c->get().add_color_stop(bt(t), o, r, g, b, a);
}
void cy_canvas_set_pattern(cy_canvas *c, int t, const unsigned char *img, int w, int h, int stride, int rep) {
    c->get().set_pattern(bt(t), img, w, h, stride, static_cast<canvas_ity::repetition_style>(rep));
}
void cy_canvas_begin_path(cy_canvas *c) { c->get().begin_path(); }
void cy_canvas_move_to(cy_canvas *c, float x, float y) { c->get().move_to(x, y); }
void cy_canvas_close_path(cy_canvas *c) { c->get().close_path(); }
void cy_canvas_line_to(cy_canvas *c, float x, float y) { c->get().line_to(x, y); }
void cy_canvas_quadratic_curve_to(cy_canvas *c, float cx, float cy, float x, float y) {
    c->get().quadratic_curve_to(cx, cy, x, y);
}
void cy_canvas_bezier_curve_to(cy_canvas *c, float a, float b, float cc, float d, float x, float y) {
    c->get().bezier_curve_to(a, b, cc, d, x, y);
}
void cy_canvas_arc_to(cy_canvas *c, float vx, float vy, float x, float y, float r) { c->get().arc_to(vx, vy, x, y, r); }
void cy_canvas_arc(cy_canvas *c, float x, float y, float r, float a0, float a1, int ccw) {
    c->get().arc(x, y, r, a0, a1, ccw != 0);
}
void cy_canvas_rectangle(cy_canvas *c, float x, float y, float w, float h) { c->get().rectangle(x, y, w, h); }
void cy_canvas_fill(cy_canvas *c) { c->get().fill(); }
void cy_canvas_stroke(cy_canvas *c) { c->get().stroke(); }
void cy_canvas_clip(cy_canvas *c) { c->get().clip(); }
int cy_canvas_is_point_in_path(cy_canvas *c, float x, float y) { return c->get().is_point_in_path(x, y) ? 1 : 0; }
void cy_canvas_clear_rectangle(cy_canvas *c, float x, float y, float w, float h) { c->get().clear_rectangle(x, y, w, h); }
void cy_canvas_fill_rectangle(cy_canvas *c, float x, float y, float w, float h) { c->get().fill_rectangle(x, y, w, h); }
void cy_canvas_stroke_rectangle(cy_canvas *c, float x, float y, float w, float h) {
    c->get().stroke_rectangle(x, y, w, h);
}
void cy_canvas_set_text_align(cy_canvas *c, int v) { c->get().text_align = static_cast<canvas_ity::align_style>(v); }
void cy_canvas_set_text_baseline(cy_canvas *c, int v) {
    c->get().text_baseline = static_cast<canvas_ity::baseline_style>(v);
}
int cy_canvas_set_font(cy_canvas *c, const unsigned char *f, int n, float s) { return c->get().set_font(f, n, s) ? 1 : 0; }
void cy_canvas_fill_text(cy_canvas *c, const char *t, float x, float y, float m) { c->get().fill_text(t, x, y, m); }
void cy_canvas_stroke_text(cy_canvas *c, const char *t, float x, float y, float m) { c->get().stroke_text(t, x, y, m); }
float cy_canvas_measure_text(cy_canvas *c, const char *t) { return c->get().measure_text(t); }
void cy_canvas_draw_image(cy_canvas *c, const unsigned char *img, int w, int h, int stride, float x, float y,
                          float tw, float th) {
    c->get().draw_image(img, w, h, stride, x, y, tw, th);
}
void cy_canvas_get_image_data(cy_canvas *c, unsigned char *img, int w, int h, int stride, int x, int y) {
    c->get().get_image_data(img, w, h, stride, x, y);
}
void cy_canvas_put_image_data(cy_canvas *c, const unsigned char *img, int w, int h, int stride, int x, int y) {
    c->get().put_image_data(img, w, h, stride, x, y);
}
void cy_canvas_save(cy_canvas *c) { c->get().save(); }
void cy_canvas_restore(cy_canvas *c) { c->get().restore(); }
void cy_canvas_set_fill_rule(cy_canvas *c, int rule) {
    c->get().set_fill_rule(rule == 1 ? canvas_ity::even_odd : canvas_ity::nonzero);
}

int cy_canvas_points_in_path(cy_canvas *c, const float *xy, int n, unsigned char *inside) {
    if (!c) return CY_EINVAL;
    return c->get().points_in_path(xy, n, inside);
}

int cy_take_thread_status(void);
void cy_ctx_set_transient(cy_ctx *ctx, int transient);

int cy_replay(const void *trace, size_t trace_len, void *images, size_t images_cap, size_t *images_len,
              float *results, int results_cap, int *results_len) {
    cy_take_thread_status();
    int rc = cy_trace::replay_to_buffers<traits>(trace, trace_len, images, images_cap, images_len, results,
                                                 results_cap, results_len);
    int gpu = cy_take_thread_status();
    return gpu ? gpu : rc;
}

int cy_replay_linear(const void *trace, size_t trace_len, float *out, size_t out_floats, int *width,
                     int *height) {
    cy_take_thread_status();
    cy_trace::output sink;
    std::unique_ptr<canvas> keep;
    int rc = cy_trace::replay<traits>(static_cast<const uint8_t *>(trace), trace_len, sink, &keep);
    if (rc == 0 && !keep) rc = -1;
    if (rc == 0) {
        int w = 0, h = 0;
        const uint8_t *t = static_cast<const uint8_t *>(trace);
        std::memcpy(&w, t + 12, 4);
        std::memcpy(&h, t + 16, 4);
        if (width) *width = w;
        if (height) *height = h;
        if (static_cast<size_t>(w) * h * 4 > out_floats) rc = -2;
        else rc = keep->read_linear(out);
    }
    int gpu = cy_take_thread_status();
    return gpu ? gpu : rc;
}

cy_canvas *cy_canvas_from_trace(const void *trace, size_t trace_len, int *status) {
    // Replay with reads deferred: drawing is recorded, nothing runs yet.
    cy_take_thread_status();
    cy_set_deferred(1);
    cy_trace::output sink;
    std::unique_ptr<canvas> keep;
    int rc = cy_trace::replay<traits>(static_cast<const uint8_t *>(trace), trace_len, sink, &keep);
    cy_set_deferred(0);
    int gpu = cy_take_thread_status();
    if (status) *status = gpu ? gpu : rc;
    if (rc != 0 || gpu != 0 || !keep) return nullptr;
    cy_canvas *c = new (std::nothrow) cy_canvas();
    if (!c) return nullptr;
    c->owned.reset(keep.release());
    return c;
}

void *cy_canvas_ctx(cy_canvas *c) { return c ? c->get().gpu_context() : nullptr; }

int cy_canvases_from_traces(const void *const *traces, const size_t *lens, int n, int engine, int threads,
                            cy_canvas **out) {
    if (n < 0 || (n > 0 && (!traces || !lens || !out))) return CY_EINVAL;
    for (int i = 0; i < n; ++i) out[i] = nullptr;
    if (n == 0) return CY_OK;
    if (threads <= 0) threads = static_cast<int>(std::thread::hardware_concurrency());
    if (threads < 1) threads = 1;
    if (threads > n) threads = n;
    if (threads > 256) threads = 256;
    std::atomic<int> next(0), failure(0);
    // Each canvas is an independent instance (as in the reference, separate
    // canvases may be used from different threads), so the host halves of the
    // replays run side by side; their device contexts only queue work.
    auto work = [&]() {
        cy_set_engine(engine);
        for (;;) {
            int i = next.fetch_add(1);
            if (i >= n) break;
            int st = 0;
            out[i] = cy_canvas_from_trace(traces[i], lens[i], &st);
            if (!out[i]) {
                int none = 0;
                failure.compare_exchange_strong(none, st ? st : CY_EINVAL);
            }
        }
    };
    std::vector<std::thread> pool;
    try {
        for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    } catch (...) {
        // fewer threads than asked: the ones started and this one finish the work
    }
    work();
    for (std::thread &t : pool) t.join();
    int rc = failure.load();
    if (rc) {
        for (int i = 0; i < n; ++i) {
            delete out[i];
            out[i] = nullptr;
        }
    }
    return rc;
}

int cy_render_traces(const void *const *traces, const size_t *lens, int n, int engine, long long frame_pixels,
                     unsigned char *out, const size_t *offsets, long long *stats) {
    if (n < 0 || (n > 0 && (!traces || !lens || !offsets || (!out && offsets[n] > 0)))) return CY_EINVAL;
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    if (n == 0) return CY_OK;
    // 32 Mpx frames: on 4096 workload canvases end to end, 8% faster than 64 Mpx and 10% faster than 128 Mpx
    if (frame_pixels <= 0) frame_pixels = 32LL << 20;
    // frames: consecutive call lists up to frame_pixels canvas pixels
    std::vector<int> starts;
    long long acc = 0;
    for (int i = 0; i < n; ++i) {
        int w = 0, h = 0;
        if (lens[i] >= 20) {
            std::memcpy(&w, static_cast<const unsigned char *>(traces[i]) + 12, 4);
            std::memcpy(&h, static_cast<const unsigned char *>(traces[i]) + 16, 4);
        }
        long long px = static_cast<long long>(w > 0 ? w : 0) * (h > 0 ? h : 0);
        if (starts.empty() || (acc > 0 && acc + px > frame_pixels)) {
            starts.push_back(i);
            acc = 0;
        }
        acc += px;
    }
    starts.push_back(n);
    struct job { cy_frame *f = nullptr; std::vector<cy_canvas *> cv; int first = 0; };
    // CY_DEBUG: per-frame host timings on stderr
    const bool trace_timing = std::getenv("CY_DEBUG") != nullptr;
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const int nf = static_cast<int>(starts.size()) - 1;
    std::vector<job> slots(static_cast<size_t>(nf));
    std::vector<char> ready(static_cast<size_t>(nf), 0);
    std::mutex m;
    std::condition_variable cv_ready, cv_space;
    int taken = 0, inflight = 0;
    bool producers_done = false;
    const int max_inflight = 3;
    std::atomic<int> failure(0);
    std::atomic<long long> up(0), down(0);
    auto fail = [&](int rc) { int none = 0; failure.compare_exchange_strong(none, rc); };
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return CY_ENODEV;
    }
    // Producers (two): replay a frame's call lists and create the frame,
    // which uploads it and queues its first run.  While one waits for its
    // frame's size read-backs, the other replays the next frame.
    auto produce = [&]() {
        cudaSetDevice(dev);
        for (;;) {
            int fi;
            {
                std::unique_lock<std::mutex> hold(m);
                cv_space.wait(hold, [&] { return inflight < max_inflight || failure.load() != 0; });
                if (failure.load() != 0 || taken >= nf) return;
                fi = taken++;
                ++inflight;
            }
            job j;
            j.first = starts[fi];
            const int k = starts[fi + 1] - j.first;
            j.cv.assign(static_cast<size_t>(k), nullptr);
            auto t0 = std::chrono::steady_clock::now();
            int rc = cy_canvases_from_traces(traces + j.first, lens + j.first, k, engine, 0, j.cv.data());
            auto t1 = std::chrono::steady_clock::now();
            if (rc == CY_OK) {
                std::vector<cy_ctx *> ctx(static_cast<size_t>(k));
                for (int i = 0; i < k; ++i) {
                    ctx[i] = static_cast<cy_ctx *>(cy_canvas_ctx(j.cv[i]));
                    cy_ctx_set_transient(ctx[i], 1);   // deleted once its reads are out
                }
                rc = cy_frame_create(ctx.data(), k, engine, &j.f);
                // A canvas wider than a tile-engine strip renders on the plain engine.
                if (rc == CY_EINVAL && engine == 0) rc = cy_frame_create(ctx.data(), k, 1, &j.f);
                if (trace_timing)
                    std::fprintf(stderr, "render_traces frame %d: %d canvases, replay %.1f ms, create %.1f ms\n", fi, k,
                                 ms(t0, t1), ms(t1, std::chrono::steady_clock::now()));
                if (rc == CY_OK) {
                    long long st[10] = {};
                    if (cy_frame_stats(j.f, st, 10) >= 10) up += st[9];
                }
            }
            if (rc) fail(rc);
            {
                std::lock_guard<std::mutex> hold(m);
                slots[fi] = std::move(j);
                ready[fi] = 1;
            }
            cv_ready.notify_all();
        }
    };
    // Finisher: frames in order; waits for each, copies its reads out and
    // frees it.
    std::thread finisher([&]() {
        cudaSetDevice(dev);
        for (int fi = 0; fi < nf; ++fi) {
            job j;
            {
                std::unique_lock<std::mutex> hold(m);
                cv_ready.wait(hold, [&] { return ready[fi] || (producers_done && fi >= taken); });
                if (!ready[fi]) return;
                j = std::move(slots[fi]);
            }
            const int k = static_cast<int>(j.cv.size());
            if (j.f && failure.load() == 0) {
                std::vector<size_t> offs(static_cast<size_t>(k) + 1);
                const unsigned char *data = nullptr;
                auto t0 = std::chrono::steady_clock::now();
                int rc = cy_frame_finish_views(j.f, &data, offs.data());
                auto t1 = std::chrono::steady_clock::now();
                if (rc) fail(rc);
                for (int i = 0; rc == 0 && i < k; ++i)
                    if (offs[i + 1] - offs[i] != offsets[j.first + i + 1] - offsets[j.first + i]) {
                        fail(CY_EINVAL);
                        rc = CY_EINVAL;
                    }
                if (rc == 0) {
                    down += static_cast<long long>(offs[k]);
                    // copy out on a few threads
                    const int t = std::max(1, std::min(8, k));
                    std::vector<std::thread> pool;
                    for (int a = 0; a < t; ++a)
                        pool.emplace_back([&, a]() {
                            for (int i = a; i < k; i += t) {
                                size_t len = offs[i + 1] - offs[i];
                                if (len) std::memcpy(out + offsets[j.first + i], data + offs[i], len);
                            }
                        });
                    for (std::thread &th : pool) th.join();
                    if (trace_timing)
                        std::fprintf(stderr, "render_traces frame %d: finish %.1f ms, copy out %.1f ms\n", fi, ms(t0, t1),
                                     ms(t1, std::chrono::steady_clock::now()));
                }
            }
            if (j.f) cy_frame_destroy(j.f);
            for (cy_canvas *c : j.cv) delete c;
            {
                std::lock_guard<std::mutex> hold(m);
                --inflight;
            }
            cv_space.notify_all();
        }
    });
    std::thread second(produce);
    produce();
    second.join();
    {
        std::lock_guard<std::mutex> hold(m);
        producers_done = true;
    }
    cv_ready.notify_all();
    finisher.join();
    if (stats) {
        stats[0] = nf;
        stats[1] = up.load();
        stats[2] = down.load();
    }
    return failure.load();
}

}  // extern "C"
