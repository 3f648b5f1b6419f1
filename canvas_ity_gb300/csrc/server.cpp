// server.cpp -- continuous-batching render server over the frame engine.
//
// Requests are recorded call lists (cy_trace.h).  Worker threads, one CUDA
// stream each, repeatedly take every waiting request that fits the device
// memory budget (oldest first), render them together as one frame and hand
// back each request's get_image_data bytes.  A request that arrives while
// other frames are on the GPU joins the next frame a worker forms, as soon as
// budget frees up, so frames of different workers overlap on the device and
// the host halves (call-list replay, staging) overlap the device halves.
// Each canvas and its clip masks stay on the device while its frame runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/canvas_ity_c.h"
#include "../../include/cy_batch.h"
#include "../../include/cy_serve.h"

extern "C" void cy_ctx_set_transient(cy_ctx *ctx, int transient);   // engine.cu

namespace {

double now_s() {
    using clk = std::chrono::steady_clock;
    return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

struct request {
    uint64_t id = 0;
    std::vector<uint8_t> trace;
    int64_t cost = 0;       // admission estimate, bytes of device memory
    int64_t pixels = 0;
    double t_arrive = 0.0;
};

struct finished {
    uint64_t id = 0;
    int status = 0;
    std::vector<uint8_t> images;
    double t_arrive = 0.0, t_start = 0.0, t_done = 0.0;
    int64_t pixels = 0;
    int batch = 0;
};

}  // namespace

struct cy_server {
    int device = 0;
    int engine = 0;
    int host_threads = 0;
    int max_batch = 256;
    int64_t max_pixels = 16 << 20;   // pixels per frame, so several workers share a burst
    int64_t budget = 0;
    int64_t in_use = 0;     // admitted and not yet finished
    uint64_t next_id = 1;
    bool stopping = false;
    std::mutex m;
    std::condition_variable work_cv, done_cv;
    std::deque<request> waiting;
    std::deque<finished> done;
    std::vector<std::thread> workers;
    // statistics
    int64_t frames = 0, requests_done = 0, pixels_done = 0, max_in_use = 0, max_batch_seen = 0;

    void worker();
};

namespace {

// Device memory a request may need while its frame runs: the float canvas
// and clip visibility (16 + 4 B/px), its runs and their sums (about 6 runs of
// 12 B per pixel on the mixed scenes, doubled for margin), and its uploaded
// geometry (well under 16x the call-list size).
int64_t estimate_cost(const uint8_t *trace, size_t len, int64_t *pixels) {
    int32_t w = 0, h = 0;
    if (len >= 20) {
        std::memcpy(&w, trace + 12, 4);
        std::memcpy(&h, trace + 16, 4);
    }
    int64_t px = static_cast<int64_t>(std::max(w, 0)) * std::max(h, 0);
    *pixels = px;
    return px * (16 + 4 + 2 * 72) + static_cast<int64_t>(len) * 16 + (1 << 20);
}

}  // namespace

void cy_server::worker() {
    cudaSetDevice(device);
    cy_set_engine(engine);
    for (;;) {
        std::vector<request> batch;
        int64_t batch_cost = 0, batch_px = 0;
        {
            std::unique_lock<std::mutex> lk(m);
            for (;;) {
                if (stopping && waiting.empty()) return;
                // Admit the oldest waiting requests that fit the budget; a
                // request larger than the whole budget runs alone.
                while (!waiting.empty() && static_cast<int>(batch.size()) < max_batch) {
                    request &r = waiting.front();
                    bool fits = in_use + batch_cost + r.cost <= budget;
                    bool alone = batch.empty() && in_use == 0;
                    if (!fits && !alone) break;
                    if (!batch.empty() && batch_px + r.pixels > max_pixels) break;
                    batch_cost += r.cost;
                    batch_px += r.pixels;
                    batch.push_back(std::move(r));
                    waiting.pop_front();
                }
                if (!batch.empty()) break;
                work_cv.wait(lk);
            }
            in_use += batch_cost;
            max_in_use = std::max(max_in_use, in_use);
            max_batch_seen = std::max<int64_t>(max_batch_seen, static_cast<int64_t>(batch.size()));
        }
        double t_start = now_s();
        int n = static_cast<int>(batch.size());
        std::vector<const void *> ptrs(n);
        std::vector<size_t> lens(n);
        for (int i = 0; i < n; ++i) {
            ptrs[i] = batch[i].trace.data();
            lens[i] = batch[i].trace.size();
        }
        std::vector<cy_canvas *> canvases(n, nullptr);
        std::vector<finished> out(n);
        int rc = cy_canvases_from_traces(ptrs.data(), lens.data(), n, engine, host_threads, canvases.data());
        cy_frame *fr = nullptr;
        if (rc == 0) {
            std::vector<cy_ctx *> ctxs(n);
            for (int i = 0; i < n; ++i) {
                ctxs[i] = static_cast<cy_ctx *>(cy_canvas_ctx(canvases[i]));
                cy_ctx_set_transient(ctxs[i], 1);   // deleted once its reads are out
            }
            rc = cy_frame_create(ctxs.data(), n, engine, &fr);
            // A canvas wider than a tile-engine strip renders on the plain engine.
            if (rc == CY_EINVAL && engine == 0) rc = cy_frame_create(ctxs.data(), n, 1, &fr);
            if (rc == 0) rc = cy_frame_finish(fr);
            for (int i = 0; i < n && rc == 0; ++i) {
                size_t len = 0;
                cy_ctx_take_reads(ctxs[i], nullptr, 0, &len);
                out[i].images.resize(len);
                int r2 = cy_ctx_take_reads(ctxs[i], out[i].images.data(), len, &len);
                out[i].status = r2;
            }
        }
        if (fr) cy_frame_destroy(fr);
        for (cy_canvas *c : canvases)
            if (c) cy_canvas_delete(c);
        double t_done = now_s();
        {
            std::lock_guard<std::mutex> lk(m);
            in_use -= batch_cost;
            ++frames;
            for (int i = 0; i < n; ++i) {
                finished &f = out[i];
                f.id = batch[i].id;
                if (rc != 0) f.status = rc;
                f.t_arrive = batch[i].t_arrive;
                f.t_start = t_start;
                f.t_done = t_done;
                f.pixels = batch[i].pixels;
                f.batch = n;
                ++requests_done;
                pixels_done += batch[i].pixels;
                done.push_back(std::move(f));
            }
        }
        done_cv.notify_all();
        work_cv.notify_all();   // budget freed: others may admit now
    }
}

extern "C" {

int cy_server_create(long long budget_bytes, int workers, int host_threads, int max_batch, long long max_pixels,
                     cy_server **out) {
    if (!out || budget_bytes <= 0 || workers <= 0 || workers > 16 || max_batch <= 0 || max_pixels <= 0)
        return CY_EINVAL;
    *out = nullptr;
    cy_server *s = new (std::nothrow) cy_server();
    if (!s) return CY_ENOMEM;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return CY_ENODEV;
    }
    s->budget = budget_bytes;
    s->host_threads = host_threads;
    s->max_batch = max_batch;
    s->max_pixels = max_pixels;
    s->engine = 0;
    try {
        for (int i = 0; i < workers; ++i) s->workers.emplace_back([s] { s->worker(); });
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(s->m);
            s->stopping = true;
        }
        s->work_cv.notify_all();
        for (std::thread &t : s->workers) t.join();
        delete s;
        return CY_ENOMEM;
    }
    *out = s;
    return CY_OK;
}

int cy_server_submit(cy_server *s, const void *trace, size_t len, unsigned long long *id) {
    if (!s || !trace || len < 20) return CY_EINVAL;
    request r;
    try {
        r.trace.assign(static_cast<const uint8_t *>(trace), static_cast<const uint8_t *>(trace) + len);
    } catch (...) {
        return CY_ENOMEM;
    }
    r.cost = estimate_cost(r.trace.data(), len, &r.pixels);
    r.t_arrive = now_s();
    {
        std::lock_guard<std::mutex> lk(s->m);
        if (s->stopping) return CY_EINVAL;
        r.id = s->next_id++;
        if (id) *id = r.id;
        s->waiting.push_back(std::move(r));
    }
    s->work_cv.notify_one();
    return CY_OK;
}

int cy_server_poll(cy_server *s, int wait_ms, unsigned long long *id, int *status, unsigned char *images,
                   size_t cap, size_t *len, double *latency_ms) {
    if (!s || !id || !len) return CY_EINVAL;
    std::unique_lock<std::mutex> lk(s->m);
    if (s->done.empty() && wait_ms != 0) {
        if (wait_ms < 0)
            s->done_cv.wait(lk, [s] { return !s->done.empty(); });
        else
            s->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [s] { return !s->done.empty(); });
    }
    if (s->done.empty()) return 1;   // nothing finished yet
    finished &f = s->done.front();
    *len = f.images.size();
    if (f.images.size() > cap) return -2;   // buffer too small; the result stays queued
    if (images && !f.images.empty()) std::memcpy(images, f.images.data(), f.images.size());
    *id = f.id;
    if (status) *status = f.status;
    if (latency_ms) *latency_ms = (f.t_done - f.t_arrive) * 1e3;
    s->done.pop_front();
    return CY_OK;
}

int cy_server_stats(cy_server *s, long long *stats, int n) {
    if (!s || !stats) return CY_EINVAL;
    std::lock_guard<std::mutex> lk(s->m);
    long long v[] = {s->frames, s->requests_done, s->pixels_done, static_cast<long long>(s->waiting.size()),
                     s->in_use, s->max_in_use, s->max_batch_seen, s->budget};
    int k = std::min(n, static_cast<int>(sizeof(v) / sizeof(v[0])));
    for (int i = 0; i < k; ++i) stats[i] = v[i];
    return k;
}

void cy_server_destroy(cy_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stopping = true;
    }
    s->work_cv.notify_all();
    for (std::thread &t : s->workers) t.join();
    delete s;
}

}  // extern "C"
