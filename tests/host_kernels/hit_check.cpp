// hit_check.cpp -- CPU check of the batched is_point_in_path: the items,
// flattening (flatten.cuh) and hit kernel (hit.cuh) that cy_points_in_path
// runs on the GPU, run here once per thread index, against the class's own
// sequential is_point_in_path (src/canvas_ity.hpp:3101-3132 restated in
// canvas.cpp).  The engine's other entry points are stubs.  Prints
// "queries N, differing M".
#include "shim.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../../canvas_ity_gb300/csrc/flatten.cuh"
#include "../../canvas_ity_gb300/csrc/hit.cuh"
using namespace cyg;
#include "../../include/canvas_ity.hpp"
#include "../../include/cy_gpu.h"
struct cy_ctx { int w, h; };
extern "C" {
int cy_points_in_path(const float *points, const int *counts, int n_sub, const float *queries, int n_queries,
                      int fill_rule, unsigned char *inside) {
    std::vector<flat_item> items; size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s]; if (!n) continue;
        int head = items.size(); items.push_back(flat_item{(int)at, 0, -1.0f});
        for (int k = 1; k < n; k += 3) items.push_back(flat_item{(int)(at + k - 1), -1, -1.0f});
        items[head].sub_end = items.size(); at += n;
    }
    if (items.empty()) { memset(inside, 0, n_queries); return 0; }
    int ni = items.size();
    std::vector<int> cnt(ni + 1), off(ni + 1);
    blockDim.x = 256;
    for (int i = 0; i < ni; ++i) { blockIdx.x = i / 256; threadIdx.x = i % 256; k_flat_count((const float2*)points, items.data(), ni, cnt.data()); }
    long long sum = 0; for (int i = 0; i < ni; ++i) { off[i] = sum; sum += cnt[i]; } off[ni] = sum;
    std::vector<float2> pts(sum); std::vector<int> prev(sum);
    for (int i = 0; i < ni; ++i) { blockIdx.x = i / 256; threadIdx.x = i % 256; k_flat_emit((const float2*)points, items.data(), ni, off.data(), pts.data(), prev.data(), sum); }
    for (int q = 0; q < n_queries; ++q) { blockIdx.x = q / 256; threadIdx.x = q % 256; k_points_in_path(pts.data(), prev.data(), sum, (const float2*)queries, n_queries, fill_rule == 1, inside); }
    return 0;
}
int cy_ctx_create(int w, int h, cy_ctx **out) { *out = new cy_ctx{w, h}; return 0; }
void cy_ctx_destroy(cy_ctx *c) { delete c; }
int cy_fill_path(cy_ctx *, const float *, const int *, int, const cy_paint *, const cy_draw_state *) { return 0; }
int cy_fill_lines(cy_ctx *, const float *, const int *, int, const cy_paint *, const cy_draw_state *) { return 0; }
int cy_stroke_path(cy_ctx *, const float *, const int *, const int *, int, const cy_stroke_style *, const cy_paint *, const cy_draw_state *) { return 0; }
void cy_set_device_stroke(int) {}
int cy_device_stroke(void) { return 1; }
int cy_clip_path(cy_ctx *, const float *, const int *, int, int, int, int *out) { *out = 1; return 0; }
int cy_mask_retain(cy_ctx *, int) { return 0; }
int cy_mask_release(cy_ctx *, int) { return 0; }
int cy_get_image(cy_ctx *, unsigned char *, int, int, int, int, int) { return 0; }
int cy_put_image(cy_ctx *, const unsigned char *, int, int, int, int, int) { return 0; }
int cy_read_linear(cy_ctx *, float *) { return 0; }
int cy_flush(cy_ctx *) { return 0; }
int cy_ctx_status(const cy_ctx *) { return 0; }
void cy_set_engine(int) {}
int cy_take_thread_status(void) { return 0; }
void cy_ctx_set_transient(cy_ctx *, int) {}
void cy_set_deferred(int) {}
}
int main() {
    srand(7);
    auto r = [](float a, float b) { return a + (b - a) * (rand() / (float)RAND_MAX); };
    long total = 0, bad = 0;
    for (int t = 0; t < 600; ++t) {
        canvas_ity::canvas c(200, 150);
        if (t % 3 == 1) c.set_fill_rule(canvas_ity::even_odd);
        if (t % 4 == 2) { c.translate(30, 10); c.rotate(0.3f); c.scale(1.25f, 0.8f); }
        c.begin_path();
        std::vector<float> q;
        int subs = 1 + rand() % 3;
        for (int s = 0; s < subs; ++s) {
            float x = (float)(rand() % 150), y = (float)(rand() % 150);
            c.move_to(x, y); q.push_back(x); q.push_back(y);
            int n = 2 + rand() % 6;
            for (int k = 0; k < n; ++k) {
                float u = (float)(rand() % 150), v = (float)(rand() % 150);
                int kind = rand() % 4;
                if (kind == 0) c.line_to(u, v);
                else if (kind == 1) c.bezier_curve_to(r(0,150), r(0,150), r(0,150), r(0,150), u, v);
                else if (kind == 2) c.quadratic_curve_to(r(0,150), r(0,150), u, v);
                else c.arc(u, v, r(5, 40), 0.0f, r(1, 6.28f));
                q.push_back(u); q.push_back(v); q.push_back(u + 0.5f); q.push_back(v);
            }
            if (rand() % 2) c.close_path();
        }
        for (int k = 0; k < 300; ++k) { q.push_back(r(-10, 210)); q.push_back(r(-10, 160)); }
        int nq = q.size() / 2;
        std::vector<unsigned char> got(nq);
        c.points_in_path(q.data(), nq, got.data());
        for (int k = 0; k < nq; ++k) {
            bool want = c.is_point_in_path(q[2*k], q[2*k+1]);
            ++total; if (want != (got[k] != 0)) ++bad;
        }
    }
    printf("queries %ld, differing %ld\n", total, bad);
}
