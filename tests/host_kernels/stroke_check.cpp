// stroke_check.cpp -- CPU check of the device stroke expansion: the
// flattening, dash, piece, walk and join kernels of flatten.cuh and
// stroke.cuh, run as host C++ (warp_emu.h), against the host class's own
// stroke expansion (canvas.cpp, the reference's dash_lines / stroke_lines
// restated, built with cr_trig.h so its round joins round acos/tan from
// double as the device does).  Every call list given on the command line is
// replayed twice, strokes expanded by the kernels and by the host, and every
// filled polygon is compared bit for bit.  Prints "commands N, differing M".
#include "warp_emu.h"
#include <cstdio>
#include <cstdlib>
#include <string>
#include "../../canvas_ity_gb300/csrc/flatten.cuh"
#include "../../canvas_ity_gb300/csrc/stroke.cuh"
#include "../../include/cy_gpu.h"
#include "../../include/cy_batch.h"
#include "../../include/canvas_ity_c.h"
using namespace cyg;

struct cy_ctx { int w, h; };
typedef std::vector<std::vector<float2>> polys;
static std::vector<polys> g_seq;   // the filled polygons of every draw, in order
static int g_device = 0;

// The outline of one stroke() through the kernels, as the engine runs them
// (engine.cu queue_stroke and frame::stroke_passes) for one path.
static polys device_outline(const float *points, const int *counts, const int *closed, int n_sub,
                            const cy_stroke_style *style) {
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
    if (style->n_dash > 0) {   // the dash phase at a subpath's start, hpp:1867-1876
        const float *dash = style->dash;
        int nd = style->n_dash;
        float sum = 0.0f;
        for (int i = 0; i < nd; ++i) sum = sum + dash[i];
        float offset = fmodf(style->dash_offset, sum);
        if (offset < 0.0f) offset += sum;
        int start = 0;
        while (offset >= dash[start]) {
            offset -= dash[start];
            start = start + 1 < nd ? start + 1 : 0;
        }
        st.dash_n = nd;
        st.dash_start = start;
        st.dash_next = dash[start] - offset;
    }
    float tol = 0.125f;
    float ratio = tol / (0.5f * style->line_width < tol ? tol : 0.5f * style->line_width);
    float angular = (ratio - 2.0f) * ratio * 2.0f + 1.0f;
    // flattening items and groups (one per subpath)
    std::vector<flat_item> items;
    std::vector<stroke_group> groups;
    size_t at = 0;
    for (int s = 0; s < n_sub; ++s) {
        int n = counts[s];
        if (n == 0) continue;
        stroke_group g;
        g.head = static_cast<int32_t>(items.size());
        g.closed = closed[s] ? 1 : 0;
        g.style = 0;
        items.push_back(flat_item{static_cast<int32_t>(at), 0, angular});
        for (int k = 1; k < n; k += 3) items.push_back(flat_item{static_cast<int32_t>(at + k - 1), -1, angular});
        g.end = static_cast<int32_t>(items.size());
        items[g.head].sub_end = g.end;
        groups.push_back(g);
        at += n;
    }
    polys ps;
    const int ni = static_cast<int>(items.size()), ng = static_cast<int>(groups.size());
    if (ng == 0) return ps;
    const float2 *bez = reinterpret_cast<const float2 *>(points);
    std::vector<int32_t> cnt(ni + 1), off(ni + 1);
    run_threads(ni, 256, [&] { k_flat_count(bez, items.data(), ni, cnt.data()); });
    off[0] = 0;
    for (int i = 0; i < ni; ++i) off[i + 1] = off[i] + cnt[i];
    const int nflat = off[ni];
    std::vector<float2> flat(nflat + 1);
    std::vector<int32_t> flat_prev(nflat + 1);
    run_threads(ni, 256, [&] { k_flat_emit(bez, items.data(), ni, off.data(), flat.data(), flat_prev.data(), nflat); });
    std::vector<float> dash(style->dash, style->dash + style->n_dash);
    int32_t err = 0;
    std::vector<int32_t> dcnt(ng + 2), doff(ng + 2), dnsub(ng + 2);
    std::vector<float2> dpts(1);
    std::vector<int2> dsubs(1);
    stroke_in si;
    std::memset(&si, 0, sizeof(si));
    si.flat = flat.data();
    si.item_off = off.data();
    si.groups = groups.data();
    si.styles = &st;
    si.dash = dash.data();
    si.dash_pts = dpts.data();
    si.dash_subs = dsubs.data();
    si.dash_off = doff.data();
    si.dash_nsub = dnsub.data();
    std::vector<dash_state> dstate(static_cast<size_t>(nflat) + 1);
    si.dash_state_at = dstate.data();
    si.nflat = nflat;
    si.n = ng;
    si.error = &err;
    if (st.dash_n > 0) {
        run_warps(ng, kStrokeWarps, [&] { k_dash<false>(si, dcnt.data()); });
        doff[0] = 0;
        for (int g = 0; g < ng; ++g) doff[g + 1] = doff[g] + dcnt[g];
        dpts.resize(doff[ng] + 1);
        dsubs.resize(doff[ng] + 1);
        si.dash_pts = dpts.data();
        si.dash_subs = dsubs.data();
        run_warps(ng, kStrokeWarps, [&] { k_dash<true>(si, nullptr); });
    }
    std::vector<int32_t> pcnt(ng + 2), pbase(ng + 2);
    run_threads(ng, 256, [&] { k_piece_count(si, pcnt.data()); });
    pbase[0] = 0;
    for (int g = 0; g < ng; ++g) pbase[g + 1] = pbase[g] + pcnt[g];
    const int npc = pbase[ng];
    std::vector<stroke_piece> pieces(npc + 1);
    run_threads(ng, 256, [&] { k_pieces(si, pbase.data(), pieces.data()); });
    std::vector<int32_t> wcnt(npc + 2), wbase(npc + 2);
    run_threads(npc, 256, [&] { k_piece_chunks(si, pieces.data(), npc, wcnt.data()); });
    wbase[0] = 0;
    for (int i = 0; i < npc; ++i) wbase[i + 1] = wbase[i] + wcnt[i];
    const int nch = wbase[npc];
    std::vector<walk_chunk> chunks(nch + 1);
    run_warps(npc, kStrokeWarps, [&] { k_walk(si, pieces.data(), npc, wbase.data(), chunks.data()); });
    std::vector<int32_t> lanes(nch + 1), pos_base(nch + 2);
    run_threads(nch, 256, [&] { k_chunk_lanes(chunks.data(), nch, lanes.data()); });
    pos_base[0] = 0;
    for (int c = 0; c < nch; ++c) pos_base[c + 1] = pos_base[c] + lanes[c];
    const int njp = pos_base[nch];
    std::vector<int32_t> pos_chunk(njp + 1, -1);
    run_threads(nch * 32, 256, [&] { k_chunk_positions(chunks.data(), nch, pos_base.data(), pos_chunk.data()); });
    for (int p = 0; p < njp; ++p)
        if (pos_chunk[p] < 0) {
            std::fprintf(stderr, "unmapped position %d\n", p);
            std::exit(2);
        }
    std::vector<int32_t> jcnt(njp + 1);
    std::vector<float> jalpha(njp + 1);
    std::vector<int64_t> joff(njp + 2);
    run_threads(njp, kStrokeWarps * 32, [&] {
        k_join<false>(si, chunks.data(), pos_base.data(), pos_chunk.data(), njp, jcnt.data(), jalpha.data(), nullptr,
                      nullptr, nullptr, 0, 0);
    });
    joff[0] = 0;
    for (int p = 0; p < njp; ++p) joff[p + 1] = joff[p] + jcnt[p];
    if (err) {
        std::fprintf(stderr, "stroke error flag\n");
        std::exit(2);
    }
    const int64_t n = joff[njp];
    const int base = 1000;
    std::vector<float2> out(n + 1);
    std::vector<int32_t> prev(n + 1, -7);
    run_threads(njp, kStrokeWarps * 32, [&] {
        k_join<true>(si, chunks.data(), pos_base.data(), pos_chunk.data(), njp, jcnt.data(), jalpha.data(), joff.data(),
                     out.data(), prev.data(), base, n);
    });
    // polygons from the links: prev of a polygon's first point is its last
    for (int64_t k = 0; k < n;) {
        int64_t last = prev[k] - base;
        if (last < k || last >= n) {
            std::fprintf(stderr, "bad link at %lld\n", static_cast<long long>(k));
            std::exit(2);
        }
        for (int64_t j = k + 1; j <= last; ++j)
            if (prev[j] - base != j - 1) {
                std::fprintf(stderr, "bad inner link at %lld\n", static_cast<long long>(j));
                std::exit(2);
            }
        ps.push_back(std::vector<float2>(out.begin() + k, out.begin() + last + 1));
        k = last + 1;
    }
    return ps;
}

// The engine's entry points: draws are recorded, nothing is rendered.
extern "C" {
void cy_set_device_stroke(int on) { g_device = on; }
int cy_device_stroke(void) { return g_device; }
int cy_ctx_create(int w, int h, cy_ctx **out) {
    *out = new cy_ctx{w, h};
    return 0;
}
void cy_ctx_destroy(cy_ctx *c) { delete c; }
int cy_fill_path(cy_ctx *, const float *, const int *, int, const cy_paint *, const cy_draw_state *) { return 0; }
int cy_fill_lines(cy_ctx *, const float *p, const int *n, int ns, const cy_paint *, const cy_draw_state *) {
    polys ps;
    size_t at = 0;
    for (int s = 0; s < ns; ++s) {
        std::vector<float2> v;
        for (int k = 0; k < n[s]; ++k, ++at) v.push_back(make_float2(p[2 * at], p[2 * at + 1]));
        if (!v.empty()) ps.push_back(v);
    }
    g_seq.push_back(ps);
    return 0;
}
int cy_stroke_path(cy_ctx *, const float *points, const int *counts, const int *closed, int n_sub,
                   const cy_stroke_style *style, const cy_paint *, const cy_draw_state *) {
    const float *fw = style->forward;
    if (fw[0] * fw[3] - fw[1] * fw[2] == 0.0f) return 0;
    g_seq.push_back(device_outline(points, counts, closed, n_sub, style));
    return 0;
}
int cy_points_in_path(const float *, const int *, int, const float *, int, int, unsigned char *) { return 0; }
int cy_clip_path(cy_ctx *, const float *, const int *, int, int, int, int *out) {
    *out = 1;
    return 0;
}
int cy_mask_retain(cy_ctx *, int) { return 0; }
int cy_mask_release(cy_ctx *, int) { return 0; }
int cy_get_image(cy_ctx *, unsigned char *img, int w, int h, int stride, int, int) {
    for (int y = 0; y < h; ++y) std::memset(img + static_cast<size_t>(y) * stride, 0, static_cast<size_t>(w) * 4);
    return 0;
}
int cy_put_image(cy_ctx *, const unsigned char *, int, int, int, int, int) { return 0; }
int cy_read_linear(cy_ctx *, float *) { return 0; }
int cy_flush(cy_ctx *) { return 0; }
int cy_ctx_status(const cy_ctx *) { return 0; }
void cy_set_engine(int) {}
void cy_set_deferred(int) {}
int cy_take_thread_status(void) { return 0; }
void cy_ctx_set_transient(cy_ctx *, int) {}
int cy_frame_create(cy_ctx *const *, int, int, cy_frame **) { return CY_ENODEV; }
int cy_frame_stats(cy_frame *, long long *, int) { return 0; }
int cy_frame_finish_views(cy_frame *, const unsigned char **, size_t *) { return CY_ENODEV; }
void cy_frame_destroy(cy_frame *) {}
}

int main(int argc, char **argv) {
    std::vector<unsigned char> img(64 << 20);
    std::vector<float> res(1 << 16);
    long long cmds = 0, bad = 0;
    for (int a = 1; a < argc; ++a) {
        FILE *f = std::fopen(argv[a], "rb");
        if (!f) return 1;
        std::fseek(f, 0, SEEK_END);
        long len = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        std::vector<unsigned char> tr(len);
        if (std::fread(tr.data(), 1, len, f) != static_cast<size_t>(len)) return 1;
        std::fclose(f);
        std::vector<polys> by_mode[2];
        for (int mode = 0; mode < 2; ++mode) {
            g_seq.clear();
            g_device = mode;
            size_t il = 0;
            int rl = 0;
            cy_replay(tr.data(), tr.size(), img.data(), img.size(), &il, res.data(), static_cast<int>(res.size()), &rl);
            by_mode[mode] = g_seq;
        }
        if (by_mode[0].size() != by_mode[1].size()) {
            std::printf("%s: %zu draws on the host, %zu through the kernels\n", argv[a], by_mode[0].size(),
                        by_mode[1].size());
            ++bad;
            continue;
        }
        for (size_t i = 0; i < by_mode[0].size(); ++i) {
            ++cmds;
            const polys &h = by_mode[0][i], &d = by_mode[1][i];
            bool same = h.size() == d.size();
            for (size_t q = 0; same && q < h.size(); ++q)
                same = h[q].size() == d[q].size() && !std::memcmp(h[q].data(), d[q].data(), h[q].size() * sizeof(float2));
            if (!same) ++bad;
        }
    }
    std::printf("commands %lld, differing %lld\n", cmds, bad);
    return 0;
}
