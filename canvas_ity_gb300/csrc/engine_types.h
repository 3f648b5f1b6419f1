// engine_types.h -- records shared by the host engine and the CUDA kernels.
#ifndef CY_ENGINE_TYPES_H
#define CY_ENGINE_TYPES_H

#include <stdint.h>

namespace cyg {

enum { CMD_FILL = 1, CMD_CLIP = 2, CMD_PUT = 3, CMD_GET = 4 };

// One flattening work item: the start point of a subpath (emits one point)
// or one cubic of it (emits its adaptive polyline, hpp:1398-1487).
struct flat_item {
    int32_t pt;       // index into the Bezier point array (cubic: its start point)
    int32_t sub_end;  // start items: index of the first item after the subpath; cubics: -1
    float angular;    // -1: fill mode; stroking: the cosine limit of hpp:1499-1500
};

// Stroke expansion on the device (stroke_lines, hpp:2070-2100): one style
// per stroked path and one group per subpath of it.
struct stroke_style {
    float half, ratio;            // line_width / 2 and miter_limit^2 * half^2 (hpp:1952-1953)
    int32_t join, cap;            // join_style / cap_style values (hpp:149-150)
    int32_t dash_first, dash_n;   // the dash pattern (dash_n 0: solid)
    int32_t dash_start;           // pattern entry the offset falls in (hpp:1871-1876)
    float dash_next;              // its remaining length (hpp:1888)
    float fwd[6], inv[6];         // current transform and its inverse (a, b, c, d, e, f)
};

struct stroke_group {
    int32_t head, end;   // flat_item range of the subpath (head: its start item)
    int32_t closed;
    int32_t style;
};

// One queued draw, clip or put_image_data, with everything the kernels need.
struct __align__(16) command {
    int32_t kind, op;
    float alpha;
    int32_t geom;         // 0: host polylines, 1: polylines flattened on the GPU, 2: stroke outlines
                          // expanded on the GPU
    int32_t first, count; // geom 0: point range; geom 1: flat_item range; geom 2: stroke_group range
    int32_t line_first, line_count;  // resolved polyline range (filled at flush)
    // paint (paint_pixel, hpp:2265-2377)
    int32_t paint, clamp;
    float inv[6];
    float color[4];
    float p0x, p0y, p1x, p1y, r0, r1;
    int32_t stop_first, stop_count;
    int32_t pat_first, pat_w, pat_h, pat_rep;
    // shadow (render_shadow, hpp:2395-2539)
    int32_t shadow, sh_radius, sh_border, fill_rule;   // fill_rule: 0 nonzero, 1 even-odd
    float sh_color[4];
    float sh_w1, sh_w2, sh_offx, sh_offy;
    // put_image_data
    int32_t put_x, put_y, put_w, put_h;
    int64_t put_first;
    // get_image_data: compact RGBA8 rectangle at get_out in the frame's buffer
    int32_t get_x, get_y, get_w, get_h;
    int64_t get_out;
    // conservative bounds of the geometry, device pixels (host-computed)
    int32_t gx0, gy0, gx1, gy1;
    // pattern texels held by the device image cache (0: pat_first indexes
    // the frame's own texels)
    int64_t pat_ptr;
    int64_t pad_;
};

// Exact bounds of the nonzero coverage deltas a scan conversion produced.
struct cover_box {
    int32_t x0, x1, y0, y1;   // nonzero cells (inclusive); empty if x0 > x1
    int64_t first_key;        // min over all cells of (y << 32 | x), zero deltas included
};

// One signed-area change of a pixel run (the reference's pixel_run,
// hpp:174), bucketed by row so the row index is implicit.
struct run {
    int32_t x;
    float delta;
};

// A clip mask in the reference's sparse form (hpp:1167, 3057-3099): per row
// a list of coalesced runs sorted by x; plus the dense visibility it implies.
struct mask_view {
    const int32_t *row_off;   // H+1 offsets (capacity-based)
    const int32_t *row_len;   // H counts
    const run *runs;
    const float *vis;         // W*H min(|running sum|, 1), 0 outside the runs
};

}  // namespace cyg

#endif
