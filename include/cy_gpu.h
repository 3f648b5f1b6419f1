/*
 * cy_gpu.h -- C ABI of the GB300 render engine behind canvas_ity::canvas.
 *
 * The reference library renders on the CPU inside the canvas class; the
 * host class of this library (include/canvas_ity.hpp) keeps the state and
 * geometry work and hands each draw to these entry points.  Every function
 * names the reference code it replaces (hpp = src/canvas_ity.hpp).
 *
 * Plain pointers and sizes only.  All input buffers are copied before the
 * call returns.  Work is queued per context, in call order, on the
 * context's own CUDA stream, and runs when pixels are read (cy_get_image),
 * on cy_flush, or when the queue grows large.  Status codes: 0 success,
 * negative on failure (CY_E*).  A context is not thread-safe; separate
 * contexts may be used from separate threads.
 */
#ifndef CY_GPU_H
#define CY_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CY_OK 0
#define CY_EINVAL (-1)    /* invalid argument                               */
#define CY_ENOMEM (-2)    /* device or pinned host allocation failed        */
#define CY_ECUDA (-3)     /* a CUDA call failed                             */
#define CY_ENODEV (-4)    /* no usable CUDA device                          */
#define CY_EBUDGET (-5)   /* request exceeds the admission memory budget     */

typedef struct cy_ctx cy_ctx;

/* Paint of one draw: the reference's paint_brush (hpp:165-168) resolved at
 * draw time, plus the canvas inverse transform used to map pixel centres
 * into pattern / gradient space (paint_pixel, hpp:2265-2377). */
enum cy_paint_kind {
    CY_PAINT_NONE = 0,     /* empty brush: transparent black            */
    CY_PAINT_SOLID = 1,    /* color[] premultiplied linear              */
    CY_PAINT_LINEAR = 2,
    CY_PAINT_RADIAL = 3,
    CY_PAINT_PATTERN = 4
};

typedef struct cy_paint {
    int kind;                  /* enum cy_paint_kind                           */
    int clamp_edges;           /* 1 for draw_image (clamp), 0 for patterns (wrap) */
    float inverse[6];          /* a b c d e f of the inverse canvas transform  */
    float color[4];            /* SOLID: premultiplied linear RGBA             */
    float start[2], end[2];    /* gradient geometry                            */
    float start_radius, end_radius;
    const float *stop_offsets; /* n_stops offsets, sorted ascending            */
    const float *stop_colors;  /* n_stops * 4, linear straight-alpha RGBA      */
    int n_stops;
    const unsigned char *pattern; /* PATTERN: sRGB RGBA8, width*4 row stride   */
    int pattern_width, pattern_height;
    int repetition;            /* repeat, repeat_x, repeat_y, no_repeat        */
} cy_paint;

/* Compositing state of one draw (hpp:2395-2605). */
typedef struct cy_draw_state {
    int operation;             /* composite_operation value                   */
    float global_alpha;
    int mask;                  /* clip mask id; 0 = whole canvas              */
    float shadow_color[4];     /* premultiplied linear                        */
    float shadow_blur;
    float shadow_offset_x, shadow_offset_y;
    int fill_rule;             /* extension: 0 nonzero (the reference's), 1 even-odd */
} cy_draw_state;

/* canvas::canvas (hpp:2607-2644): transparent W x H canvas, full clip. */
int cy_ctx_create(int width, int height, cy_ctx **out);

/* canvas::~canvas (hpp:2646-2655). */
void cy_ctx_destroy(cy_ctx *ctx);

/* fill() of a Bezier path: path_to_lines(false) + render_main
 * (hpp:3044-3048, 1495-1524, 2551-2605).  `points` holds device-space x,y
 * pairs laid out as the reference's bezier_path: each subpath is one start
 * point followed by 3 points per cubic; subpath_counts[i] is its point count
 * (1 + 3k).  Flattening happens on the GPU. */
int cy_fill_path(cy_ctx *ctx, const float *points, const int *subpath_counts, int n_subpaths,
                 const cy_paint *paint, const cy_draw_state *state);

/* render_main on ready polylines (hpp:2551-2605): strokes expanded on the
 * host (stroke_rectangle, stroke_text, or cy_set_device_stroke(0)),
 * rectangles, images and text.  Every subpath is implicitly
 * closed, as in lines_to_runs (hpp:2193-2253). */
int cy_fill_lines(cy_ctx *ctx, const float *points, const int *subpath_counts, int n_subpaths,
                  const cy_paint *paint, const cy_draw_state *state);

/* Stroke style of one stroke() (hpp:375-440, 1858-2100). */
typedef struct cy_stroke_style {
    float line_width;
    float miter_limit;
    int line_join;             /* canvas_ity::join_style: 0 miter, 1 bevel, 2 rounded */
    int line_cap;              /* canvas_ity::cap_style: 0 butt, 1 square, 2 circle  */
    const float *dash;         /* the pattern as set_line_dash stores it, or NULL    */
    int n_dash;                /* 0: solid                                           */
    float dash_offset;
    float forward[6];          /* a b c d e f of the current transform               */
    float inverse[6];          /* and of its inverse                                 */
} cy_stroke_style;

/* stroke() with the stroke expansion on the GPU: path_to_lines(true),
 * dash_lines, stroke_lines and render_main (hpp:3050-3055, 1495-1524,
 * 1858-2100, 2551-2605).  `points` and `subpath_counts` are laid out as for
 * cy_fill_path; subpath_closed[i] is the subpath's closed flag.  The
 * outline is the reference's point for point, except that a round join's
 * acosf/tanf are taken in double precision and rounded to float.  Fails
 * with CY_ENOMEM when a subpath would dash into more than 2^22 points. */
int cy_stroke_path(cy_ctx *ctx, const float *points, const int *subpath_counts, const int *subpath_closed,
                   int n_subpaths, const cy_stroke_style *style, const cy_paint *paint,
                   const cy_draw_state *state);

/* is_point_in_path (hpp:3101-3132) for many points at once: the path is
 * laid out as for cy_fill_path (device-space Bezier points, 1 + 3k per
 * subpath); queries holds n_queries x,y pairs in device space, as the
 * reference takes them; inside[i] receives 1 when query i is inside (on
 * the boundary counts as inside) under fill_rule (0 nonzero, 1 even-odd).
 * The path is flattened and tested on the GPU; returns after the results
 * are written.  No counterpart in the reference (one point per call). */
int cy_points_in_path(const float *points, const int *subpath_counts, int n_subpaths, const float *queries,
                      int n_queries, int fill_rule, unsigned char *inside);

/* Where canvas_ity::canvas::stroke() expands strokes, for every canvas of
 * the process: 1 (the default) on the GPU through cy_stroke_path, 0 on the
 * host (the reference's own acosf/tanf) through cy_fill_lines. */
void cy_set_device_stroke(int on);
int cy_device_stroke(void);

/* clip() (hpp:3057-3099): intersects mask `mask_in` with the coverage of
 * the Bezier path under `fill_rule` (0 nonzero as in the reference, 1
 * even-odd); the new mask id is written to *mask_out.  Mask ids are
 * reference counted: a new mask starts with one reference. */
int cy_clip_path(cy_ctx *ctx, const float *points, const int *subpath_counts, int n_subpaths,
                 int mask_in, int fill_rule, int *mask_out);

/* Reference counting of mask ids for save()/restore() (hpp:3410-3465). */
int cy_mask_retain(cy_ctx *ctx, int mask);
int cy_mask_release(cy_ctx *ctx, int mask);

/* get_image_data (hpp:3348-3381): runs queued work, then converts the
 * rectangle to unpremultiplied sRGB RGBA8 with the 4x4 ordered dither. */
int cy_get_image(cy_ctx *ctx, unsigned char *image, int width, int height, int stride, int x, int y);

/* put_image_data (hpp:3383-3408), ordered with queued draws. */
int cy_put_image(cy_ctx *ctx, const unsigned char *image, int width, int height, int stride,
                 int x, int y);

/* Extension, no reference counterpart: runs queued work, then copies the
 * canvas's premultiplied linear float RGBA pixels (the reference's private
 * `bitmap`, hpp:1171) into out[W*H*4].  Used to check coverage exactly. */
int cy_read_linear(cy_ctx *ctx, float *out);

/* No counterpart in the reference's library: get_image_data of a rectangle
 * written as an image file, packed on the GPU.  format 0: TGA as the
 * reference's tiger demo writes it (demos/tiger/tiger.cpp:4336-4343,
 * BGRA, top-left origin, w and h up to 65535); format 1: PNG as the
 * reference's test harness writes it (test/test.cpp:2415-2511, RGBA8, one
 * stored deflate block per row, w up to 16383).  Runs queued work first.
 * *len receives the file size; CY_ENOMEM (nothing written) when out is
 * NULL or cap is smaller. */
int cy_encode_image(cy_ctx *ctx, int format, int x, int y, int width, int height, unsigned char *out, size_t cap,
                    size_t *len);

/* Run all queued work and wait for it. */
int cy_flush(cy_ctx *ctx);

/* Largest rectangle cy_get_image_noalloc reads: 1024 x 1024 pixels (a
 * 4 MiB device array that every GPU loading this library keeps until exit). */
#define CY_GET_IMAGE_NOALLOC_MAX_PIXELS (1024 * 1024)

/* No counterpart in the reference.  get_image_data for callers that must
 * not allocate: code running under a memory pool or budget it does not own
 * (a serving loop admitting work against a fixed HBM budget, a host program
 * whose GPU memory is reserved by another framework), or on a latency path
 * where cudaMalloc/cudaFree would stall other streams while the device
 * synchronises.  Converts the canvas as of its last flush exactly like
 * cy_get_image, staging in one fixed device array instead of allocated
 * memory, and calls no allocating routine.
 *   - Call with the context's device current (CY_EINVAL otherwise; the
 *     context stays usable).  The first call on a device
 *     looks up the array's device address (cudaGetSymbolAddress) and, if no
 *     frame has run on the device yet, copies the 16 KiB colour-conversion
 *     table into its fixed device array; make that first call before any
 *     stream capture on the device.
 *   - Fails with CY_EINVAL when width*height exceeds
 *     CY_GET_IMAGE_NOALLOC_MAX_PIXELS, when stride < 4*width, or when the
 *     context still holds queued commands (run cy_flush first: a flush may
 *     allocate).  Returns when the pixels are in `image`.
 *   - No batched frame (include/cy_batch.h) that holds the context may be
 *     running: after cy_frame_run, call cy_frame_sync or cy_frame_finish
 *     first, since the frame's stream writes the canvas.
 *   - All calls share the array.  Each call writes every pixel it copies
 *     back, so no part of the array has to start at zero.  Calls from the
 *     threads of one process are serialised by a lock and each waits for
 *     its copy; calls whose kernels and copies overlapped on the GPU would
 *     race on the array. */
int cy_get_image_noalloc(cy_ctx *ctx, unsigned char *image, int width, int height, int stride, int x, int y);

/* First failure seen by the context (0 if none). */
int cy_ctx_status(const cy_ctx *ctx);

/* Engine selection for contexts created afterwards in this thread:
 * 0 = tile engine (whole flush in one persistent launch, default),
 * 1 = plain engine (per-draw launches over the float canvas). */
void cy_set_engine(int engine);

#ifdef __cplusplus
}
#endif

#endif /* CY_GPU_H */
