/*
 * cy_batch.h -- batched many-canvas rendering and engine controls.
 *
 * No reference counterpart: the reference renders one canvas at a time on
 * the calling thread.  A frame renders the queued work of many canvases in
 * one set of launches; with the tile engine (0) all pixel work happens in
 * one persistent kernel that keeps each strip of a canvas in shared memory
 * across all of its draws.  Contexts made while deferred mode is on queue
 * their get_image_data reads instead of flushing; the results are collected
 * with cy_ctx_take_reads after the frame finishes.
 */
#ifndef CY_BATCH_H
#define CY_BATCH_H

#include <stddef.h>

#include "cy_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cy_frame cy_frame;
struct cy_canvas;   /* canvas_ity_c.h */

/* Contexts created afterwards in this thread queue their reads (1) or
 * flush on every read as the reference API requires (0, default). */
void cy_set_deferred(int deferred);

/* Tile engine strip size in pixels (256..12288, shared memory is 16 B per
 * pixel, 24 B with binned coverage, which caps it at 9216) and threads per
 * block (128, 256 or 512). */
void cy_set_strip_config(int strip_pixels, int threads);

/* Coverage of the tile engine's draws, for frames prepared afterwards in
 * any thread.  0 (default), binned: each draw's segments are clipped to the
 * canvas one by one (the polygon clip's result, hpp:2204-2239, in sum),
 * listed per band of rows and accumulated per strip in shared memory as
 * fixed-point signed areas (add_runs' cell areas, hpp:2109-2170, with no
 * sorted runs in memory); coverage is within 1e-5 of the reference's and
 * RGBA8 within +-1 LSB while paths stay within a few hundred pixels of the
 * canvas (further out, the reference's own clip rounding grows with the
 * coordinates, and the binned clip's projection onto x = 0 is exact).  1, exact: row-sorted runs summed in the reference's order
 * (lines_to_runs and render_main, hpp:2193-2253, 2551-2605), so the float
 * canvas is the reference's bit for bit.  The plain engine is always exact. */
void cy_set_coverage(int exact);
int cy_get_coverage(void);

/* Device image cache (no counterpart in the reference, which keeps each
 * pattern and draw_image source with its canvas): an image (set_pattern,
 * draw_image; hpp:568-600, 1030-1067) drawn a second time, on any canvas or
 * request, is kept on the current device already linearised and
 * premultiplied, and later draws of the same bytes use it instead of
 * uploading and converting their own copy.  Up to 1 GiB of texels per
 * device, kept until the process exits.  Statistics for the current device
 * (first n of): hits, images inserted, images held, texel bytes held, pool
 * bytes. */
int cy_image_cache_stats(long long *stats, int n);

/* Build a frame over the queued work of n contexts, upload it and run it
 * once.  engine: 0 tile, 1 plain.  The contexts' queues are consumed by
 * cy_frame_finish. */
int cy_frame_create(cy_ctx *const *ctxs, int n, int engine, cy_frame **out);

/* Run the prepared frame again on the device (asynchronous, no host
 * synchronisation); for timing. */
int cy_frame_run(cy_frame *frame);

/* Autotuner of the tile engine: times the frame's paint stage (the strip
 * kernel alone, which a frame of deferred canvases can repeat) for strip
 * sizes 2048..12288 pixels (no narrower than the widest canvas) and 128,
 * 256 or 512 threads per block, keeps the fastest for this frame and makes
 * it the process's strip configuration (cy_set_strip_config).  After the
 * frame's first run; CY_EINVAL for the plain engine or non-deferred
 * contexts. */
int cy_frame_autotune(cy_frame *frame, int *strip_pixels, int *threads, float *paint_ms);

/* Capture one device-only run of the frame (after its first run) into a
 * CUDA graph; later cy_frame_run calls launch the graph instead of issuing
 * each kernel.  Not used while profiling is on.  CY_EINVAL before the first
 * run; a capture that fails leaves the frame running without a graph. */
int cy_frame_capture(cy_frame *frame);

/* Wait for the frame's stream. */
int cy_frame_sync(cy_frame *frame);

/* The frame's CUDA stream (cudaStream_t), for event timing. */
void *cy_frame_stream(cy_frame *frame);

/* Copy the reads out, release queued resources. */
int cy_frame_finish(cy_frame *frame);

/* Destroying a frame keeps its device and pinned buffers (up to four sets
 * per device) for the next cy_frame_create, which then allocates only what
 * grows.  cy_frame_workspace_release frees what is kept. */
void cy_frame_destroy(cy_frame *frame);
void cy_frame_workspace_release(void);

/* Profiling: when on, each run records CUDA events on the frame's stream at
 * its phase boundaries.  cy_frame_profile waits for the stream and writes
 * the phase durations in ms: [0] patterns + flattening, [1] scan conversion
 * (run counting, bucketing, row sort/prefix), [2] clip masks + shadow
 * images, [3] paint (the strip kernel, or all per-draw launches).  Returns
 * the number of phases written. */
int cy_frame_set_profiling(cy_frame *frame, int on);
int cy_frame_profile(cy_frame *frame, float *phase_ms, int n);

/* Frame statistics (first n of): pixels, commands, segments (scanned: run
 * jobs' after the polygon clip, binned draws' as given), runs, rows,
 * runs of draws, rows of draws, shadow image floats, read-back bytes,
 * uploaded bytes, kernel launches per run, shadows, clips, binned segment
 * entries, binned (1) or exact (0) coverage. */
int cy_frame_stats(cy_frame *frame, long long *stats, int n);

/* Replay n call lists (cy_trace.h) into n new canvases whose reads are
 * deferred, on `threads` host threads (0: one per core); engine as for
 * cy_set_engine.  out[i] receives canvas i (release with
 * cy_canvas_delete); cy_canvas_ctx gives the contexts for cy_frame_create.
 * On failure no canvas is kept and the first failing status is returned. */
int cy_canvases_from_traces(const void *const *traces, const size_t *lens, int n, int engine, int threads,
                            struct cy_canvas **out);

/* After cy_frame_finish: the deferred reads of all the frame's contexts,
 * context by context (each in call order), copied into `out`;
 * offsets[0..n] (n = contexts) receive where each context's bytes start and
 * the total.  -2 if cap is too small (offsets are still filled).  The
 * contexts' reads are consumed, as by cy_ctx_take_reads. */
int cy_frame_collect(cy_frame *frame, unsigned char *out, size_t cap, size_t *offsets);

/* cy_frame_finish without moving the reads: the frame keeps them in its
 * pinned host buffer, which the device->host copy fills directly.  *data
 * receives that buffer and offsets[0..n] where each context's reads start
 * and their end (each context's reads in call order, compact RGBA8).  The
 * bytes stay valid until the frame runs again or is destroyed; the
 * contexts' own deferred reads stay empty. */
int cy_frame_finish_views(cy_frame *frame, const unsigned char **data, size_t *offsets);

/* End to end over many call lists: replay on the host, upload, render and
 * read back, in frames of about `frame_pixels` canvas pixels (0: 32 Mi).
 * While the device renders one frame, the host replays and stages the
 * next, and copies out the one before.  Canvas i's reads (compact RGBA8
 * rectangles in call order) are written to out[offsets[i] .. offsets[i+1]);
 * the caller knows them from its get_image_data calls, and a canvas whose
 * reads do not fill its range exactly fails the call with CY_EINVAL.
 * stats (may be NULL) receives [0] frames, [1] bytes uploaded, [2] bytes
 * read back. */
int cy_render_traces(const void *const *traces, const size_t *lens, int n, int engine, long long frame_pixels,
                     unsigned char *out, const size_t *offsets, long long *stats);

/* Deferred reads of a context, concatenated in call order (compact RGBA8
 * rectangles); -2 if cap is too small (*len holds the size). */
int cy_ctx_take_reads(cy_ctx *ctx, unsigned char *out, size_t cap, size_t *len);

#ifdef __cplusplus
}
#endif

#endif /* CY_BATCH_H */
