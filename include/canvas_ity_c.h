/*
 * canvas_ity_c.h -- C binding of the canvas_ity public API.
 *
 * The reference (src/canvas_ity.hpp) is a C++ class with no C interface;
 * this is the flat binding an FFI (ctypes, cgo, JNI, N-API) would wrap.
 * One function per public member, same argument order and meaning, same
 * silent handling of invalid arguments.  Public data members of the class
 * (global_composite_operation, shadow_offset_x, ...) get setters.
 * Citations: hpp = src/canvas_ity.hpp.
 */
#ifndef CANVAS_ITY_C_H
#define CANVAS_ITY_C_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cy_canvas cy_canvas;

cy_canvas *cy_canvas_new(int width, int height);                               /* hpp:194-204  */
void cy_canvas_delete(cy_canvas *c);                                            /* hpp:206-210  */
int cy_canvas_status(const cy_canvas *c);   /* 0 or the first engine failure (cy_gpu.h codes) */
void cy_canvas_scale(cy_canvas *c, float x, float y);                          /* hpp:212-226  */
void cy_canvas_rotate(cy_canvas *c, float angle);                              /* hpp:228-237  */
void cy_canvas_translate(cy_canvas *c, float x, float y);                      /* hpp:239-249  */
void cy_canvas_transform(cy_canvas *c, float a, float b, float cc, float d, float e, float f); /* hpp:251-271 */
void cy_canvas_set_transform(cy_canvas *c, float a, float b, float cc, float d, float e, float f); /* hpp:273-294 */
void cy_canvas_set_global_alpha(cy_canvas *c, float alpha);                    /* hpp:298-309  */
void cy_canvas_set_global_composite_operation(cy_canvas *c, int op);           /* hpp:311-330  */
void cy_canvas_set_shadow_color(cy_canvas *c, float r, float g, float b, float a); /* hpp:334-354 */
void cy_canvas_set_shadow_offset_x(cy_canvas *c, float v);                     /* hpp:356-361  */
void cy_canvas_set_shadow_offset_y(cy_canvas *c, float v);                     /* hpp:363-368  */
void cy_canvas_set_shadow_blur(cy_canvas *c, float level);                     /* hpp:370-383  */
void cy_canvas_set_line_width(cy_canvas *c, float width);                      /* hpp:387-396  */
void cy_canvas_set_line_cap(cy_canvas *c, int cap);                            /* hpp:398-404  */
void cy_canvas_set_line_join(cy_canvas *c, int join);                          /* hpp:406-415  */
void cy_canvas_set_miter_limit(cy_canvas *c, float limit);                     /* hpp:417-431  */
void cy_canvas_set_line_dash_offset(cy_canvas *c, float offset);               /* hpp:433-440  */
void cy_canvas_set_line_dash(cy_canvas *c, const float *segments, int count);  /* hpp:442-466  */
void cy_canvas_set_color(cy_canvas *c, int type, float r, float g, float b, float a); /* hpp:470-487 */
void cy_canvas_set_linear_gradient(cy_canvas *c, int type, float x0, float y0, float x1, float y1); /* hpp:489-510 */
void cy_canvas_set_radial_gradient(cy_canvas *c, int type, float x0, float y0, float r0,
                                   float x1, float y1, float r1);               /* hpp:512-538  */
void cy_canvas_add_color_stop(cy_canvas *c, int type, float offset, float r, float g, float b,
                              float a);                                         /* hpp:540-566  */
void cy_canvas_set_pattern(cy_canvas *c, int type, const unsigned char *image, int width, int height,
                           int stride, int repetition);                         /* hpp:568-600  */
void cy_canvas_begin_path(cy_canvas *c);                                        /* hpp:611-617  */
void cy_canvas_move_to(cy_canvas *c, float x, float y);                        /* hpp:619-628  */
void cy_canvas_close_path(cy_canvas *c);                                        /* hpp:630-637  */
void cy_canvas_line_to(cy_canvas *c, float x, float y);                        /* hpp:639-651  */
void cy_canvas_quadratic_curve_to(cy_canvas *c, float cx, float cy, float x, float y); /* hpp:653-673 */
void cy_canvas_bezier_curve_to(cy_canvas *c, float c1x, float c1y, float c2x, float c2y,
                               float x, float y);                              /* hpp:675-699  */
void cy_canvas_arc_to(cy_canvas *c, float vx, float vy, float x, float y, float radius); /* hpp:701-729 */
void cy_canvas_arc(cy_canvas *c, float x, float y, float radius, float a0, float a1, int ccw); /* hpp:731-756 */
void cy_canvas_rectangle(cy_canvas *c, float x, float y, float w, float h);    /* hpp:758-776  */
void cy_canvas_fill(cy_canvas *c);                                              /* hpp:780-797  */
void cy_canvas_stroke(cy_canvas *c);                                            /* hpp:799-816  */
void cy_canvas_clip(cy_canvas *c);                                              /* hpp:818-832  */
int cy_canvas_is_point_in_path(cy_canvas *c, float x, float y);                /* hpp:834-848  */
void cy_canvas_clear_rectangle(cy_canvas *c, float x, float y, float w, float h); /* hpp:852-868 */
void cy_canvas_fill_rectangle(cy_canvas *c, float x, float y, float w, float h);  /* hpp:870-888 */
void cy_canvas_stroke_rectangle(cy_canvas *c, float x, float y, float w, float h);/* hpp:890-910 */
void cy_canvas_set_text_align(cy_canvas *c, int align);                        /* hpp:912-924  */
void cy_canvas_set_text_baseline(cy_canvas *c, int baseline);                  /* hpp:926-937  */
int cy_canvas_set_font(cy_canvas *c, const unsigned char *font, int bytes, float size); /* hpp:939-958 */
void cy_canvas_fill_text(cy_canvas *c, const char *text, float x, float y, float max_width); /* hpp:960-983 */
void cy_canvas_stroke_text(cy_canvas *c, const char *text, float x, float y, float max_width); /* hpp:985-1008 */
float cy_canvas_measure_text(cy_canvas *c, const char *text);                  /* hpp:1010-1026 */
void cy_canvas_draw_image(cy_canvas *c, const unsigned char *image, int width, int height, int stride,
                          float x, float y, float to_width, float to_height);  /* hpp:1030-1067 */
void cy_canvas_get_image_data(cy_canvas *c, unsigned char *image, int width, int height, int stride,
                              int x, int y);                                    /* hpp:1071-1095 */
void cy_canvas_put_image_data(cy_canvas *c, const unsigned char *image, int width, int height,
                              int stride, int x, int y);                        /* hpp:1097-1124 */
void cy_canvas_save(cy_canvas *c);                                              /* hpp:1128-1136 */
void cy_canvas_restore(cy_canvas *c);                                           /* hpp:1138-1145 */
/* Extension, no reference counterpart: 0 nonzero (default), 1 even-odd for
 * fill(), clip() and is_point_in_path(). */
void cy_canvas_set_fill_rule(cy_canvas *c, int rule);
/* Extension, no reference counterpart: is_point_in_path for n points (x, y
 * pairs) at once on the GPU; inside[i] receives 0 or 1.  Returns 0 or a
 * negative status (cy_gpu.h). */
int cy_canvas_points_in_path(cy_canvas *c, const float *xy, int n, unsigned char *inside);

/* Replay a recorded call list (cy_trace.h) through canvas_ity::canvas.
 * Every non-null get_image_data appends its compact RGBA8 rectangle to
 * `images`; is_point_in_path / measure_text append their value to
 * `results`.  Returns 0, -1 for a malformed trace, -2 when a buffer is too
 * small (the needed sizes are still reported), or an engine status. */
int cy_replay(const void *trace, size_t trace_len, void *images, size_t images_cap, size_t *images_len,
              float *results, int results_cap, int *results_len);

/* Extension: replay a call list and return the final premultiplied linear
 * float RGBA canvas (width*height*4 floats; the canvas size is reported),
 * for exact coverage comparisons.  Returns 0, -1, -2 (out too small) or an
 * engine status. */
int cy_replay_linear(const void *trace, size_t trace_len, float *out, size_t out_floats, int *width,
                     int *height);

/* Batched rendering helpers (cy_batch.h): replay a call list into a new
 * canvas whose reads are deferred (nothing runs on the GPU yet), and get
 * its engine context to put into a frame. */
cy_canvas *cy_canvas_from_trace(const void *trace, size_t trace_len, int *status);
void *cy_canvas_ctx(cy_canvas *c);

#ifdef __cplusplus
}
#endif

#endif /* CANVAS_ITY_C_H */
