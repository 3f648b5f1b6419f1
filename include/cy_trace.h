/*
 * cy_trace.h -- binary format of a recorded canvas_ity API call list.
 *
 * A trace is the sequence of public `canvas_ity::canvas` calls made by an
 * application (reference API: src/canvas_ity.hpp:194-1148).  The same trace
 * is replayed through three implementations: the reference header compiled
 * from its own sources, the CPU oracle under oracle/, and the GB300 canvas
 * of this library.  Their pixel outputs are then compared.
 *
 * Layout (little endian):
 *   u32 magic 'CYTR', u32 version (1), then records:
 *   i32 opcode, followed by the opcode's payload as listed below.
 *   Images are stored compactly (row stride = 4 * width).  Strings are
 *   stored without their terminator.  Public data members of the canvas
 *   (global_composite_operation, shadow_offset_x, ...) appear as SET_*
 *   records at the point where the application changed them.
 */
#ifndef CY_TRACE_H
#define CY_TRACE_H

#define CY_TRACE_MAGIC 0x52545943u /* "CYTR" */
#define CY_TRACE_VERSION 1

enum cy_trace_op {
    CYT_END = 0,
    CYT_CANVAS = 1,              /* i32 w, i32 h                          */
    CYT_SCALE = 2,               /* f x, f y                              */
    CYT_ROTATE = 3,              /* f angle                               */
    CYT_TRANSLATE = 4,           /* f x, f y                              */
    CYT_TRANSFORM = 5,           /* f a b c d e f                         */
    CYT_SET_TRANSFORM = 6,       /* f a b c d e f                         */
    CYT_SET_GLOBAL_ALPHA = 7,    /* f                                     */
    CYT_SET_COMPOSITE_OP = 8,    /* i32 (public member)                   */
    CYT_SET_SHADOW_COLOR = 9,    /* f r g b a                             */
    CYT_SET_SHADOW_OFFSET_X = 10,/* f (public member)                     */
    CYT_SET_SHADOW_OFFSET_Y = 11,/* f (public member)                     */
    CYT_SET_SHADOW_BLUR = 12,    /* f                                     */
    CYT_SET_LINE_WIDTH = 13,     /* f                                     */
    CYT_SET_LINE_CAP = 14,       /* i32 (public member)                   */
    CYT_SET_LINE_JOIN = 15,      /* i32 (public member)                   */
    CYT_SET_MITER_LIMIT = 16,    /* f                                     */
    CYT_SET_LINE_DASH_OFFSET = 17,/* f (public member)                    */
    CYT_SET_LINE_DASH = 18,      /* i32 count, i32 nonnull, f[count] if nonnull && count > 0 */
    CYT_SET_COLOR = 19,          /* i32 type, f r g b a                   */
    CYT_SET_LINEAR_GRADIENT = 20,/* i32 type, f x0 y0 x1 y1               */
    CYT_SET_RADIAL_GRADIENT = 21,/* i32 type, f x0 y0 r0 x1 y1 r1         */
    CYT_ADD_COLOR_STOP = 22,     /* i32 type, f offset r g b a            */
    CYT_SET_PATTERN = 23,        /* i32 type, i32 w, i32 h, i32 repetition, i32 nonnull,
                                    u8[w*h*4] if nonnull && w > 0 && h > 0 */
    CYT_BEGIN_PATH = 24,
    CYT_MOVE_TO = 25,            /* f x y                                 */
    CYT_CLOSE_PATH = 26,
    CYT_LINE_TO = 27,            /* f x y                                 */
    CYT_QUADRATIC_CURVE_TO = 28, /* f cx cy x y                           */
    CYT_BEZIER_CURVE_TO = 29,    /* f c1x c1y c2x c2y x y                 */
    CYT_ARC_TO = 30,             /* f vx vy x y radius                    */
    CYT_ARC = 31,                /* f x y radius a0 a1, i32 ccw           */
    CYT_RECTANGLE = 32,          /* f x y w h                             */
    CYT_FILL = 33,
    CYT_STROKE = 34,
    CYT_CLIP = 35,
    CYT_IS_POINT_IN_PATH = 36,   /* f x y, i32 expected (-1 = unknown)    */
    CYT_CLEAR_RECTANGLE = 37,    /* f x y w h                             */
    CYT_FILL_RECTANGLE = 38,     /* f x y w h                             */
    CYT_STROKE_RECTANGLE = 39,   /* f x y w h                             */
    CYT_SET_TEXT_ALIGN = 40,     /* i32 (public member)                   */
    CYT_SET_TEXT_BASELINE = 41,  /* i32 (public member)                   */
    CYT_SET_FONT = 42,           /* i32 bytes, i32 nonnull, f size, u8[bytes] if nonnull && bytes > 0 */
    CYT_FILL_TEXT = 43,          /* f x y max_width, i32 nonnull, i32 len, u8[len] */
    CYT_STROKE_TEXT = 44,        /* f x y max_width, i32 nonnull, i32 len, u8[len] */
    CYT_MEASURE_TEXT = 45,       /* i32 nonnull, i32 len, u8[len], f expected (NaN = unknown) */
    CYT_DRAW_IMAGE = 46,         /* i32 w, i32 h, i32 nonnull, f x y to_w to_h,
                                    u8[w*h*4] if nonnull && w > 0 && h > 0 */
    CYT_GET_IMAGE_DATA = 47,     /* i32 w, i32 h, i32 x, i32 y, i32 nonnull, i32 has_expected,
                                    u8[w*h*4] if has_expected            */
    CYT_PUT_IMAGE_DATA = 48,     /* i32 w, i32 h, i32 x, i32 y, i32 nonnull,
                                    u8[w*h*4] if nonnull && w > 0 && h > 0 */
    CYT_SAVE = 49,
    CYT_RESTORE = 50,
    CYT_SET_FILL_RULE = 51,      /* i32 rule: 0 nonzero, 1 even-odd (extension, no reference counterpart) */
    CYT_OP_COUNT = 52
};

#endif /* CY_TRACE_H */
