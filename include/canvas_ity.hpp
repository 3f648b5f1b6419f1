// canvas_ity.hpp -- drop-in GB300 implementation of the canvas_ity API.
//
// Same public interface as the reference single-header library
// (src/canvas_ity.hpp:142-1148: enums at 146-156, class canvas at 177-1148),
// so application code written against the reference compiles unchanged.
// Drawing state, path building, dashing and stroke expansion stay on the
// host; rendering (Bezier flattening of fills and clips, exact-area coverage,
// paint, compositing, clipping, shadow blur, sRGB/dither output) runs as
// hand-written sm_103a CUDA kernels on the current CUDA device.  Link with
// libcanvas_ity_gb300.so.  Defining CANVAS_ITY_IMPLEMENTATION before
// including this header is accepted and has no effect: the implementation
// lives in the shared library.
//
// Semantics follow the reference: invalid arguments are ignored, buffers
// passed in are copied, and every drawing call is observable through the
// next get_image_data.  Drawing is recorded on the host and executed on the
// GPU in call order when pixels are read or written, or when the canvas is
// destroyed.  Separate canvas instances may be used from different threads.
#ifndef CANVAS_ITY_HPP
#define CANVAS_ITY_HPP

#include <cstddef>
#include <vector>
// The reference's implementation section includes these; programs written
// against it may rely on them being available.
#include <algorithm>
#include <cmath>
#include <numeric>

namespace canvas_ity {

// Public API enums (src/canvas_ity.hpp:146-156).  The composite operation
// values encode the blend: bit 1 -> fore weight uses back alpha, bit 2 ->
// inverted, bit 4 -> back weight uses fore alpha, bit 8 -> inverted.
enum composite_operation {
    source_in = 1, source_copy, source_out, destination_in,
    destination_atop = 7, lighter = 10, destination_over, destination_out,
    source_atop, source_over, exclusive_or };
enum cap_style { butt, square, circle };
enum join_style { miter, bevel, rounded };
enum brush_type { fill_style, stroke_style };
enum repetition_style { repeat, repeat_x, repeat_y, no_repeat };
enum align_style { leftward, rightward, center, start = 0, ending };
enum baseline_style {
    alphabetic, top, middle, bottom, hanging, ideographic = 3 };
// Extension, no reference counterpart (the reference fills nonzero only).
enum fill_rule_style { nonzero, even_odd };

namespace detail { struct canvas_state; }

class canvas
{
public:
    // Lifecycle (hpp:194-210).  Sizes must be between 1 and 32768.
    canvas( int width, int height );
    ~canvas();

    // Transforms (hpp:219-294).
    void scale( float x, float y );
    void rotate( float angle );
    void translate( float x, float y );
    void transform( float a, float b, float c, float d, float e, float f );
    void set_transform( float a, float b, float c, float d, float e, float f );

    // Compositing (hpp:296-330).
    void set_global_alpha( float alpha );
    composite_operation global_composite_operation;

    // Shadows (hpp:332-383).
    void set_shadow_color( float red, float green, float blue, float alpha );
    float shadow_offset_x;
    float shadow_offset_y;
    void set_shadow_blur( float level );

    // Line styles (hpp:385-466).
    void set_line_width( float width );
    cap_style line_cap;
    join_style line_join;
    void set_miter_limit( float limit );
    float line_dash_offset;
    void set_line_dash( float const *segments, int count );

    // Fill and stroke styles (hpp:468-607).
    void set_color( brush_type type, float red, float green, float blue, float alpha );
    void set_linear_gradient( brush_type type, float start_x, float start_y,
                              float end_x, float end_y );
    void set_radial_gradient( brush_type type, float start_x, float start_y,
                              float start_radius, float end_x, float end_y,
                              float end_radius );
    void add_color_stop( brush_type type, float offset, float red, float green,
                         float blue, float alpha );
    void set_pattern( brush_type type, unsigned char const *image, int width,
                      int height, int stride, repetition_style repetition );

    // Building paths (hpp:609-776).
    void begin_path();
    void move_to( float x, float y );
    void close_path();
    void line_to( float x, float y );
    void quadratic_curve_to( float control_x, float control_y, float x, float y );
    void bezier_curve_to( float control_1_x, float control_1_y, float control_2_x,
                          float control_2_y, float x, float y );
    void arc_to( float vertex_x, float vertex_y, float x, float y, float radius );
    void arc( float x, float y, float radius, float start_angle, float end_angle,
              bool counter_clockwise = false );
    void rectangle( float x, float y, float width, float height );

    // Drawing paths (hpp:778-848).
    void fill();
    void stroke();
    void clip();
    bool is_point_in_path( float x, float y );

    // Drawing rectangles (hpp:850-920).
    void clear_rectangle( float x, float y, float width, float height );
    void fill_rectangle( float x, float y, float width, float height );
    void stroke_rectangle( float x, float y, float width, float height );

    // Drawing text (hpp:922-1026).
    align_style text_align;
    baseline_style text_baseline;
    bool set_font( unsigned char const *font, int bytes, float size );
    void fill_text( char const *text, float x, float y, float maximum_width = 1.0e30f );
    void stroke_text( char const *text, float x, float y, float maximum_width = 1.0e30f );
    float measure_text( char const *text );

    // Drawing images (hpp:1028-1067).
    void draw_image( unsigned char const *image, int width, int height, int stride,
                     float x, float y, float to_width, float to_height );

    // Pixel manipulation (hpp:1069-1124).
    void get_image_data( unsigned char *image, int width, int height, int stride,
                         int x, int y );
    void put_image_data( unsigned char const *image, int width, int height,
                         int stride, int x, int y );

    // Canvas state (hpp:1126-1145).
    void save();
    void restore();

    // Extension, no reference counterpart: the winding rule of fill(),
    // clip() and is_point_in_path() (nonzero by default, as in the
    // reference).  Strokes, text and rectangles always fill nonzero.
    void set_fill_rule( fill_rule_style rule );

    // Extension, no reference counterpart: is_point_in_path() for n points
    // (x, y pairs in xy) at once, tested on the GPU; inside[i] receives 0 or
    // 1.  Returns 0 or a negative status (see cy_gpu.h).
    int points_in_path( float const *xy, int n, unsigned char *inside );

    // Extension, no reference counterpart: 0 if every GPU operation so far
    // succeeded, else the first negative status (see cy_gpu.h).  The
    // reference API has no error channel; this lets callers detect device
    // failures (e.g. out of memory) that the silent API would hide.
    int gpu_status() const;

    // Extension, no reference counterpart: copies the premultiplied linear
    // float RGBA pixels (width*height*4 floats) after running queued work.
    // Returns 0 or a negative status.  Used to check coverage exactly.
    int read_linear( float *rgba );

    // Extension, no reference counterpart: the GPU context (cy_ctx in
    // cy_gpu.h) holding this canvas's queued work, for batched rendering of
    // many canvases in one frame (cy_batch.h).
    void *gpu_context() const;

private:
    detail::canvas_state *self;
    void sync_public_state();
    canvas( canvas const & );
    canvas &operator=( canvas const & );
};

}  // namespace canvas_ity

#endif  // CANVAS_ITY_HPP
