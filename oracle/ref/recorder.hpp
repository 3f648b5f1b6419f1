// recorder.hpp -- recording stand-in for the canvas_ity public API.
//
// TEST INFRASTRUCTURE ONLY (golden-fixture generation).  The reference's own
// test program (test/test.cpp) is compiled against this header instead of
// the library header, so that every public call the 76 reference tests make
// is recorded into a call list (include/cy_trace.h) while being forwarded to
// the real reference canvas, built from src/canvas_ity.hpp in recorder.cpp.
// The public API below mirrors src/canvas_ity.hpp:146-1148.
#ifndef CY_RECORDER_HPP
#define CY_RECORDER_HPP

#include <cstddef>
#include <vector>
// The reference's implementation section pulls these in; programs written
// against it (test/test.cpp) rely on them.
#include <algorithm>
#include <cmath>
#include <numeric>

namespace canvas_ity {

enum composite_operation {
    source_in = 1, source_copy, source_out, destination_in,
    destination_atop = 7, lighter = 10, destination_over, destination_out,
    source_atop, source_over, exclusive_or };
enum cap_style { butt, square, circle };
enum join_style { miter, bevel, rounded };
enum brush_type { fill_style, stroke_style };
enum repetition_style { repeat, repeat_x, repeat_y, no_repeat };
enum align_style { leftward, rightward, center, start = 0, ending };
enum baseline_style { alphabetic, top, middle, bottom, hanging, ideographic = 3 };

class canvas {
public:
    canvas(int width, int height);
    ~canvas();
    void scale(float x, float y);
    void rotate(float angle);
    void translate(float x, float y);
    void transform(float a, float b, float c, float d, float e, float f);
    void set_transform(float a, float b, float c, float d, float e, float f);
    void set_global_alpha(float alpha);
    composite_operation global_composite_operation;
    void set_shadow_color(float red, float green, float blue, float alpha);
    float shadow_offset_x;
    float shadow_offset_y;
    void set_shadow_blur(float level);
    void set_line_width(float width);
    cap_style line_cap;
    join_style line_join;
    void set_miter_limit(float limit);
    float line_dash_offset;
    void set_line_dash(float const *segments, int count);
    void set_color(brush_type type, float red, float green, float blue, float alpha);
    void set_linear_gradient(brush_type type, float start_x, float start_y, float end_x, float end_y);
    void set_radial_gradient(brush_type type, float start_x, float start_y, float start_radius,
                             float end_x, float end_y, float end_radius);
    void add_color_stop(brush_type type, float offset, float red, float green, float blue, float alpha);
    void set_pattern(brush_type type, unsigned char const *image, int width, int height, int stride,
                     repetition_style repetition);
    void begin_path();
    void move_to(float x, float y);
    void close_path();
    void line_to(float x, float y);
    void quadratic_curve_to(float control_x, float control_y, float x, float y);
    void bezier_curve_to(float control_1_x, float control_1_y, float control_2_x, float control_2_y,
                         float x, float y);
    void arc_to(float vertex_x, float vertex_y, float x, float y, float radius);
    void arc(float x, float y, float radius, float start_angle, float end_angle,
             bool counter_clockwise = false);
    void rectangle(float x, float y, float width, float height);
    void fill();
    void stroke();
    void clip();
    bool is_point_in_path(float x, float y);
    void clear_rectangle(float x, float y, float width, float height);
    void fill_rectangle(float x, float y, float width, float height);
    void stroke_rectangle(float x, float y, float width, float height);
    align_style text_align;
    baseline_style text_baseline;
    bool set_font(unsigned char const *font, int bytes, float size);
    void fill_text(char const *text, float x, float y, float maximum_width = 1.0e30f);
    void stroke_text(char const *text, float x, float y, float maximum_width = 1.0e30f);
    float measure_text(char const *text);
    void draw_image(unsigned char const *image, int width, int height, int stride, float x, float y,
                    float to_width, float to_height);
    void get_image_data(unsigned char *image, int width, int height, int stride, int x, int y);
    void put_image_data(unsigned char const *image, int width, int height, int stride, int x, int y);
    void save();
    void restore();

private:
    struct impl;
    impl *self;
    void sync();
    canvas(canvas const &);
    canvas &operator=(canvas const &);
};

}  // namespace canvas_ity

#endif  // CY_RECORDER_HPP
