// ref_replay.cpp -- C entry point that replays a call list through the
// reference canvas_ity header itself (src/canvas_ity.hpp), compiled from its
// own sources where they lie.  TEST INFRASTRUCTURE ONLY: used to pin the
// oracle (oracle/cy_oracle.cpp) and as the reference CPU arm of bench.py in
// environments where the reference sources are present.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <memory>
#include <numeric>
#include <vector>

#define canvas_ity canvas_ity_ref
#define CANVAS_ITY_IMPLEMENTATION
#include CY_REFERENCE_HEADER
#undef CANVAS_ITY_IMPLEMENTATION
#undef canvas_ity

#include "../../include/cy_replay.hpp"

namespace {
struct ref_traits {
    typedef canvas_ity_ref::canvas canvas_type;
    typedef canvas_ity_ref::brush_type brush_type;
    typedef canvas_ity_ref::composite_operation composite_operation;
    typedef canvas_ity_ref::cap_style cap_style;
    typedef canvas_ity_ref::join_style join_style;
    typedef canvas_ity_ref::repetition_style repetition_style;
    typedef canvas_ity_ref::align_style align_style;
    typedef canvas_ity_ref::baseline_style baseline_style;
    static std::unique_ptr<canvas_type> make(int w, int h) {
        return std::unique_ptr<canvas_type>(new canvas_type(w, h));
    }
    // The reference fills nonzero only.
    static bool set_fill_rule(canvas_type &, int rule) { return rule == 0; }
};
}  // namespace

extern "C" int cyr_replay(const void *trace, size_t trace_len, void *images, size_t images_cap,
                          size_t *images_len, float *results, int results_cap, int *results_len) {
    return cy_trace::replay_to_buffers<ref_traits>(trace, trace_len, images, images_cap, images_len,
                                                    results, results_cap, results_len);
}
