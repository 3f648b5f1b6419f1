// hit.cuh -- batched is_point_in_path kernel.
//
// Depends on device.cuh only, so the same source also compiles as host C++
// for the CPU checks in tests/host_kernels/.
#ifndef CY_HIT_CUH
#define CY_HIT_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace cyg {

// ------------------------------------------------------------ hit testing
// is_point_in_path (hpp:3101-3132) for many query points, one thread per
// point, over the fill-mode polyline of one path.  Each point k with its
// previous-point link is the reference's segment from pts[prev[k]] to
// pts[k] (the last point of a subpath links back to its first).  The
// crossing count is an integer sum and a point on the boundary is inside
// whichever segment finds it, so the segment order does not matter.
__global__ void k_points_in_path(const float2 *__restrict__ pts, const int32_t *__restrict__ prev, int n_pts,
                                 const float2 *__restrict__ queries, int n_queries, int even_odd,
                                 unsigned char *__restrict__ inside) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_queries) return;
    const float x = queries[q].x, y = queries[q].y;
    int winding = 0;
    bool boundary = false;
    for (int k = 0; k < n_pts && !boundary; ++k) {
        float2 from = pts[prev[k]], to = pts[k];
        if ((from.y < y && y <= to.y) || (to.y < y && y <= from.y)) {
            float side = dot2(perp2(sub2(to, from)), sub2(f2(x, y), from));
            if (side == 0.0f) boundary = true;
            else winding += side > 0.0f ? 1 : -1;
        } else if (from.y == y && y == to.y && ((from.x <= x && x <= to.x) || (to.x <= x && x <= from.x))) {
            boundary = true;
        }
    }
    inside[q] = boundary || (even_odd ? (winding & 2) != 0 : winding != 0) ? 1 : 0;
}

}  // namespace cyg

#endif
