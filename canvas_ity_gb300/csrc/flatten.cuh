// flatten.cuh -- Bezier flattening kernels: one item per subpath start or cubic.
//
// Depends on device.cuh only, so the same source also compiles as host C++
// for the CPU checks in tests/host_kernels/.
#ifndef CY_FLATTEN_CUH
#define CY_FLATTEN_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace cyg {

// ------------------------------------------------------------- flattening
__global__ void k_flat_count(const float2 *__restrict__ bez, const flat_item *__restrict__ items, int n,
                             int32_t *__restrict__ counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flat_item it = items[i];
    if (it.sub_end >= 0) { counts[i] = 1; return; }
    counts[i] = flatten_cubic<false>(bez[it.pt], bez[it.pt + 1], bez[it.pt + 2], bez[it.pt + 3], it.angular, nullptr, 0);
}

__global__ void k_flat_emit(const float2 *__restrict__ bez, const flat_item *__restrict__ items, int n,
                            const int32_t *__restrict__ offs, float2 *__restrict__ pts,
                            int32_t *__restrict__ prev, int64_t cap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flat_item it = items[i];
    int o = offs[i];
    int cnt = offs[i + 1] - o;
    if (o < 0 || static_cast<int64_t>(o) + cnt > cap) return;
    if (it.sub_end >= 0) {
        pts[o] = bez[it.pt];
        prev[o] = offs[it.sub_end] - 1;   // closing segment from the subpath's last point
        return;
    }
    flatten_cubic<true>(bez[it.pt], bez[it.pt + 1], bez[it.pt + 2], bez[it.pt + 3], it.angular, pts + o, cnt);
    for (int k = 0; k < cnt; ++k) prev[o + k] = o + k - 1;
}

}  // namespace cyg

#endif
