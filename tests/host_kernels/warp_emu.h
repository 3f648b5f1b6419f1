// warp_emu.h -- run warp-level device kernels as host C++ for CPU checks.
//
// One warp is 32 host threads that meet at every warp collective (shuffles,
// votes, __syncwarp) through a barrier; run_warps calls a kernel for warps
// 0..n-1 in turn.  The kernels only use collectives at points every lane of
// a warp reaches, which is what makes this emulation exact.  Shared arrays
// become static (one warp runs at a time, and each warp indexes its own
// slice).
#ifndef CY_WARP_EMU_H
#define CY_WARP_EMU_H
#include <cuda_runtime.h>
#include <algorithm>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>
using std::isfinite;
using std::max;
using std::min;
static inline int __float2int_rz(float v) { return static_cast<int>(v); }
static inline long long __float2ll_rn(float v) { return llrintf(v); }
extern "C" inline float __powf(float a, float b) { return powf(a, b); }
#define __launch_bounds__(x)
#define __noinline__
#undef __shared__
#define __shared__ static
static thread_local uint3 threadIdx, blockIdx;
static dim3 blockDim;
static inline void __syncthreads() {}
static std::barrier<> *g_bar = nullptr;
static long long g_slot[32];
static inline int emu_lane() { return threadIdx.x & 31; }
template <class T> static T emu_exchange(T v, int from) {
    long long b = 0;
    std::memcpy(&b, &v, sizeof(T));
    g_slot[emu_lane()] = b;
    g_bar->arrive_and_wait();
    long long r = g_slot[from];
    g_bar->arrive_and_wait();
    T out;
    std::memcpy(&out, &r, sizeof(T));
    return out;
}
template <class T> static T __shfl_sync(unsigned, T v, int src) { return emu_exchange(v, src & 31); }
template <class T> static T __shfl_up_sync(unsigned, T v, int d) {
    int l = emu_lane();
    return emu_exchange(v, l >= d ? l - d : l);
}
template <class T> static T __shfl_xor_sync(unsigned, T v, int d) { return emu_exchange(v, emu_lane() ^ d); }
static unsigned __ballot_sync(unsigned, int p) {
    g_slot[emu_lane()] = p ? 1 : 0;
    g_bar->arrive_and_wait();
    unsigned m = 0;
    for (int i = 0; i < 32; ++i)
        if (g_slot[i]) m |= 1u << i;
    g_bar->arrive_and_wait();
    return m;
}
static int __all_sync(unsigned, int p) { return __ballot_sync(~0u, p) == ~0u; }
static int __any_sync(unsigned, int p) { return __ballot_sync(~0u, p) != 0; }
static void __syncwarp(unsigned = ~0u) { g_bar->arrive_and_wait(); }
static int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
static int __ffs(unsigned x) { return __builtin_ffs(static_cast<int>(x)); }
static int atomicOr(int *p, int v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
// Kernel calls for warps 0..nwarps-1 in blocks of warps_per_block warps.
static void run_warps(int nwarps, int warps_per_block, const std::function<void()> &fn) {
    std::barrier<> bar(32);
    g_bar = &bar;
    blockDim.x = warps_per_block * 32;
    std::vector<std::thread> th;
    for (int lane = 0; lane < 32; ++lane)
        th.emplace_back([&, lane] {
            for (int w = 0; w < nwarps; ++w) {
                threadIdx.x = (w % warps_per_block) * 32 + lane;
                blockIdx.x = w / warps_per_block;
                fn();
                bar.arrive_and_wait();
            }
        });
    for (auto &t : th) t.join();
}
// Kernel calls for threads 0..n-1 in blocks of `block` threads, one at a time.
static void run_threads(int n, int block, const std::function<void()> &fn) {
    blockDim.x = block;
    for (int i = 0; i < n; ++i) {
        blockIdx.x = i / block;
        threadIdx.x = i % block;
        fn();
    }
}
#endif
