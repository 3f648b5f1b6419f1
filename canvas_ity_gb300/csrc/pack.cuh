// pack.cuh -- image file packing kernels (TGA and PNG payloads, PNG row checksums).
//
// Depends on device.cuh only, so the same source also compiles as host C++
// for the CPU checks in tests/host_kernels/.
#ifndef CY_PACK_CUH
#define CY_PACK_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace cyg {

// ---------------------------------------------------------- file packing
// get_image_data's conversion (as k_get) written straight into an image
// file's layout (encode.hpp): TGA pixels as BGRA after an 18-byte header;
// PNG pixels after each row's 6-byte stored-block prefix (final flag, LEN,
// NLEN, filter byte 0) at 56 + y * (6 + 4w).  `blank`: the canvas was never
// painted (its buffer is not cleared), so every pixel is transparent black.
__global__ void k_encode(const float4 *__restrict__ bitmap, int W, int H, int blank, int w, int h, int x0, int y0,
                         int png, unsigned char *__restrict__ out) {
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= w || iy >= h) return;
    int cx = x0 + ix, cy = y0 + iy;
    float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!blank && 0 <= cx && cx < W && 0 <= cy && cy < H) c = bitmap[static_cast<size_t>(cy) * W + cx];
    uchar4 p = to_srgb8(c, cx, cy);
    if (!png) {
        unsigned char *d = out + 18 + (static_cast<size_t>(iy) * w + ix) * 4;
        d[0] = p.z;
        d[1] = p.y;
        d[2] = p.x;
        d[3] = p.w;
        return;
    }
    const size_t row = 56 + static_cast<size_t>(iy) * (6 + static_cast<size_t>(w) * 4);
    unsigned char *d = out + row + 6 + static_cast<size_t>(ix) * 4;
    d[0] = p.x;
    d[1] = p.y;
    d[2] = p.z;
    d[3] = p.w;
    if (ix == 0) {
        const unsigned size = 1 + static_cast<unsigned>(w) * 4;
        unsigned char *r = out + row;
        r[0] = iy + 1 == h ? 1 : 0;
        r[1] = static_cast<unsigned char>(size);
        r[2] = static_cast<unsigned char>(size >> 8);
        r[3] = static_cast<unsigned char>(~size);
        r[4] = static_cast<unsigned char>(~size >> 8);
        r[5] = 0;
    }
}

// Per PNG row (one thread each): the CRC-32 of its 6 + 4w bytes from a zero
// register, and the Adler-32 partials of its 1 + 4w zlib data bytes (filter
// byte and pixels): a = sum of bytes, b = sum of byte * (distance to the
// row's end), both mod 65521.
__global__ void k_png_rows(const unsigned char *__restrict__ out, int w, int h, uint32_t *__restrict__ row_crc,
                           uint32_t *__restrict__ row_a, uint32_t *__restrict__ row_b) {
    __shared__ uint32_t tab[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t v = static_cast<uint32_t>(i);
        for (int k = 0; k < 8; ++k) v = (v & 1 ? 0xedb88320u : 0u) ^ (v >> 1);
        tab[i] = v;
    }
    __syncthreads();
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= h) return;
    const size_t n = 6 + static_cast<size_t>(w) * 4;
    const unsigned char *r = out + 56 + static_cast<size_t>(y) * n;
    uint32_t c = 0;
    for (size_t k = 0; k < n; ++k) c = tab[(c ^ r[k]) & 0xff] ^ (c >> 8);
    const uint64_t nd = n - 5;   // filter byte + pixels
    uint64_t a = 0, b = 0;
    for (uint64_t j = 0; j < nd; ++j) {
        uint64_t v = r[5 + j];
        a += v;
        b += (nd - j) * v;
    }
    row_crc[y] = c;
    row_a[y] = static_cast<uint32_t>(a % 65521);
    row_b[y] = static_cast<uint32_t>(b % 65521);
}

}  // namespace cyg

#endif
