// pack_check.cpp -- CPU check of pack.cuh (k_encode, k_png_rows) with the
// framing of encode.hpp against a sequential restatement of the reference's
// PNG writer (test/test.cpp:2415-2511) and TGA writer
// (demos/tiger/tiger.cpp:4336-4343).  Prints "cases N, mismatching M".
#include "shim.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../../canvas_ity_gb300/csrc/pack.cuh"
#include "../../canvas_ity_gb300/csrc/encode.hpp"
using namespace cyg;

static std::vector<unsigned char> ref_png(const unsigned char *image, int width, int height) {
    std::vector<unsigned char> o;
    unsigned table[256];
    for (unsigned index = 0; index < 256; ++index) { unsigned value = index; for (int step = 0; step < 8; ++step) value = (value & 1 ? 0xedb88320u : 0u) ^ (value >> 1); table[index] = value; }
    int idat_size = 6 + height * (6 + width * 4);
    unsigned char header[] = {137,80,78,71,13,10,26,10, 0,0,0,13,73,72,68,82,
        (unsigned char)(width>>24),(unsigned char)(width>>16),(unsigned char)(width>>8),(unsigned char)width,
        (unsigned char)(height>>24),(unsigned char)(height>>16),(unsigned char)(height>>8),(unsigned char)height,
        8,6,0,0,0, 0,0,0,0, 0,0,0,1,115,82,71,66, 0, 174,206,28,233,
        (unsigned char)(idat_size>>24),(unsigned char)(idat_size>>16),(unsigned char)(idat_size>>8),(unsigned char)idat_size,
        73,68,65,84, 120,1};
    unsigned crc = ~0u;
    for (int i = 12; i < 29; ++i) crc = table[(crc ^ header[i]) & 0xff] ^ (crc >> 8);
    header[29] = ~crc >> 24; header[30] = ~crc >> 16; header[31] = ~crc >> 8; header[32] = ~crc;
    o.insert(o.end(), header, header + 56);
    crc = ~0u; for (int i = 50; i < 56; ++i) crc = table[(crc ^ header[i]) & 0xff] ^ (crc >> 8);
    int c1 = 1, c2 = 0, row_size = 1 + width * 4;
    for (int y = 0; y < height; ++y, image += width * 4) {
        unsigned char prefix[] = {(unsigned char)(y + 1 == height), (unsigned char)row_size, (unsigned char)(row_size >> 8), (unsigned char)~row_size, (unsigned char)~(row_size >> 8), 0};
        o.insert(o.end(), prefix, prefix + 6);
        for (int i = 0; i < 6; ++i) crc = table[(crc ^ prefix[i]) & 0xff] ^ (crc >> 8);
        o.insert(o.end(), image, image + width * 4);
        c2 = (c2 + c1) % 65521;
        for (int i = 0; i < width * 4; ++i) { c1 = (c1 + image[i]) % 65521; c2 = (c2 + c1) % 65521; crc = table[(crc ^ image[i]) & 0xff] ^ (crc >> 8); }
    }
    unsigned char footer[] = {(unsigned char)(c2>>8),(unsigned char)c2,(unsigned char)(c1>>8),(unsigned char)c1, 0,0,0,0, 0,0,0,0,73,69,78,68, 174,66,96,130};
    for (int i = 0; i < 4; ++i) crc = table[(crc ^ footer[i]) & 0xff] ^ (crc >> 8);
    footer[4] = ~crc >> 24; footer[5] = ~crc >> 16; footer[6] = ~crc >> 8; footer[7] = ~crc;
    o.insert(o.end(), footer, footer + 20);
    return o;
}
int main() {
    srand(3);
    for (int i = 0; i < 16 * 256; ++i) (&g_srgb_thr[0][0])[i] = (float)(i % 256) / 256.0f;
    long bad = 0, cases = 0;
    for (int t = 0; t < 60; ++t) {
        int W = 1 + rand() % 90, H = 1 + rand() % 70;
        std::vector<float4> bmp((size_t)W * H);
        for (auto &p : bmp) { float a = (rand() % 1000) / 999.0f; p = make_float4(a * (rand() % 1000) / 999.0f, a * (rand() % 1000) / 999.0f, a * (rand() % 1000) / 999.0f, a); }
        int x0 = rand() % 20 - 10, y0 = rand() % 20 - 10, w = 1 + rand() % 100, h = 1 + rand() % 80;
        int blank = t % 7 == 3;
        std::vector<unsigned char> rgba((size_t)w * h * 4);
        std::vector<float4> src = bmp; if (blank) for (auto &p : src) p = make_float4(0,0,0,0);
        for (int iy = 0; iy < h; ++iy) for (int ix = 0; ix < w; ++ix) {
            int cx = x0 + ix, cy = y0 + iy;
            float4 c = make_float4(0, 0, 0, 0);
            if (0 <= cx && cx < W && 0 <= cy && cy < H) c = src[(size_t)cy * W + cx];
            ((uchar4 *)rgba.data())[(size_t)iy * w + ix] = to_srgb8(c, cx, cy);
        }
        for (int png = 0; png < 2; ++png) {
            size_t size = png ? encode::png_size(w, h) : encode::tga_size(w, h);
            std::vector<unsigned char> out(size, 0xcd);
            for (int iy = 0; iy < h; ++iy) for (int ix = 0; ix < w; ++ix) {
                blockIdx = make_uint3(0,0,0); threadIdx = make_uint3(ix, iy, 0); blockDim = dim3(1 << 30, 1 << 30);
                k_encode(bmp.data(), W, H, blank, w, h, x0, y0, png, out.data());
            }
            std::vector<unsigned char> want;
            if (png) {
                std::vector<uint32_t> sums(3 * h);
                blockDim = dim3(128, 1);
                for (int pass = 0; pass < 2; ++pass)   // the first pass fills the block's table (every thread's share)
                    for (int y = 0; y < std::max(h, 128); ++y) { blockIdx = make_uint3(y / 128, 0, 0); threadIdx = make_uint3(y % 128, 0, 0); k_png_rows(out.data(), w, h, sums.data(), sums.data() + h, sums.data() + 2 * h); }
                encode::png_frame(out.data(), w, h, sums.data(), sums.data() + h, sums.data() + 2 * h);
                want = ref_png(rgba.data(), w, h);
            } else {
                encode::tga_header(out.data(), w, h);
                unsigned char hdr[] = {0,0,2,0,0,0,0,0,0,0,0,0,(unsigned char)(w & 255),(unsigned char)(w >> 8),(unsigned char)(h & 255),(unsigned char)(h >> 8),32,40};
                want.assign(hdr, hdr + 18);
                std::vector<unsigned char> px = rgba;
                for (size_t p = 0; p < (size_t)w * h; ++p) std::swap(px[p * 4], px[p * 4 + 2]);
                want.insert(want.end(), px.begin(), px.end());
            }
            ++cases;
            if (want != out) { ++bad; size_t k = 0; while (k < want.size() && k < out.size() && want[k] == out[k]) ++k; if (bad < 4) printf("mismatch png=%d %dx%d size %zu/%zu first diff at %zu: %d vs %d\n", png, w, h, want.size(), out.size(), k, k < want.size() ? want[k] : -1, k < out.size() ? out[k] : -1); }
        }
    }
    printf("cases %ld, mismatching %ld\n", cases, bad);
}
