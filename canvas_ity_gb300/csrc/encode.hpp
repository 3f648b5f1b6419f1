// encode.hpp -- image file framing around device-packed RGBA8 (host code).
//
// The device writes a file's pixel payload in place and, for PNG, one CRC-32
// and one Adler-32 partial per row (kernels.cuh k_encode, k_png_rows); this
// file writes the fixed header and footer bytes and combines the row
// partials.  The formats are the reference's own writers, byte for byte:
//   - TGA as the tiger demo writes it (demos/tiger/tiger.cpp:4336-4343):
//     18-byte header, uncompressed 32-bit BGRA, top-left origin;
//   - PNG as the test harness writes it (test/test.cpp:2415-2511): IHDR,
//     an sRGB chunk, one IDAT whose zlib stream has a stored deflate block
//     per row (filter byte 0), then IEND.
// CRC-32 (the polynomial 0xedb88320 of PNG) is linear over GF(2) in its
// register, so the register after a row is the register before it pushed
// through n zero bytes (a 32x32 bit matrix, Z) xor the row's own CRC from a
// zero register.  Adler-32 sums combine as in RFC 1950's definition.
#ifndef CY_ENCODE_HPP
#define CY_ENCODE_HPP

#include <cstddef>
#include <cstdint>
#include <cstring>

namespace cyg {
namespace encode {

enum { TGA = 0, PNG = 1 };

inline size_t tga_size(int w, int h) { return 18 + static_cast<size_t>(w) * h * 4; }
inline size_t png_size(int w, int h) { return 76 + static_cast<size_t>(h) * (6 + static_cast<size_t>(w) * 4); }
inline size_t png_row_offset(int w, int y) { return 56 + static_cast<size_t>(y) * (6 + static_cast<size_t>(w) * 4); }

struct crc_table {
    uint32_t t[256];
    crc_table() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1 ? 0xedb88320u : 0u) ^ (v >> 1);
            t[i] = v;
        }
    }
    uint32_t update(uint32_t c, const unsigned char *p, size_t n) const {
        for (size_t i = 0; i < n; ++i) c = t[(c ^ p[i]) & 0xff] ^ (c >> 8);
        return c;
    }
};

// A linear operator on the 32-bit CRC register: column i is the image of bit i.
struct gf2_op {
    uint32_t col[32];
    uint32_t apply(uint32_t v) const {
        uint32_t r = 0;
        for (int i = 0; v; ++i, v >>= 1)
            if (v & 1) r ^= col[i];
        return r;
    }
    gf2_op then(const gf2_op &b) const {   // b after this
        gf2_op r;
        for (int i = 0; i < 32; ++i) r.col[i] = b.apply(col[i]);
        return r;
    }
};

// The register pushed through n zero bytes.
inline gf2_op zeros_op(const crc_table &tab, size_t n) {
    gf2_op byte, acc;
    for (int i = 0; i < 32; ++i) {
        uint32_t v = 1u << i;
        byte.col[i] = tab.t[v & 0xff] ^ (v >> 8);
        acc.col[i] = v;
    }
    while (n) {
        if (n & 1) acc = acc.then(byte);
        byte = byte.then(byte);
        n >>= 1;
    }
    return acc;
}

inline void put_be32(unsigned char *p, uint32_t v) {
    p[0] = static_cast<unsigned char>(v >> 24);
    p[1] = static_cast<unsigned char>(v >> 16);
    p[2] = static_cast<unsigned char>(v >> 8);
    p[3] = static_cast<unsigned char>(v);
}

inline void tga_header(unsigned char *out, int w, int h) {
    const unsigned char hdr[18] = {0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                   static_cast<unsigned char>(w & 255), static_cast<unsigned char>(w >> 8),
                                   static_cast<unsigned char>(h & 255), static_cast<unsigned char>(h >> 8), 32, 40};
    std::memcpy(out, hdr, 18);
}

// PNG header and footer around rows already in out (each row's 6-byte
// stored-block prefix, filter byte included, and pixels), from the rows'
// CRC-32 (zero register) and Adler-32 partials (a = byte sum, b = sum of
// byte times its distance from the row's end, both mod 65521).
inline void png_frame(unsigned char *out, int w, int h, const uint32_t *row_crc, const uint32_t *row_a,
                      const uint32_t *row_b) {
    static const crc_table tab;
    const uint32_t idat = 6 + static_cast<uint32_t>(h) * (6 + static_cast<uint32_t>(w) * 4);
    const unsigned char sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    std::memcpy(out, sig, 8);
    const unsigned char ihdr_len[4] = {0, 0, 0, 13};
    std::memcpy(out + 8, ihdr_len, 4);
    const unsigned char ihdr[4] = {73, 72, 68, 82};
    std::memcpy(out + 12, ihdr, 4);
    put_be32(out + 16, static_cast<uint32_t>(w));
    put_be32(out + 20, static_cast<uint32_t>(h));
    const unsigned char ihdr_tail[5] = {8, 6, 0, 0, 0};
    std::memcpy(out + 24, ihdr_tail, 5);
    put_be32(out + 29, ~tab.update(~0u, out + 12, 17));
    const unsigned char srgb[13] = {0, 0, 0, 1, 115, 82, 71, 66, 0, 174, 206, 28, 233};
    std::memcpy(out + 33, srgb, 13);
    put_be32(out + 46, idat);
    const unsigned char idat_head[6] = {73, 68, 65, 84, 120, 1};
    std::memcpy(out + 50, idat_head, 6);
    uint32_t crc = tab.update(~0u, out + 50, 6);
    const gf2_op z = zeros_op(tab, 6 + static_cast<size_t>(w) * 4);
    const uint64_t n_data = 1 + static_cast<uint64_t>(w) * 4;   // filter byte + pixels
    uint64_t a = 1, b = 0;
    for (int y = 0; y < h; ++y) {
        crc = z.apply(crc) ^ row_crc[y];
        b = (b + n_data % 65521 * a + row_b[y]) % 65521;
        a = (a + row_a[y]) % 65521;
    }
    unsigned char *f = out + png_size(w, h) - 20;
    f[0] = static_cast<unsigned char>(b >> 8);
    f[1] = static_cast<unsigned char>(b);
    f[2] = static_cast<unsigned char>(a >> 8);
    f[3] = static_cast<unsigned char>(a);
    crc = tab.update(crc, f, 4);
    put_be32(f + 4, ~crc);
    const unsigned char iend[12] = {0, 0, 0, 0, 73, 69, 78, 68, 174, 66, 96, 130};
    std::memcpy(f + 8, iend, 12);
}

}  // namespace encode
}  // namespace cyg

#endif
