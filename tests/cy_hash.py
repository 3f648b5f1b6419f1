"""The reference test suite's locality-sensitive image hash.

Restates `hash_image` from the reference harness (test/test.cpp:2351-2413):
per channel, edges against the right and lower neighbours (wrapping) set
bits that are rotated by a xorshift32 stream and XORed into a 32-bit hash.
A test passes when the Hamming distance to the golden hash is at most 5
(test/test.cpp:2614-2618).
"""
import functools

import numpy as np


@functools.lru_cache(maxsize=8)
def _rolls(n: int) -> np.ndarray:
    state = 0xFFFFFFFF
    out = np.empty(n, np.uint32)
    for i in range(n):
        state ^= (state & 0x7FFFF) << 13
        state ^= state >> 17
        state ^= (state & 0x7FFFFFF) << 5
        state &= 0xFFFFFFFF
        out[i] = state >> 27
    return out


def hash_image(image: np.ndarray) -> int:
    img = np.asarray(image, np.uint8)
    h, w = img.shape[:2]
    cur = img.astype(np.int64)
    down = np.roll(cur, -1, axis=0)
    right = np.roll(cur, -1, axis=1)
    thr = np.full(4, 8, np.int64)
    thr[:3] *= 255
    a_c, a_d, a_r = cur[..., 3:4], down[..., 3:4], right[..., 3:4]
    c = np.where(np.arange(4) < 3, cur * a_c, cur)
    d = np.where(np.arange(4) < 3, down * a_d, down)
    r = np.where(np.arange(4) < 3, right * a_r, right)
    e = ((c - d > thr * 16) * 128 | (c - d > thr) * 64 | (d - c > thr * 16) * 32 | (d - c > thr) * 16 |
         (c - r > thr * 16) * 8 | (c - r > thr) * 4 | (r - c > thr * 16) * 2 | (r - c > thr) * 1)
    e = e.astype(np.uint64).reshape(-1)
    roll = _rolls(e.size).astype(np.uint64)
    rot = np.where(roll > 0, ((e << roll) | (e >> (np.uint64(32) - roll))) & np.uint64(0xFFFFFFFF), e)
    return int(np.bitwise_xor.reduce(rot.astype(np.uint32)))


def hamming(a: int, b: int) -> int:
    return bin((a ^ b) & 0xFFFFFFFF).count("1")
