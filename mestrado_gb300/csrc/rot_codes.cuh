// Row-rotated lookup order of the precision form of the scan.
//
// The list-centric scan's precision form sums a row's m FP16 table entries in
// FP32 in the order s = rot, rot + 1, ..., rot + m - 1 (mod m), rot =
// row_rot(the row's index in its list), instead of s = 0 .. m-1. One 16-byte
// shared load there fetches one entry for 8 queries, and the table is laid
// out sub-quantizer-minor (entry (s, c) in slot c m + s), so the 8 lanes of a
// quarter-warp -- 8 consecutive 16-byte groups of rows -- read 8 different
// sub-quantizers in every step, i.e. 8 different bank quads (m = 16 and 8):
// no bank conflicts, where the s-ordered loop met 2 to 3 per load. Only the
// approximate sums change (the rounding of a few FP32 additions); the exact
// re-score decides the returned distances. The exact form keeps the
// reference's order s = 0 .. m-1: its sums are the reference's bit for bit.
#pragma once
#include <cstdint>

namespace gbivf {

// the rotation of row `row` of a list: its 16-byte group's index mod m (a group holds 16 / m rows)
template <int M>
__device__ __forceinline__ int row_rot(int row) { return (row / (16 / M)) & (M - 1); }

// code bytes rotated: byte k of the result is byte (k + r) mod 16 of v, 0 <= r < 16
__device__ __forceinline__ uint4 rot_bytes(uint4 v, int r) {
    uint32_t w0 = v.x, w1 = v.y, w2 = v.z, w3 = v.w;
    if (r & 8) {  // two words
        uint32_t t = w0;
        w0 = w2;
        w2 = t;
        t = w1;
        w1 = w3;
        w3 = t;
    }
    if (r & 4) {  // one word
        const uint32_t t = w0;
        w0 = w1;
        w1 = w2;
        w2 = w3;
        w3 = t;
    }
    const int sh = 8 * (r & 3);
    return make_uint4(__funnelshift_r(w0, w1, sh), __funnelshift_r(w1, w2, sh), __funnelshift_r(w2, w3, sh),
                      __funnelshift_r(w3, w0, sh));
}

// 8 code bytes rotated by r, 0 <= r < 8
__device__ __forceinline__ uint2 rot_bytes(uint2 v, int r) {
    uint32_t w0 = v.x, w1 = v.y;
    if (r & 4) {
        const uint32_t t = w0;
        w0 = w1;
        w1 = t;
    }
    const int sh = 8 * (r & 3);
    return make_uint2(__funnelshift_r(w0, w1, sh), __funnelshift_r(w1, w0, sh));
}

// 4 code bytes rotated by r, 0 <= r < 4
__device__ __forceinline__ uint32_t rot_bytes(uint32_t v, int r) { return __funnelshift_r(v, v, 8 * r); }

// word i of a rotated code row held as 1, 2 or 4 words
__device__ __forceinline__ uint32_t row_word(uint32_t v, int) { return v; }
__device__ __forceinline__ uint32_t row_word(uint2 v, int i) { return i ? v.y : v.x; }
__device__ __forceinline__ uint32_t row_word(uint4 v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

}  // namespace gbivf
