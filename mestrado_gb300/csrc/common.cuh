// Shared device helpers of the GB300 IVF-PQ engine.
//
// Keys: every selection in the engine (coarse k-min, ADC top-kl, re-rank)
// ranks 64-bit keys  (orderable(distance) << 32) | payload  where payload is
// a unique index (centroid, candidate position or re-rank slot). Ties in
// distance are therefore broken by the payload, deterministically.
//
// Arithmetic: the plain form reproduces the reference's float rounding
// (sequential/yael_needs/nn.c:113-150 with a netlib-order sgemm): every
// product and sum is rounded on its own, which the __fmul_rn / __fadd_rn
// intrinsics guarantee (they are never contracted into an FMA).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbivf {

typedef unsigned long long u64;

constexpr u64 KEY_MAX = ~0ull;

// monotone float -> uint32 (negative below positive; -0 folds onto +0)
__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t u = __float_as_uint(__fadd_rn(f, 0.0f));
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float fkey_inv(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__device__ __forceinline__ u64 make_key(float dist, uint32_t payload) {
    return ((u64)fkey(dist) << 32) | payload;
}

__device__ __forceinline__ uint32_t key_payload(u64 k) { return (uint32_t)k; }
__device__ __forceinline__ float key_dist(u64 k) { return fkey_inv((uint32_t)(k >> 32)); }

// float dot product in ascending index order, no fused multiply-add
// (the sgemm inner loop: TEMP = TEMP + A(L,I)*B(L,J))
__device__ __forceinline__ float dot_seq(const float* __restrict__ a, const float* __restrict__ b, int n) {
    float t = 0.0f;
    for (int l = 0; l < n; l++) t = __fadd_rn(t, __fmul_rn(a[l], b[l]));
    return t;
}

// float squared norm, sequential (nn.c:129-135)
__device__ __forceinline__ float norm_f_seq(const float* __restrict__ a, int n) {
    float s = 0.0f;
    for (int l = 0; l < n; l++) s = __fadd_rn(s, __fmul_rn(a[l], a[l]));
    return s;
}

// the expansion-form distance given both norms (nn.c:143-145, 85-86):
// c = (float)(norm_b + norm_a) in double, then c = (-2 * dot) + c
__device__ __forceinline__ float expansion_from(double norm_b, float norm_a, float dot) {
    float c = __double2float_rn(__dadd_rn(norm_b, (double)norm_a));
    return __fadd_rn(__fmul_rn(-2.0f, dot), c);
}

// parallel2's dist2: sum of squared differences (ivf_search.cpp:49-57)
__device__ __forceinline__ float direct_seq(const float* __restrict__ a, const float* __restrict__ b, int n) {
    float s = 0.0f;
    for (int l = 0; l < n; l++) {
        float df = __fsub_rn(a[l], b[l]);
        s = __fadd_rn(s, __fmul_rn(df, df));
    }
    return s;
}

}  // namespace gbivf
