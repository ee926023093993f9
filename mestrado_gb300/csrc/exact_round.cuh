// Exact reproduction of the reference's norm sum without FP64 throughput.
//
// The reference computes every distance-table entry's constant term as
//     c = (float)(sum_d2 + sum_c2)            (sequential/yael_needs/nn.c:143-145)
// with sum_d2 a double (the centroid's norm, accumulated in double) and
// sum_c2 a float (the residual's norm): a double add rounded to double, then
// to float -- RN32(RN64(D + f)). On GB300 FP64 runs at a small fraction of
// the FP32 rate, so the engine computes the same bits in FP32 arithmetic:
//
//   D is split once per index into hi = RN32(D) and lo = RN32(D - hi);
//   S  = RN32(hi + f) and its exact error e1 (Knuth's TwoSum);
//   t  = RN32(e1 + lo)  ~  (D + f) - S, within 2^-22 ulp(S);
//   the answer is S, or its neighbour above (t > ulp/2) or below (t < -ulp/2).
//
// When t lies within 2^-21 ulp(S) of a rounding boundary (+-ulp/2), or S is
// a power of two, zero, or extreme, the double computation decides instead
// (a case that arises about once per million entries). Both branches return
// RN32(RN64(D + f)) exactly for D >= 0, f >= 0.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gbivf {

#if defined(__CUDA_ARCH__)
GB_HD float xr_add(float a, float b) { return __fadd_rn(a, b); }
GB_HD float xr_sub(float a, float b) { return __fsub_rn(a, b); }
GB_HD uint32_t xr_bits(float x) { return __float_as_uint(x); }
GB_HD float xr_float(uint32_t u) { return __uint_as_float(u); }
GB_HD float xr_d2f(double x) { return __double2float_rn(x); }
GB_HD double xr_dadd(double a, double b) { return __dadd_rn(a, b); }
GB_HD float xr_abs(float x) { return fabsf(x); }
#else
// host build: compile with -ffp-contract=off (no fused operations)
GB_HD float xr_add(float a, float b) { return a + b; }
GB_HD float xr_sub(float a, float b) { return a - b; }
GB_HD uint32_t xr_bits(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
GB_HD float xr_float(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }
GB_HD float xr_d2f(double x) { return (float)x; }
GB_HD double xr_dadd(double a, double b) { return a + b; }
GB_HD float xr_abs(float x) { return std::fabs(x); }
#endif

// hi/lo split of a double norm, done once per index on the host
inline void split_norm(double D, float* hi, float* lo) {
    float h = (float)D;
    *hi = h;
    *lo = (float)(D - (double)h);
}

// RN32(RN64(D + f)) for D >= 0 (with its split hi, lo) and f >= 0.
// D is only read on the rare exact path: Dp points at it.
GB_HD float add_norms_rn(const double* Dp, float hi, float lo, float f) {
    const float S = xr_add(hi, f);
    const float bb = xr_sub(S, hi);
    const float e1 = xr_add(xr_sub(hi, xr_sub(S, bb)), xr_sub(f, bb));
    const float t = xr_add(e1, lo);
    const uint32_t sb = xr_bits(S);
    const uint32_t ex = sb & 0x7f800000u;
    if ((sb & 0x007fffffu) != 0u && ex >= (64u << 23) && ex <= (200u << 23)) {
        const float half = xr_float(ex - (24u << 23));  // ulp(S) / 2
        const float eps = xr_float(ex - (44u << 23));   // ulp(S) * 2^-21
        const float up = xr_sub(t, half);
        const float dn = xr_add(t, half);
        if (xr_abs(up) > eps && xr_abs(dn) > eps)
            return up > 0.0f ? xr_float(sb + 1u) : (dn < 0.0f ? xr_float(sb - 1u) : S);
    }
    return xr_d2f(xr_dadd(*Dp, (double)f));
}

#if defined(__CUDACC__)
// split_norm on the device
__device__ __forceinline__ void split_norm_dev(double D, float* hi, float* lo) {
    const float h = __double2float_rn(D);
    *hi = h;
    *lo = __double2float_rn(__dsub_rn(D, (double)h));
}

// the rounding decision of add_norms_rn, given S = RN32(hi + f) and t ~ (D + f) - S
__device__ __forceinline__ float add_norms_finish(const double* Dp, float S, float t, float f) {
    const uint32_t sb = __float_as_uint(S);
    const uint32_t ex = sb & 0x7f800000u;
    if ((sb & 0x007fffffu) != 0u && ex >= (64u << 23) && ex <= (200u << 23)) {
        const float half = __uint_as_float(ex - (24u << 23));
        const float eps = __uint_as_float(ex - (44u << 23));
        const float up = __fsub_rn(t, half);
        const float dn = __fadd_rn(t, half);
        if (fabsf(up) > eps && fabsf(dn) > eps)
            return up > 0.0f ? __uint_as_float(sb + 1u) : (dn < 0.0f ? __uint_as_float(sb - 1u) : S);
    }
    return __double2float_rn(__dadd_rn(*Dp, (double)f));
}
#endif

}  // namespace gbivf
