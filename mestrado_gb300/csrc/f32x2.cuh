// Packed FP32 pairs (PTX .f32x2, sm_100 and later): two independent FP32
// operations per instruction, each rounded to nearest like the scalar
// __fadd_rn / __fsub_rn / __fmul_rn. Unlike the scalar .rn forms, a packed
// multiply feeding a packed add IS contracted into a fused multiply-add by
// ptxas (measured on GB300), so use the packed forms only where fusion cannot
// change a result (add/sub chains, or products that are exact).
#pragma once
#include <cstdint>

namespace gbivf {

typedef unsigned long long f2_t;  // (lo = first, hi = second) FP32 pair

__device__ __forceinline__ f2_t f2_pack(float a, float b) {
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
    f2_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b) {
    f2_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
    f2_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// a * b + c, each pair fused (one rounding): for approximate arithmetic only
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
    f2_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

}  // namespace gbivf
