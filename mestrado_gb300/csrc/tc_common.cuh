// tcgen05 / TMA / mbarrier helpers shared by the tensor-core kernels.
//
// Operand tiles are BF16, K-major, without swizzle, in the UMMA canonical
// layout: 8-row x 16-byte core matrices, core matrices adjacent along K
// CORE_LBO bytes apart, 8-row groups CORE_SBO bytes apart.
#pragma once
#include <cstdint>

namespace gbivf {

constexpr int MM_M = 128, MM_N = 128, MM_K = 128;
constexpr int A_TILE_BYTES = MM_M * MM_K * 2;      // 32 KB of queries
constexpr int B_HALF_BYTES = MM_N * MM_K * 2;      // 32 KB: one of c_hi / c_lo
constexpr int B_TILE_BYTES = 2 * B_HALF_BYTES;     // c_hi tile then c_lo tile
constexpr uint32_t CORE_LBO = 128;                 // next core matrix along K
constexpr uint32_t CORE_SBO = 2048;                // next 8-row group
// Every mbarrier wait is bounded: it gives up after WAIT_NS nanoseconds of the global timer
// (try_wait may suspend the thread for an implementation-defined time per poll, so a poll count
// alone bounds nothing in time), or after WAIT_LIMIT polls as a backstop.
constexpr uint32_t WAIT_LIMIT = 1u << 28;
constexpr uint64_t WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// BF16 x BF16 -> F32, K-major A and B, M = 128, N = 128 (kind::f16 descriptor:
// D format bits 4-5, A/B formats bits 7-9 / 10-12, N>>3 bits 17-22, M>>4 bits 24-28)
constexpr uint32_t MMA_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(MM_N >> 3) << 17) |
                               ((uint32_t)(MM_M >> 4) << 24);

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle, sm_100 version bits
__device__ __forceinline__ uint64_t make_smem_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(CORE_LBO >> 4) << 16) |
           ((uint64_t)(CORE_SBO >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// wait for the phase with the given parity; false once *abort is set (abort may be NULL) or the
// wait runs out (WAIT_NS, WAIT_LIMIT)
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t phase, volatile int* abort) {
    const uint32_t a = smem_addr(bar);
    uint64_t t0 = 0;
    for (uint32_t i = 0; i < WAIT_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(phase)
            : "memory");
        if (done) return true;
        if ((i & 7) == 7) {
            if (abort && *abort) return false;
            const uint64_t now = globaltimer_ns();
            if (t0 == 0) t0 = now;
            else if (now - t0 > WAIT_NS) return false;
        }
    }
    return false;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) { return mbar_wait_or_abort(bar, phase, nullptr); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// element (row, k) of a K-major no-swizzle tile, in bytes (k-groups of 8 BF16)
__host__ __device__ inline uint32_t tile_offset(int row, int k) {
    return (uint32_t)(row >> 3) * CORE_SBO + (uint32_t)(k >> 3) * CORE_LBO + (uint32_t)(row & 7) * 16u +
           (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared, completing on an mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// D (TMEM) (+)= A (smem desc) x B (smem desc)^T, kind::f16, issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on an mbarrier once every tcgen05 operation issued so far by this thread completes
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane, without waiting
// (tmem_wait_ld makes every load issued so far visible)
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace gbivf
