// Mixed-precision coarse assignment on the tcgen05 tensor cores.
//
// The coarse stage of ivfpq_search is a dense nq x C x d contraction
// (knn_full over the coarse centroids, sequential/ivf_pq/ivf_search.cpp:37-38).
// Here it runs as a BF16 GEMM with FP32 accumulation in tensor memory:
//
//   * queries and centroids are converted once into BF16 tiles laid out as the
//     UMMA K-major, no-swizzle canonical form (8-row x 16-byte core matrices,
//     core matrices adjacent in K 128 bytes apart, 8-row groups 2048 bytes
//     apart); byte-valued queries are exact in BF16; each centroid is split
//     into c_hi = bf16(c) and c_lo = bf16(c - c_hi), so that c_hi + c_lo is
//     within 2^-16 |c| of c;
//   * one CTA (4 warps) per 128-query x 128-centroid tile: thread 0 stages the
//     query tile and the centroid hi/lo tiles with 1-D TMA bulk copies
//     (cp.async.bulk, mbarrier completion), issues 16 tcgen05.mma (K = 16 each:
//     q.c_hi then q.c_lo) into one 128 x 128 FP32 accumulator in TMEM and
//     commits to an mbarrier; each warp then reads its 32 TMEM lanes with
//     tcgen05.ld and writes approximate distances ||q||^2 + ||c||^2 - 2 q.c;
//   * a selection kernel finds, per query, the w-th smallest upper bound
//     approx + eps(q, c) and re-checks every centroid with approx - eps <= that
//     bound in the reference's exact FP32 arithmetic; the exact keyed top-w of
//     those is the plain path's result, bit for bit.
//
// eps(q, c) = MIXED_EPS_REL * ||q|| * ||c|| + 2^-20 (||q||^2 + ||c||^2) bounds the
// distance error: the hi/lo split (|sum q_l (c~_l - c_l)| <= 2^-16 ||q|| ||c||),
// an FP32 accumulator allowed to lose 4 ulps (2^-21) per addition over the
// 2K = 256 products (every product of two BF16 values is exact in FP32),
// doubled for the -2 q.c term and with a factor 2 of slack; the second term
// covers the FP32 epilogue.
//
// Every wait is bounded: on a timeout the CTA sets an error flag, frees its
// TMEM and returns, and the host reports the error.
#include <cuda_bf16.h>

#include <algorithm>

#include "block_topk.cuh"
#include "kernels.cuh"
#include "tc_common.cuh"

namespace gbivf {

// rows of x (n x 128 float) -> BF16 tiles of `rows_per_tile` rows; rows past n are zero
__global__ void bf16_tiles_kernel(const float* __restrict__ x, int n, int rows_per_tile, int padded,
                                  uint8_t* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)padded * 16) return;
    const int row = (int)(idx >> 4), kg = (int)(idx & 15);
    const int tile = row / rows_per_tile, r = row % rows_per_tile;
    __align__(16) __nv_bfloat16 v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __float2bfloat16_rn(row < n ? x[(int64_t)row * MM_K + kg * 8 + i] : 0.0f);
    uint8_t* dst = out + (int64_t)tile * rows_per_tile * MM_K * 2 + tile_offset(r, kg * 8);
    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(v);
}

// centroids (n x 128 float) -> per MM_N-row tile: the c_hi tile, then the c_lo tile
__global__ void bf16_split_tiles_kernel(const float* __restrict__ x, int n, int padded, uint8_t* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)padded * 16) return;
    const int row = (int)(idx >> 4), kg = (int)(idx & 15);
    const int tile = row / MM_N, r = row % MM_N;
    __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const float v = row < n ? x[(int64_t)row * MM_K + kg * 8 + i] : 0.0f;
        hi[i] = __float2bfloat16_rn(v);
        lo[i] = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi[i])));
    }
    uint8_t* base = out + (int64_t)tile * B_TILE_BYTES + tile_offset(r, kg * 8);
    *reinterpret_cast<uint4*>(base) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(base + B_HALF_BYTES) = *reinterpret_cast<const uint4*>(lo);
}

// out != NULL: approximate distances, nq x C row-major. amin != NULL instead:
// per (row, centroid tile) the smallest (distance, centroid) key, nq x gridDim.x.
// flt.thr != NULL instead: per row, centroids with approx - eps <= thr are
// appended to the row's candidates and those with approx + eps <= thr counted.
__global__ void __launch_bounds__(128) coarse_mma_kernel(const uint8_t* __restrict__ qtiles,
                                                         const uint8_t* __restrict__ ctiles, int nq, int C,
                                                         const double* __restrict__ qnorm,
                                                         const float* __restrict__ cnorm, float* __restrict__ out,
                                                         unsigned long long* __restrict__ amin, CoarseFilter flt,
                                                         int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + A_TILE_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + A_TILE_BYTES + B_TILE_BYTES);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ct = blockIdx.x, qt = blockIdx.y;

    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"((uint32_t)MM_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (tid == 0) {
        const uint32_t bytes = A_TILE_BYTES + B_TILE_BYTES;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&bars[0])), "r"(bytes)
                     : "memory");
        const uint8_t* ga = qtiles + (int64_t)qt * A_TILE_BYTES;
        const uint8_t* gb = ctiles + (int64_t)ct * B_TILE_BYTES;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(sA)),
            "l"(ga), "r"((uint32_t)A_TILE_BYTES), "r"(smem_addr(&bars[0]))
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(sB)),
            "l"(gb), "r"((uint32_t)B_TILE_BYTES), "r"(smem_addr(&bars[0]))
            : "memory");
    }
    bool ok = mbar_wait(&bars[0], 0);
    ok = __syncthreads_and(ok);
    if (ok && tid == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB);
        // q.c_hi over K (8 steps of 16), then q.c_lo accumulated on top
#pragma unroll
        for (int step = 0; step < 2 * (MM_K / 16); step++) {
            const int k = step % (MM_K / 16), half = step / (MM_K / 16);
            const uint64_t ad = make_smem_desc(a0 + k * 2 * CORE_LBO);
            const uint64_t bd = make_smem_desc(b0 + half * B_HALF_BYTES + k * 2 * CORE_LBO);
            const uint32_t acc = step > 0 ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(MMA_IDESC), "r"(acc)
                : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(&bars[1]))
                     : "memory");
    }
    if (ok) ok = mbar_wait(&bars[1], 0);
    ok = __syncthreads_and(ok);
    tc_fence_after();
    if (ok) {
        const int row = qt * MM_M + warp * 32 + lane;
        const float qn = row < nq ? (float)qnorm[row] : 0.0f;
        const float qlen = sqrtf(qn);
        const float T = (flt.thr && row < nq) ? flt.thr[row] : 0.0f;
        int below = 0;
        u64 best = KEY_MAX;
#pragma unroll 1
        for (int ch = 0; ch < MM_N / 32; ch++) {
            uint32_t r[32];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(ch * 32);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int c0 = ct * MM_N + ch * 32;
            if (amin) {
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    if (c0 + j < C) {
                        const u64 key =
                            make_key(qn + cnorm[c0 + j] - 2.0f * __uint_as_float(r[j]), (uint32_t)(c0 + j));
                        best = key < best ? key : best;
                    }
                }
            } else if (flt.thr) {
                if (row < nq) {
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const int c = c0 + j;
                        if (c < C) {
                            const float cn = cnorm[c];
                            const float a = qn + cn - 2.0f * __uint_as_float(r[j]);
                            const float e = mixed_eps(qn, qlen, cn, flt.clen[c]);
                            below += (a + e <= T) ? 1 : 0;
                            if (a - e <= T) {
                                const int slot = atomicAdd(&flt.ncand[row], 1);
                                if (slot < flt.cap) flt.cand[(int64_t)row * flt.cap + slot] = c;
                            }
                        }
                    }
                }
            } else if (row < nq) {
                float* o = out + (int64_t)row * C + c0;
                if (c0 + 32 <= C && (C & 3) == 0) {
#pragma unroll
                    for (int j = 0; j < 32; j += 4) {
                        float4 v;
                        v.x = qn + cnorm[c0 + j] - 2.0f * __uint_as_float(r[j]);
                        v.y = qn + cnorm[c0 + j + 1] - 2.0f * __uint_as_float(r[j + 1]);
                        v.z = qn + cnorm[c0 + j + 2] - 2.0f * __uint_as_float(r[j + 2]);
                        v.w = qn + cnorm[c0 + j + 3] - 2.0f * __uint_as_float(r[j + 3]);
                        *reinterpret_cast<float4*>(o + j) = v;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (c0 + j < C) o[j] = qn + cnorm[c0 + j] - 2.0f * __uint_as_float(r[j]);
                }
            }
        }
        if (amin && row < nq) amin[(int64_t)row * gridDim.x + ct] = best;
        if (flt.thr && row < nq && below) atomicAdd(&flt.cnt[row], below);
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)MM_N)
                     : "memory");
}

// Per query: U = w-th smallest (approx + eps); exact re-check of every centroid
// with approx - eps <= U; exact keyed top-w of those.
constexpr int MS_NT = 128;

__global__ void __launch_bounds__(MS_NT) coarse_recheck_kernel(const float* __restrict__ approx, int C, int w,
                                                               int kcap, int bcap, const float* __restrict__ q,
                                                               const double* __restrict__ qnorm,
                                                               const float* __restrict__ coa,
                                                               const float* __restrict__ cnorm,
                                                               const float* __restrict__ clen, int32_t* __restrict__ coaidx,
                                                               float* __restrict__ coadis, int* __restrict__ ncand) {
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem);
    u64* tmp = best + kcap;
    u64* buf = tmp + kcap;
    u64* thresh = buf + bcap;
    unsigned char* work = reinterpret_cast<unsigned char*>(thresh + 1);
    int* cnt = reinterpret_cast<int*>(work + TOPK_WORK_BYTES);
    float* xq = reinterpret_cast<float*>(cnt + 4);
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, bcap, work};
    const int qi = blockIdx.x, tid = threadIdx.x;
    const float* row = approx + (int64_t)qi * C;
    const double qn = qnorm[qi];
    const float qlen = sqrtf((float)qn);
    for (int x = tid; x < MM_K; x += MS_NT) xq[x] = q[(int64_t)qi * MM_K + x];
    auto eps_of = [&](int c) { return mixed_eps((float)qn, qlen, cnorm[c], clen[c]); };
    // pass 1: the w-th smallest upper bound
    topk_init(s, w);
    for (int i0 = 0; i0 < C; i0 += MS_NT * 8) {
#pragma unroll
        for (int it = 0; it < 8; it++) {
            const int c = i0 + it * MS_NT + tid;
            const bool valid = c < C;
            const float up = valid ? row[c] + eps_of(c) : 0.0f;
            topk_offer(s, make_key(up, (uint32_t)c), valid);
        }
        topk_round_end(s, MS_NT * 8);
    }
    topk_finish(s);
    const float U = key_dist(best[w - 1]);
    __syncthreads();
    // pass 2: exact distances of the candidates (nn.c:143-145 + 85-86)
    topk_init(s, w);
    int mine = 0;
    for (int i0 = 0; i0 < C; i0 += MS_NT) {
        const int c = i0 + tid;
        bool cand = false;
        float dist = 0.0f;
        if (c < C && row[c] - eps_of(c) <= U) {
            cand = true;
            mine++;
            dist = expansion_from(qn, cnorm[c], dot_seq(coa + (int64_t)c * MM_K, xq, MM_K));
        }
        topk_offer(s, make_key(dist, (uint32_t)c), cand);
        topk_round_end(s, MS_NT);
    }
    topk_finish(s);
    for (int j = tid; j < w; j += MS_NT) {
        coaidx[(int64_t)qi * w + j] = (int32_t)key_payload(best[j]);
        coadis[(int64_t)qi * w + j] = key_dist(best[j]);
    }
    if (ncand) atomicAdd(ncand, mine);
}

cudaError_t launch_bf16_tiles(const float* x, int n, int rows_per_tile, uint8_t* out, cudaStream_t st) {
    const int tiles = (n + rows_per_tile - 1) / rows_per_tile;
    const int padded = tiles * rows_per_tile;
    const int64_t work = (int64_t)padded * 16;
    if (work == 0) return cudaSuccess;
    bf16_tiles_kernel<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(x, n, rows_per_tile, padded, out);
    return cudaGetLastError();
}

cudaError_t launch_bf16_split_tiles(const float* x, int n, uint8_t* out, cudaStream_t st) {
    const int padded = (n + MM_N - 1) / MM_N * MM_N;
    const int64_t work = (int64_t)padded * 16;
    if (work == 0) return cudaSuccess;
    bf16_split_tiles_kernel<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(x, n, padded, out);
    return cudaGetLastError();
}

size_t coarse_mma_tile_bytes(int n, bool centroids) {
    if (centroids) return (size_t)((n + MM_N - 1) / MM_N) * B_TILE_BYTES;
    return (size_t)((n + MM_M - 1) / MM_M) * A_TILE_BYTES;
}

cudaError_t launch_coarse_mma(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C, const double* qnorm,
                              const float* cnorm, float* out, int* err, cudaStream_t st,
                              unsigned long long* amin) {
    if (nq <= 0) return cudaSuccess;
    const size_t sm = A_TILE_BYTES + B_TILE_BYTES + 64;
    cudaError_t e = cudaFuncSetAttribute(coarse_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 grid((C + MM_N - 1) / MM_N, (nq + MM_M - 1) / MM_M);
    coarse_mma_kernel<<<grid, 128, sm, st>>>(qtiles, ctiles, nq, C, qnorm, cnorm, amin ? nullptr : out, amin,
                                              CoarseFilter{}, err);
    return cudaGetLastError();
}

cudaError_t launch_coarse_mma_filter(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                     const double* qnorm, const float* cnorm, const CoarseFilter& f, int* err,
                                     cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    if (!f.thr || !f.cnt || !f.ncand || !f.cand || !f.clen || f.cap <= 0) return cudaErrorInvalidValue;
    const size_t sm = A_TILE_BYTES + B_TILE_BYTES + 64;
    cudaError_t e = cudaFuncSetAttribute(coarse_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 grid((C + MM_N - 1) / MM_N, (nq + MM_M - 1) / MM_M);
    coarse_mma_kernel<<<grid, 128, sm, st>>>(qtiles, ctiles, nq, C, qnorm, cnorm, nullptr, nullptr, f, err);
    return cudaGetLastError();
}

int coarse_mma_ctiles(int C) { return (C + MM_N - 1) / MM_N; }

cudaError_t launch_coarse_recheck(const float* approx, int nq, int C, int w, const float* q, const double* qnorm,
                                  const float* coa, const float* cnorm, const float* clen, int32_t* coaidx,
                                  float* coadis, int* ncand, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    int kcap = 2;
    while (kcap < w) kcap <<= 1;
    int bcap = 2048;
    while (bcap < kcap) bcap <<= 1;
    const size_t sm = sizeof(u64) * (2 * kcap + bcap + 1) + TOPK_WORK_BYTES + 4 * sizeof(int) + MM_K * sizeof(float);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(coarse_recheck_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    coarse_recheck_kernel<<<nq, MS_NT, sm, st>>>(approx, C, w, kcap, bcap, q, qnorm, coa, cnorm, clen, coaidx, coadis,
                                                  ncand);
    return cudaGetLastError();
}

}  // namespace gbivf
