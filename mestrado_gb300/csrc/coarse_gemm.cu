// Persistent, warp-specialised tcgen05 GEMM of the mixed coarse stage.
//
// Same product as coarse_mma.cu (BF16 query tiles x split-BF16 centroid
// tiles, FP32 accumulators in TMEM; its error bound applies unchanged), laid
// out for throughput:
//
//   * one CTA per SM, 10 warps; a work item is 256 queries (two 128-row tiles,
//     resident in shared memory) against a contiguous range of 128-centroid
//     tiles; items are ordered so that the CTAs running at the same time share
//     a centroid range (centroid tiles are read from HBM about once and served
//     from L2 to the other query tiles);
//   * warp 8 streams the centroid tiles (c_hi then c_lo, 64 KB) through a
//     2-stage shared-memory ring with 1-D TMA bulk copies and mbarriers;
//   * warp 9 issues, per centroid tile, 2 x 16 tcgen05.mma (K = 16 each) into
//     one of two double-buffered pairs of 128 x 128 FP32 accumulators (all 512
//     TMEM columns) and commits to the ring's and the accumulators' barriers;
//   * warps 0-7 (two per TMEM lane quadrant, one per 64-column half) drain
//     the other accumulator pair meanwhile. Store mode writes approximate
//     distances. Chunk-minimum mode writes, per query and 32 centroids, the
//     smallest upper bound approx + eps (the sample of the filtered stage).
//     Argmin mode keeps, per query, the nearest centroid of its range (index
//     building). Filter mode tests each (query, centroid) against the query's bound T
//     with a three-operation pre-test, acc >= G_c - ||q|| K_c + H_q, the
//     candidate test a - eps <= T solved for the accumulator (G_c = ||c||^2
//     (1 - 2^-20) / 2, K_c = MIXED_EPS_REL ||c|| / 2, H_q from ||q||^2 and T
//     with a margin for rounding), so it is conservative by construction.
//     Its rare survivors are written, without atomics, to a region owned by
//     the thread (query, centroid range, column half); the exact candidate
//     and count tests run on them in the candidate kernel (coarse_filter.cu).
//
// Every wait is bounded and also gives up once another warp has failed; a
// failing CTA sets the error flag, lets its copies and MMAs in flight finish,
// frees its TMEM and returns.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"
#include "tc_common.cuh"

namespace gbivf {

constexpr int PG_QT = 2;                                 // resident query tiles (256 queries)
constexpr int PG_STAGES = 2;                             // centroid-tile ring and accumulator pairs
constexpr int PG_EPI_WARPS = 8;                          // two per TMEM lane quadrant (column halves)
constexpr int PG_LOAD_WARP = PG_EPI_WARPS, PG_MMA_WARP = PG_EPI_WARPS + 1;
constexpr int PG_THREADS = 32 * (PG_EPI_WARPS + 2);
constexpr uint32_t PG_TMEM_COLS = PG_STAGES * PG_QT * MM_N;  // 512
constexpr size_t PG_SMEM = (size_t)PG_QT * A_TILE_BYTES + (size_t)PG_STAGES * B_TILE_BYTES + 256 +
                           (size_t)PG_EPI_WARPS * 128 * sizeof(float);

struct PgArgs {
    const uint8_t* qtiles = nullptr;  // 2 * nqp query tiles
    const uint8_t* ctiles = nullptr;  // nct centroid hi/lo tiles
    int nq = 0, C = 0, nqp = 0, nct = 0, nsplit = 1, split_tiles = 1;
    const double* qnorm = nullptr;
    const float* cnorm = nullptr;
    float* out = nullptr;  // store: nq x ld approximate distances; chunk-min: nq x ld (ld >= C / 32)
    int64_t ld = 0;
    unsigned long long* amin = nullptr;  // argmin: per (query, centroid range, column half) the best key
    bool hi_only = false;                // argmin: c_hi tiles only (bf16 centroids; index building)
    CoarseFilter f;                // filter mode
    const float* colG = nullptr;   // nct * 128: ||c||^2 (1 - 2^-20) / 2, +inf past C
    const float* colK = nullptr;   // nct * 128: MIXED_EPS_REL ||c|| / 2, 0 past C
    float cn_max = 0.0f, clen_max = 0.0f;
    int* err = nullptr;
    // self-test of the bounded waits: the first centroid-tile copy is never issued, so the MMA
    // warp's wait for it runs out; the kernel must report the error and leave the context usable
    bool stall_copy = false;
};

enum PgMode { PG_STORE = 0, PG_CHUNKMIN = 1, PG_FILTER = 2, PG_ARGMIN = 3 };

// work item -> (query pair, first tile, end tile); items sharing a centroid range are adjacent
__device__ __forceinline__ void pg_item(const PgArgs& p, int it, int& qp, int& t0, int& t1) {
    const int sp = it / p.nqp;
    qp = it % p.nqp;
    t0 = sp * p.split_tiles;
    t1 = min(p.nct, t0 + p.split_tiles);
}

// 32 accumulator columns (centroids c0 .. c0+31) of one query row. gs: the
// warp's column terms for these columns (store: ||c||^2; chunk-min: G then K,
// gk_stride floats apart; filter: t_c = G_c - qlen_w K_c)
template <int MODE>
__device__ __forceinline__ void pg_chunk(const PgArgs& p, const uint32_t (&r)[32], const float* gs, int gk_stride,
                                         int c0, int row, float qn, float qlen, float h, int2* sv, int& nsv,
                                         float& bv, int& bi) {
    if (MODE == PG_FILTER) {
        // gs holds t_c = G_c - qlen_w K_c with qlen_w >= this row's ||q|| (the warp's largest), so
        // acc - t_c >= h is implied by the row's exact candidate test; survivors (rare) go to this
        // thread's region with plain stores, the exact tests run in the candidate kernel. The 32
        // columns are first reduced to their largest acc - t_c (a subtract and a max per pair), and
        // only a chunk holding a survivor is tested pair by pair.
        float mx = -__int_as_float(0x7f800000);
#pragma unroll
        for (int q4 = 0; q4 < 8; q4++) {
            const float4 t = reinterpret_cast<const float4*>(gs)[q4];
            mx = fmaxf(mx, __uint_as_float(r[4 * q4 + 0]) - t.x);
            mx = fmaxf(mx, __uint_as_float(r[4 * q4 + 1]) - t.y);
            mx = fmaxf(mx, __uint_as_float(r[4 * q4 + 2]) - t.z);
            mx = fmaxf(mx, __uint_as_float(r[4 * q4 + 3]) - t.w);
        }
        if (mx >= h) {
#pragma unroll
            for (int q4 = 0; q4 < 8; q4++) {
                const float4 t = reinterpret_cast<const float4*>(gs)[q4];
                const float tv[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float acc = __uint_as_float(r[4 * q4 + e]);
                    if (acc - tv[e] >= h) {
                        sv[min(nsv, p.f.sreg - 1)] = make_int2(c0 + 4 * q4 + e, (int)r[4 * q4 + e]);
                        nsv++;
                    }
                }
            }
        }
    } else if (MODE == PG_ARGMIN) {
        // nearest centroid: ||c||^2 - 2 acc decides it (||q||^2 is the row's constant); ties keep
        // the lower index (columns come in ascending order)
#pragma unroll
        for (int q4 = 0; q4 < 8; q4++) {
            const float4 cn = reinterpret_cast<const float4*>(gs)[q4];
            const float cv[4] = {cn.x, cn.y, cn.z, cn.w};
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float v = __fmaf_rn(-2.0f, __uint_as_float(r[4 * q4 + e]), cv[e]);
                const bool better = v < bv && c0 + 4 * q4 + e < p.C;
                bv = better ? v : bv;
                bi = better ? c0 + 4 * q4 + e : bi;
            }
        }
    } else if (MODE == PG_CHUNKMIN) {
        // min over the chunk of G + ||q|| K - acc = (upper bound - ||q||^2 (1 + 2^-20)) / 2, roughly;
        // only the filter's bound is derived from it, and any bound gives exact results
        float m = __int_as_float(0x7f800000);
#pragma unroll
        for (int q4 = 0; q4 < 8; q4++) {
            const float4 g = reinterpret_cast<const float4*>(gs)[q4];
            const float4 k = reinterpret_cast<const float4*>(gs + gk_stride)[q4];
            m = fminf(m, __fmaf_rn(qlen, k.x, g.x) - __uint_as_float(r[4 * q4 + 0]));
            m = fminf(m, __fmaf_rn(qlen, k.y, g.y) - __uint_as_float(r[4 * q4 + 1]));
            m = fminf(m, __fmaf_rn(qlen, k.z, g.z) - __uint_as_float(r[4 * q4 + 2]));
            m = fminf(m, __fmaf_rn(qlen, k.w, g.w) - __uint_as_float(r[4 * q4 + 3]));
        }
        if (row < p.nq) p.out[(int64_t)row * p.ld + (c0 >> 5)] = __fmaf_rn(2.0f, m, qn * (1.0f + 9.5367431640625e-07f));
    } else if (row < p.nq) {
        float* o = p.out + (int64_t)row * p.ld + c0;
        if (c0 + 32 <= p.C && (p.ld & 3) == 0) {
#pragma unroll
            for (int e = 0; e < 32; e += 4) {
                const float4 cn = reinterpret_cast<const float4*>(gs)[e / 4];
                float4 v;
                v.x = qn + cn.x - 2.0f * __uint_as_float(r[e]);
                v.y = qn + cn.y - 2.0f * __uint_as_float(r[e + 1]);
                v.z = qn + cn.z - 2.0f * __uint_as_float(r[e + 2]);
                v.w = qn + cn.w - 2.0f * __uint_as_float(r[e + 3]);
                *reinterpret_cast<float4*>(o + e) = v;
            }
        } else {
#pragma unroll
            for (int e = 0; e < 32; e++)
                if (c0 + e < p.C) o[e] = qn + p.cnorm[c0 + e] - 2.0f * __uint_as_float(r[e]);
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(PG_THREADS, 1) coarse_gemm_kernel(PgArgs p) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + PG_QT * A_TILE_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + PG_STAGES * B_TILE_BYTES);
    uint64_t* b_full = bars;      // [PG_STAGES] centroid tile landed
    uint64_t* b_empty = bars + 2; // [PG_STAGES] its MMAs are done
    uint64_t* t_full = bars + 4;  // [PG_STAGES] accumulator pair ready
    uint64_t* t_empty = bars + 6; // [PG_STAGES] accumulator pair drained (every epilogue warp)
    uint64_t* a_full = bars + 8;
    uint64_t* a_empty = bars + 9;
    uint64_t* drain = bars + 10;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 12);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 13);
    float* gsm = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(bars) + 256);  // [PG_EPI_WARPS][128]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nitems = p.nqp * p.nsplit;

    if (tid == 0) {
        for (int s = 0; s < PG_STAGES; s++) {
            mbar_init(&b_full[s], 1);
            mbar_init(&b_empty[s], 1);
            mbar_init(&t_full[s], 1);
            mbar_init(&t_empty[s], PG_EPI_WARPS);
        }
        mbar_init(a_full, 1);
        mbar_init(a_empty, 1);
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(PG_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == PG_LOAD_WARP) {
        // ---------------- loads ----------------
        if (lane == 0) {
            bool ok = true;
            int ua = 0, tc = 0, armed_a = -1;
            int armed_b[PG_STAGES];
            for (int s = 0; s < PG_STAGES; s++) armed_b[s] = -1;
            for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
                int qp, t0, t1;
                pg_item(p, it, qp, t0, t1);
                if (t0 >= t1) continue;
                if (!mbar_wait_or_abort(a_empty, (ua & 1) ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(a_full, PG_QT * A_TILE_BYTES);
                bulk_load(sA, p.qtiles + (int64_t)qp * PG_QT * A_TILE_BYTES, PG_QT * A_TILE_BYTES, a_full);
                armed_a = ua++;
                for (int t = t0; t < t1; t++, tc++) {
                    const int s = tc % PG_STAGES, u = tc / PG_STAGES;
                    if (!mbar_wait_or_abort(&b_empty[s], (u & 1) ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    if (p.stall_copy && tc == 0) continue;  // self-test only: b_full[0] never completes
                    const uint32_t bbytes = p.hi_only ? B_HALF_BYTES : B_TILE_BYTES;
                    mbar_expect_tx(&b_full[s], bbytes);
                    bulk_load(sB + s * B_TILE_BYTES, p.ctiles + (int64_t)t * B_TILE_BYTES, bbytes, &b_full[s]);
                    armed_b[s] = u;
                }
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                // let the copies in flight land before the CTA leaves
                for (int s = 0; s < PG_STAGES; s++)
                    if (armed_b[s] >= 0) mbar_wait_or_abort(&b_full[s], armed_b[s] & 1, nullptr);
                if (armed_a >= 0) mbar_wait_or_abort(a_full, armed_a & 1, nullptr);
            }
        }
    } else if (warp == PG_MMA_WARP) {
        // ---------------- MMA issue ----------------
        if (lane == 0) {
            bool ok = true, issued = false;
            int ua = 0, tc = 0;
            for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
                int qp, t0, t1;
                pg_item(p, it, qp, t0, t1);
                if (t0 >= t1) continue;
                if (!mbar_wait_or_abort(a_full, ua & 1, abort_flag)) {
                    ok = false;
                    break;
                }
                ua++;
                for (int t = t0; t < t1; t++, tc++) {
                    const int s = tc % PG_STAGES, u = tc / PG_STAGES;
                    if (!mbar_wait_or_abort(&b_full[s], u & 1, abort_flag) ||
                        !mbar_wait_or_abort(&t_empty[s], (u & 1) ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t b0 = smem_addr(sB + s * B_TILE_BYTES);
#pragma unroll
                    for (int j = 0; j < PG_QT; j++) {
                        const uint32_t d = tmem + (uint32_t)((s * PG_QT + j) * MM_N);
                        const uint32_t a0 = smem_addr(sA + j * A_TILE_BYTES);
                        const int steps = p.hi_only ? MM_K / 16 : 2 * (MM_K / 16);
#pragma unroll
                        for (int step = 0; step < 2 * (MM_K / 16); step++) {
                            if (step >= steps) break;
                            const int k = step % (MM_K / 16), half = step / (MM_K / 16);
                            mma_bf16(d, make_smem_desc(a0 + k * 2 * CORE_LBO),
                                     make_smem_desc(b0 + half * B_HALF_BYTES + k * 2 * CORE_LBO), MMA_IDESC,
                                     step > 0 ? 1u : 0u);
                        }
                    }
                    issued = true;
                    mma_commit(&b_empty[s]);
                    mma_commit(&t_full[s]);
                }
                if (!ok) break;
                mma_commit(a_empty);
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
            }
            if (issued) {  // every MMA retired before TMEM is freed
                mma_commit(drain);
                mbar_wait_or_abort(drain, 0, nullptr);
            }
        }
    } else {
        // ---------------- epilogue: TMEM lane quadrant warp % 4, columns 64 * (warp / 4) .. +63 ----------------
        const int qd = warp & 3, hf = warp >> 2;
        float* gs = gsm + warp * 128;  // this warp's 64 column terms (G, or ||c||^2 in store mode), then 64 K
        bool ok = true;
        int tc = 0;
        for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
            int qp, t0, t1;
            pg_item(p, it, qp, t0, t1);
            if (t0 >= t1) continue;
            int row[PG_QT];
            float qn[PG_QT], qlen[PG_QT], T[PG_QT], h[PG_QT];
#pragma unroll
            for (int j = 0; j < PG_QT; j++) {
                row[j] = qp * (PG_QT * MM_M) + j * MM_M + qd * 32 + lane;
                const bool valid = row[j] < p.nq;
                qn[j] = (valid && MODE != PG_ARGMIN) ? (float)p.qnorm[row[j]] : 0.0f;
                qlen[j] = sqrtf(qn[j]);
                T[j] = 0.0f;
                h[j] = __int_as_float(0x7f800000);
                if (MODE == PG_FILTER && valid) {
                    T[j] = p.f.thr[row[j]];
                    // a - eps <= T, with a = ||q||^2 + ||c||^2 - 2 acc and eps as in mixed_eps, is
                    // acc >= G_c - ||q|| K_c + (||q||^2 (1 - 2^-20) - T) / 2 in real arithmetic; delta
                    // (relative 2^-16 of the magnitudes involved) covers the roundings of both sides
                    const float emax = mixed_eps(qn[j], qlen[j], p.cn_max, p.clen_max);
                    const float delta = 1.52587890625e-05f * (fabsf(qn[j]) + p.cn_max + fabsf(T[j]) + emax);
                    h[j] = (qn[j] * (1.0f - 9.5367431640625e-07f) - T[j] - delta) * 0.5f;
                }
            }
            // this thread's survivor regions (filter): query row[j], centroid range sp, column half hf
            const int sp = it / p.nqp;
            int2* sv[PG_QT];
            int nsv[PG_QT];
            float bv[PG_QT];  // argmin: best ||c||^2 - 2 acc and its centroid
            int bi[PG_QT];
#pragma unroll
            for (int j = 0; j < PG_QT; j++) {
                bv[j] = __int_as_float(0x7f800000);
                bi[j] = 0;
                nsv[j] = 0;
                sv[j] = (MODE == PG_FILTER && row[j] < p.nq)
                            ? p.f.surv + (((int64_t)row[j] * p.nsplit + sp) * 2 + hf) * p.f.sreg
                            : nullptr;
            }
            // the warp's largest ||q|| over its rows of both tiles (filter pre-test)
            float qlen_w = fmaxf(qlen[0], qlen[PG_QT - 1]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) qlen_w = fmaxf(qlen_w, __shfl_xor_sync(0xffffffffu, qlen_w, o));
            for (int t = t0; t < t1; t++, tc++) {
                const int s = tc % PG_STAGES, u = tc / PG_STAGES;
                // this warp's 64 column terms, fetched before the wait
                const int cb = t * MM_N + hf * 64;
                float2 gv, kv = make_float2(0.0f, 0.0f);
                if (MODE == PG_CHUNKMIN || MODE == PG_FILTER) {
                    gv = __ldg(reinterpret_cast<const float2*>(p.colG + cb) + lane);
                    kv = __ldg(reinterpret_cast<const float2*>(p.colK + cb) + lane);
                } else if (cb + 2 * lane + 1 < p.C) {
                    gv = __ldg(reinterpret_cast<const float2*>(p.cnorm + cb) + lane);
                } else {
                    gv.x = cb + 2 * lane < p.C ? p.cnorm[cb + 2 * lane] : 0.0f;
                    gv.y = 0.0f;
                }
                bool got = mbar_wait_or_abort(&t_full[s], u & 1, abort_flag);
                if (!__all_sync(0xffffffffu, got)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // (the previous tile's reads of gs are done: __syncwarp at its end)
                if (MODE == PG_FILTER) {
                    reinterpret_cast<float2*>(gs)[lane] =
                        make_float2(__fmaf_rn(-qlen_w, kv.x, gv.x), __fmaf_rn(-qlen_w, kv.y, gv.y));
                } else {
                    reinterpret_cast<float2*>(gs)[lane] = gv;
                    if (MODE == PG_CHUNKMIN) reinterpret_cast<float2*>(gs + 64)[lane] = kv;
                }
                __syncwarp();
#pragma unroll
                for (int j = 0; j < PG_QT; j++) {
                    uint32_t ra[32], rb[32];
                    const uint32_t ta = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)((s * PG_QT + j) * MM_N + hf * 64);
                    tmem_ld32_async(ta, ra);
                    tmem_ld32_async(ta + 32, rb);
                    tmem_wait_ld();
                    pg_chunk<MODE>(p, ra, gs, 64, cb, row[j], qn[j], qlen[j], h[j], sv[j], nsv[j], bv[j], bi[j]);
                    pg_chunk<MODE>(p, rb, gs + 32, 64, cb + 32, row[j], qn[j], qlen[j], h[j], sv[j], nsv[j], bv[j],
                                   bi[j]);
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&t_empty[s]);
            }
            if (MODE == PG_FILTER && ok) {
#pragma unroll
                for (int j = 0; j < PG_QT; j++)
                    if (row[j] < p.nq) p.f.scnt[((int64_t)row[j] * p.nsplit + sp) * 2 + hf] = nsv[j];
            }
            if (MODE == PG_ARGMIN && ok) {
#pragma unroll
                for (int j = 0; j < PG_QT; j++)
                    if (row[j] < p.nq) p.amin[((int64_t)row[j] * p.nsplit + sp) * 2 + hf] = make_key(bv[j], (uint32_t)bi[j]);
            }
        }
        if (!ok && lane == 0) {
            *abort_flag = 1;
            atomicExch(p.err, 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(PG_TMEM_COLS)
                     : "memory");
}

size_t coarse_gemm_qtile_bytes(int nq) {
    const int nqp = (nq + PG_QT * MM_M - 1) / (PG_QT * MM_M);
    return (size_t)nqp * PG_QT * A_TILE_BYTES;
}

size_t coarse_gemm_col_floats(int C) { return (size_t)((C + MM_N - 1) / MM_N) * MM_N; }

template <int MODE>
static cudaError_t launch_pg_mode(const PgArgs& p, int grid, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(coarse_gemm_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)PG_SMEM);
    if (e != cudaSuccess) return e;
    coarse_gemm_kernel<MODE><<<grid, PG_THREADS, PG_SMEM, st>>>(p);
    return cudaGetLastError();
}

int coarse_gemm_nsplit(int nq, int C, int num_sms, int* split_tiles) {
    const int nqp = (nq + PG_QT * MM_M - 1) / (PG_QT * MM_M);
    const int nct = (C + MM_N - 1) / MM_N;
    // about 8 items per SM, each a range of at least 8 centroid tiles, at most 256 ranges, none empty
    const int sms = std::max(num_sms, 1);
    int nsplit = std::max(1, (8 * sms + nqp - 1) / nqp);
    nsplit = std::min(std::min(nsplit, 256), std::max(1, nct / 8));
    const int st = (nct + nsplit - 1) / nsplit;
    if (split_tiles) *split_tiles = st;
    return (nct + st - 1) / st;
}

static cudaError_t launch_pg(PgArgs& p, int mode, int num_sms, cudaStream_t st) {
    if (p.nq <= 0) return cudaSuccess;
    p.nqp = (p.nq + PG_QT * MM_M - 1) / (PG_QT * MM_M);
    p.nct = (p.C + MM_N - 1) / MM_N;
    p.nsplit = coarse_gemm_nsplit(p.nq, p.C, num_sms, &p.split_tiles);
    if (mode == PG_FILTER && p.nsplit != p.f.nsplit) return cudaErrorInvalidValue;
    const int grid = std::min(p.nqp * p.nsplit, std::max(num_sms, 1));
    switch (mode) {
        case PG_STORE: return launch_pg_mode<PG_STORE>(p, grid, st);
        case PG_CHUNKMIN: return launch_pg_mode<PG_CHUNKMIN>(p, grid, st);
        case PG_ARGMIN: return launch_pg_mode<PG_ARGMIN>(p, grid, st);
        default: return launch_pg_mode<PG_FILTER>(p, grid, st);
    }
}

cudaError_t launch_coarse_gemm_store(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                     const double* qnorm, const float* cnorm, float* out, int64_t ld, int num_sms,
                                     int* err, cudaStream_t st, bool stall_copy) {
    if (!out || ld < C) return cudaErrorInvalidValue;
    PgArgs p;
    p.stall_copy = stall_copy;
    p.qtiles = qtiles;
    p.ctiles = ctiles;
    p.nq = nq;
    p.C = C;
    p.qnorm = qnorm;
    p.cnorm = cnorm;
    p.out = out;
    p.ld = ld;
    p.err = err;
    return launch_pg(p, PG_STORE, num_sms, st);
}

cudaError_t launch_coarse_gemm_chunkmin(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                        const double* qnorm, const float* cnorm, const float* colG,
                                        const float* colK, float* out, int64_t ld, int num_sms, int* err,
                                        cudaStream_t st) {
    if (!out || !colG || !colK || ld * 32 < C || C % 32) return cudaErrorInvalidValue;
    PgArgs p;
    p.qtiles = qtiles;
    p.ctiles = ctiles;
    p.nq = nq;
    p.C = C;
    p.qnorm = qnorm;
    p.cnorm = cnorm;
    p.colG = colG;
    p.colK = colK;
    p.out = out;
    p.ld = ld;
    p.err = err;
    return launch_pg(p, PG_CHUNKMIN, num_sms, st);
}

cudaError_t launch_coarse_gemm_argmin(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C, const float* cnorm,
                                      unsigned long long* part, int num_sms, int* err, cudaStream_t st, bool hi_only) {
    if (!part) return cudaErrorInvalidValue;
    PgArgs p;
    p.hi_only = hi_only;
    p.qtiles = qtiles;
    p.ctiles = ctiles;
    p.nq = nq;
    p.C = C;
    p.cnorm = cnorm;
    p.amin = part;
    p.err = err;
    return launch_pg(p, PG_ARGMIN, num_sms, st);
}

cudaError_t launch_coarse_gemm_filter(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                      const double* qnorm, const float* cnorm, const CoarseFilter& f,
                                      const float* colG, const float* colK, float cn_max, float clen_max,
                                      int num_sms, int* err, cudaStream_t st) {
    if (!f.thr || !f.surv || !f.scnt || f.sreg <= 0 || !colG || !colK) return cudaErrorInvalidValue;
    PgArgs p;
    p.qtiles = qtiles;
    p.ctiles = ctiles;
    p.nq = nq;
    p.C = C;
    p.qnorm = qnorm;
    p.cnorm = cnorm;
    p.f = f;
    p.colG = colG;
    p.colK = colK;
    p.cn_max = cn_max;
    p.clen_max = clen_max;
    p.err = err;
    return launch_pg(p, PG_FILTER, num_sms, st);
}

}  // namespace gbivf
