// List-centric IVF-PQ scan: the (query, list) pairs of a batch grouped by
// list, one work item per (list, group of queries).
//
// The reference scans list by list inside each query (sumidxtab2 per probe,
// sequential/ivf_pq/ivf_search.cpp:182-203; the MPI pipeline dispatches the
// same per-list unit, parallel/ivf_pq/ivf_search.cpp:178-228, and the Xeon Phi
// variant per probe, phi2/ivf_pq/ivf_parallel.cpp:276-278). In a large batch
// most code bytes belong to lists that many queries probe, so here one CTA
// takes a list and G queries that probe it:
//
//   * the list's code rows stream once through shared memory (1-D bulk copies,
//     16 KB tiles, double-buffered on mbarriers) for all G queries;
//   * the G queries' m x 256 tables are interleaved, entry-major: the G values
//     of one entry fill one 16-byte word (4 FP32 in the exact form, 8 FP16 in
//     the precision form), so one 128-bit shared load serves G queries;
//   * each (row, query) sum runs in the reference's order and arithmetic, bit
//     for bit the value the query-centric kernel computes.
//
// Top-k without per-query state in the CTA: a first pass (the query-centric
// kernel, SCAN_KEYS_ONLY) scans each query's nearest probes until it holds
// k_sel rows and hands off its k_sel best keys and the k_sel-th key tau_q.
// Every key of the exact top-k_sel over all probes is <= tau_q, so the
// list-centric pass appends only keys below tau_q, to a per-query buffer in
// global memory. That first bound is loose (in 128 dimensions the nearest
// lists are hardly closer than the 200th), so the bound moves: the first
// pass's keys and every emitted key are counted in a per-query histogram of
// their distance below the first bound (256 buckets of 2^15 float ulps, about
// 0.4 % each), and each time a query's emissions pass a multiple of k_sel / 4
// the emitting warp finds
// the lowest bucket edge with k_sel counted keys below it and lowers tau_q to
// it (atomicMin). Any such edge bounds the k_sel-th key from above, so every
// work item read afterwards filters harder and none loses a true candidate.
// The select kernel takes the k_sel smallest of both sets (exact radix
// select) and writes the finalize kernel's hand-off; a query whose buffer
// still overflowed is scanned again by the query-centric kernel. Results are
// identical to the query-centric path's.
#include <cuda_fp16.h>

#include "block_topk.cuh"
#include "exact_round.cuh"
#include "f32x2.cuh"
#include "rot_codes.cuh"
#include "scan_common.cuh"
#include "tc_common.cuh"

namespace gbivf {

constexpr int LC_NT = 512;        // threads of the list-centric scan (one CTA per SM)
constexpr int LC_TILE = 65536;    // bytes of code rows per staged tile
constexpr int LC_SEL_NT = 256;    // threads of the select kernel (one CTA per query)
constexpr int LC_SEL_STAGE = 3072;  // keys of a query's pool the select kernel stages in shared memory
constexpr int LC_HIST_SHIFT = 15;   // histogram bucket width: 2^15 float ulps below the first bound

template <bool MIXED>
struct LcShape {
    static constexpr int G = MIXED ? 8 : 4;  // queries per work item: one 16-byte table word
};

__device__ __forceinline__ int lc_ksel(const ScanArgs& a, int q) {
    const int kq0 = (a.flags & (SCAN_RERANK | SCAN_REFINE)) ? a.kl : query_k(a, q);
    return (a.flags & SCAN_MIXED) ? mixed_sel(a, kq0) : kq0;
}

// ---------------------------------------------------------------------------
// planning: prefix probes per query, pairs per list, groups
// ---------------------------------------------------------------------------

// One warp per query: the first pass's probe count p_q (the fewest leading probes holding
// beta * k_sel rows, all of them when the query has fewer), and one count per remaining
// non-empty probe on its list. Zeroes the query's emission counter.
__global__ void lc_plan_kernel(DevIndex ix, ScanArgs a, ListScanWork w, int beta) {
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (q >= a.nq) return;
    const int wq = query_w(a, q);
    const int64_t target = (int64_t)beta * lc_ksel(a, q);
    int64_t carry = 0;
    int p = wq;
    for (int j0 = 0; j0 < wq && p == wq; j0 += 32) {
        const int j = j0 + lane;
        const int l = j < wq ? __ldg(a.probes + (int64_t)q * a.w + j) : -1;
        int64_t incl = l >= 0 ? __ldg(ix.list_len + l) : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const unsigned hit = __ballot_sync(0xffffffffu, j < wq && carry + incl >= target);
        if (hit) p = j0 + __ffs(hit);  // probes 0 .. j0 + ffs - 1
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) {
        w.w0[q] = p;
        w.ecnt[q] = 0;
    }
    for (int j = p + lane; j < wq; j += 32) {
        const int l = __ldg(a.probes + (int64_t)q * a.w + j);
        if (l >= 0 && __ldg(ix.list_len + l) > 0) atomicAdd(&w.pcnt[l], 1);
    }
}

// Prefix sums over the C lists of their pair counts (pbeg) and of their work items of G pairs
// (gbeg); fill cursors start at pbeg; the totals go to pbeg[C], gbeg[C], counters[0]. Two launches
// over blocks of LC_PFX lists (4 per thread): the blocks' totals, then each block's own scan from the
// sum of the totals before it -- every block at once, instead of one block walking all C lists.
constexpr int LC_PFX = 4096;

template <int G>
__device__ __forceinline__ void lc_prefix_load(int C, const ListScanWork& w, int i0, int (&c)[4], int& tp, int& tg) {
    tp = tg = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        c[j] = i0 + j < C ? w.pcnt[i0 + j] : 0;
        tp += c[j];
        tg += (c[j] + G - 1) / G;
    }
}

template <int G>
__global__ void __launch_bounds__(1024) lc_prefix_sums_kernel(int C, ListScanWork w) {
    __shared__ int s_p[32], s_g[32];
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    int c[4], tp, tg;
    lc_prefix_load<G>(C, w, blockIdx.x * LC_PFX + 4 * tid, c, tp, tg);
    tp = __reduce_add_sync(0xffffffffu, tp);
    tg = __reduce_add_sync(0xffffffffu, tg);
    if (lane == 0) {
        s_p[wp] = tp;
        s_g[wp] = tg;
    }
    __syncthreads();
    if (wp == 0) {
        const int vp = __reduce_add_sync(0xffffffffu, s_p[lane]), vg = __reduce_add_sync(0xffffffffu, s_g[lane]);
        if (lane == 0) {
            w.bsum[2 * blockIdx.x] = vp;
            w.bsum[2 * blockIdx.x + 1] = vg;
        }
    }
}

template <int G>
__global__ void __launch_bounds__(1024) lc_prefix_kernel(int C, ListScanWork w) {
    __shared__ int s_wp[32], s_wg[32], s_base[2];
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5, b = blockIdx.x;
    if (wp == 0) {  // this block's base: the totals of the blocks before it
        int bp = 0, bg = 0;
        for (int j = lane; j < b; j += 32) {
            bp += w.bsum[2 * j];
            bg += w.bsum[2 * j + 1];
        }
        bp = __reduce_add_sync(0xffffffffu, bp);
        bg = __reduce_add_sync(0xffffffffu, bg);
        if (lane == 0) {
            s_base[0] = bp;
            s_base[1] = bg;
        }
    }
    const int i0 = b * LC_PFX + 4 * tid;
    int c[4], tp, tg;
    lc_prefix_load<G>(C, w, i0, c, tp, tg);
    int ip = tp, ig = tg;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int vp = __shfl_up_sync(0xffffffffu, ip, o), vg = __shfl_up_sync(0xffffffffu, ig, o);
        if (lane >= o) {
            ip += vp;
            ig += vg;
        }
    }
    if (lane == 31) {
        s_wp[wp] = ip;
        s_wg[wp] = ig;
    }
    __syncthreads();
    if (wp == 0) {  // exclusive scan of the 32 warp totals
        const int vp = s_wp[lane], vg = s_wg[lane];
        int jp = vp, jg = vg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int up = __shfl_up_sync(0xffffffffu, jp, o), ug = __shfl_up_sync(0xffffffffu, jg, o);
            if (lane >= o) {
                jp += up;
                jg += ug;
            }
        }
        s_wp[lane] = jp - vp;
        s_wg[lane] = jg - vg;
    }
    __syncthreads();
    int rp = s_base[0] + s_wp[wp] + ip - tp, rg = s_base[1] + s_wg[wp] + ig - tg;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (i0 + j < C) {
            w.pbeg[i0 + j] = rp;
            w.fill[i0 + j] = rp;
            w.gbeg[i0 + j] = rg;
        }
        rp += c[j];
        rg += (c[j] + G - 1) / G;
    }
    if (b == gridDim.x - 1 && tid == 1023) {  // the totals
        w.pbeg[C] = rp;
        w.gbeg[C] = rg;
        w.counters[0] = rg;
    }
}

// One warp per query: the position of each probe's first row in the query's candidate order (the
// prefix of list lengths over all its probes) and a pair record per probe the first pass left.
// Also starts the query's bound at the first pass's, and its histogram with the first pass's keys.
__global__ void __launch_bounds__(256) lc_fill_kernel(DevIndex ix, ScanArgs a, ListScanWork w) {
    __shared__ unsigned int s_h[8][LC_HIST_BUCKETS];
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (q >= a.nq) return;
    const int wq = query_w(a, q), p = w.w0[q];
    const u64 t0k = w.tau0[q];
    if (lane == 0) w.tau[q] = t0k;
    for (int i = lane; i < LC_HIST_BUCKETS; i += 32) s_h[wp][i] = 0u;
    __syncwarp();
    if (t0k != KEY_MAX) {
        const uint32_t t0 = (uint32_t)(t0k >> 32);
        const int na = w.cntA[q];
        for (int i = lane; i < na; i += 32) {
            const uint32_t below = t0 - (uint32_t)(w.keysA[(int64_t)q * a.cand_stride + i] >> 32);
            atomicAdd(&s_h[wp][min(LC_HIST_BUCKETS - 1, (int)(below >> LC_HIST_SHIFT))], 1u);
        }
    }
    __syncwarp();
    for (int i = lane; i < LC_HIST_BUCKETS; i += 32) w.hist[(int64_t)q * LC_HIST_BUCKETS + i] = s_h[wp][i];
    uint32_t carry = 0;
    for (int j0 = 0; j0 < wq; j0 += 32) {
        const int j = j0 + lane;
        const int l = j < wq ? __ldg(a.probes + (int64_t)q * a.w + j) : -1;
        const uint32_t len = l >= 0 ? (uint32_t)__ldg(ix.list_len + l) : 0u;
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (j >= p && j < wq && len > 0) {
            const int slot = atomicAdd(&w.fill[l], 1);
            w.pairs[slot] = make_int4(q, j, (int)(carry + incl - len), 0);
        }
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// One thread per list: the descriptors of its work items, each up to G of its pairs. A descriptor is
// 1 + G 16-byte words: (list, pairs, 0, 0), then per slot (query, position of the probe's first row,
// k_sel, float key of the first pass's bound) -- everything the scan needs but the current bound.
template <int G>
__global__ void lc_groups_kernel(DevIndex ix, ScanArgs a, ListScanWork w) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= ix.C) return;
    const int pb = w.pbeg[l], n = w.pbeg[l + 1] - pb, g0 = w.gbeg[l];
    for (int g = 0; g * G < n; g++) {
        int4* d = w.groups + (int64_t)(g0 + g) * (1 + G);
        const int np = min(G, n - g * G);
        d[0] = make_int4(l, np, 0, 0);
        for (int i = 0; i < G; i++) {
            if (i < np) {
                const int4 pr = w.pairs[pb + g * G + i];
                d[1 + i] = make_int4(pr.x, pr.z, lc_ksel(a, pr.x), (int)(uint32_t)(w.tau0[pr.x] >> 32));
            } else {
                d[1 + i] = make_int4(-1, 0, 1, 0);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// the list-centric scan
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t lc_byte(uint32_t v, int s) { return __byte_perm(v, 0u, 0x4440u | (uint32_t)s); }

__device__ __forceinline__ float lc_add_h(float acc, uint32_t word, int hi) {
    const unsigned short h = (unsigned short)(hi ? (word >> 16) : (word & 0xffffu));
    asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(acc) : "h"(h));
    return acc;
}

__device__ __forceinline__ void lc_cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void lc_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void lc_cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }


// One warp: the lowest bucket edge of query q's histogram with at least k_sel emitted keys at or below
// it; tau_q drops to that edge. Bucket i counts keys whose float key lies 2^15 i .. 2^15 (i + 1) - 1
// ulps below the first bound t0 (the last bucket everything lower), so the keys at or below edge j,
// t0 - 2^15 j, are exactly those in buckets j and up.
__device__ __forceinline__ void lc_lower_bound(const ListScanWork& w, int q, uint32_t t0, int ksel, int lane) {
    constexpr int PER = LC_HIST_BUCKETS / 32;
    const unsigned int* hq = w.hist + (int64_t)q * LC_HIST_BUCKETS;
    uint32_t c[PER], sum = 0;
#pragma unroll
    for (int i = 0; i < PER; i++) {
        c[i] = __ldcg(hq + lane * PER + i);
        sum += c[i];
    }
    // keys in the buckets of higher lanes (suffix sum over the warp, exclusive)
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_down_sync(0xffffffffu, incl, o);
        if (lane + o < 32) incl += v;
    }
    uint32_t above = incl - sum;
    int best = -1;  // the largest bucket index j with sum over buckets >= j of at least ksel
#pragma unroll
    for (int i = PER - 1; i >= 0; i--) {
        above += c[i];
        if (best < 0 && above >= (uint32_t)ksel) best = lane * PER + i;
    }
    const unsigned cand = __ballot_sync(0xffffffffu, best >= 0);
    if (!cand) return;
    const int src = 31 - __clz(cand);  // the highest lane that found one holds the largest j
    const int j = __shfl_sync(0xffffffffu, best, src);
    const uint32_t edge = t0 - ((uint32_t)j << LC_HIST_SHIFT);
    if (lane == 0 && j > 0 && edge > 0x80000000u) atomicMin(w.tau + q, ((u64)edge << 32) | 0xffffffffull);
}

template <int M, bool MIXED>
__global__ void __launch_bounds__(LC_NT, 1) lc_scan_kernel(DevIndex ix, ScanArgs a, ListScanWork w) {
    constexpr int NT = LC_NT, D = 128, KS = 256, DS = D / M;
    constexpr int G = LcShape<MIXED>::G;
    constexpr int TPS = NT / M;       // threads per sub-quantizer
    constexpr int E = KS / TPS;       // entries per thread: c = (tid % TPS) + TPS * i
    constexpr int GR = 16 / M;        // code rows per 16-byte group
    constexpr int TILE_GROUPS = LC_TILE / 16;
    constexpr int TILE_ROWS = LC_TILE / M;
    constexpr int UG = TILE_GROUPS / NT;  // 16-byte groups per thread per tile
    constexpr int RS = UG * GR;           // rows per thread per tile
    constexpr int RB = 2;                 // rows looked up together (independent chains)
    static_assert(E % 2 == 0 && E * TPS == KS && UG * NT == TILE_GROUPS && RS % RB == 0, "shape");
    static_assert(G * RB <= 32, "pass bits of a batch fit one word");

    extern __shared__ __align__(16) unsigned char smem[];
    uint4* stage = reinterpret_cast<uint4*>(smem);              // 2 x LC_TILE of code rows
    unsigned char* tab = smem + 2 * LC_TILE;                    // M x 256 x 16 bytes
    float* xs = reinterpret_cast<float*>(tab + M * KS * 16);    // [2][G][D]: the queries of this item and the next
    float* ys = xs + 2 * G * D;                                 // [2][D]: their list centroids
    float* rr = ys + 2 * D;                                     // [G][D]: this item's residuals
    int4* desc = reinterpret_cast<int4*>(rr + G * D);           // [2][1 + G]: this item's descriptor and the next
    float* rn = reinterpret_cast<float*>(desc + 2 * (1 + G));    // [G][M]: this item's residual sub-norms
    __shared__ __align__(16) u64 s_taup[2 * G];  // per slot the 16-byte pair of bounds holding its query's
    __shared__ u64 s_tau[G];                       // per slot its query's bound
    __shared__ int s_abort;
    __shared__ __align__(8) uint64_t bar[2];

    const int tid = threadIdx.x, lane = tid & 31;
    // The exact form's table is sub-quantizer-major ([s][c][g]): a warp owns one sub-quantizer and its
    // lanes consecutive centroids. The precision form's is sub-quantizer-minor ([c][s][g], slot c m + s,
    // see rot_codes.cuh): its lanes take consecutive sub-quantizers of one centroid. Either way a warp's
    // 16-byte table stores are contiguous.
    const int my_s = MIXED ? tid % M : tid / TPS, my_cl = MIXED ? tid / M : tid % TPS;

    // this thread's slice of the codebook: entries (my_s, my_cl + TPS * i), i < E
    constexpr int EP = MIXED ? 1 : E, EM = MIXED ? E / 2 : 1;
    float cen[EP][DS];
    float nhi[EP], nlo[EP];
    f2_t cen2[EM][DS], cn2[EM];
#pragma unroll
    for (int i = 0; i < (MIXED ? 0 : E); i++) {
        const int e = my_s * KS + my_cl + TPS * i;
        const float4* src = reinterpret_cast<const float4*>(ix.pq + (int64_t)e * DS);
#pragma unroll
        for (int v = 0; v < DS / 4; v++) {
            const float4 x = __ldg(src + v);
            cen[i][4 * v] = x.x;
            cen[i][4 * v + 1] = x.y;
            cen[i][4 * v + 2] = x.z;
            cen[i][4 * v + 3] = x.w;
        }
        nhi[i] = __ldg(ix.pq_hi + e);
        nlo[i] = __ldg(ix.pq_lo + e);
    }
#pragma unroll
    for (int p = 0; p < (MIXED ? EM : 0); p++) {
        const int e0 = my_s * KS + my_cl + TPS * (2 * p), e1 = e0 + TPS;
        const float4* s0 = reinterpret_cast<const float4*>(ix.pq + (int64_t)e0 * DS);
        const float4* s1 = reinterpret_cast<const float4*>(ix.pq + (int64_t)e1 * DS);
#pragma unroll
        for (int v = 0; v < DS / 4; v++) {
            const float4 x = __ldg(s0 + v), y = __ldg(s1 + v);
            cen2[p][4 * v] = f2_pack(x.x, y.x);
            cen2[p][4 * v + 1] = f2_pack(x.y, y.y);
            cen2[p][4 * v + 2] = f2_pack(x.z, y.z);
            cen2[p][4 * v + 3] = f2_pack(x.w, y.w);
        }
        cn2[p] = f2_pack(0.25f * __ldg(ix.pq_hi + e0), 0.25f * __ldg(ix.pq_hi + e1));
    }

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    // Work items are taken in a fixed order, this CTA's being blockIdx.x, + gridDim.x, ..., so the
    // next item is known ahead: warp 0 copies its descriptor (cp.async) while this item's tables are
    // built and its query vectors and list centroid while this item is scanned.
    const int nitems = w.counters[0], istep = gridDim.x;
    auto fetch_desc = [&](int bb, int it) {
        if (lane <= G) lc_cp_async16(desc + bb * (1 + G) + lane, w.groups + (int64_t)it * (1 + G) + lane);
        lc_cp_async_commit();
    };
    // every thread: at most one 16-byte chunk of the query vectors or of the list centroid
    auto fetch_vectors = [&](int bb) {
        const int4 hd = desc[bb * (1 + G)];
        const int nc = hd.y * (D / 4);
        if (tid < nc) {
            const int g = tid / (D / 4), x4 = tid % (D / 4);
            lc_cp_async16(xs + (bb * G + g) * D + 4 * x4, a.queries + (int64_t)desc[bb * (1 + G) + 1 + g].x * D + 4 * x4);
        } else if (tid < nc + D / 4) {
            lc_cp_async16(ys + bb * D + 4 * (tid - nc), ix.coa + (int64_t)hd.x * D + 4 * (tid - nc));
        }
        lc_cp_async_commit();
    };
    if ((int)blockIdx.x < nitems) {
        if (tid < 32) {
            fetch_desc(0, blockIdx.x);
            lc_cp_async_wait_all();
        }
        __syncthreads();
        fetch_vectors(0);
    }
    uint32_t phase = 0;   // bit s: the parity the next wait on stage s expects
    uint32_t tc = 0;      // tiles consumed so far: tile tc uses stage tc & 1
    bool armed[2] = {false, false};
    bool pre = false;     // thread 0: this item's first tile was copied during the previous item
    int b = 0;            // this item's descriptor buffer

    for (int it = blockIdx.x;; it += istep, b ^= 1) {
        lc_cp_async_wait_all();  // this item's vectors (each thread its own chunk)
        __syncthreads();  // the previous item's table and stages are no longer read; this item's data is in
        if (it >= nitems || s_abort) break;
        const int4 hd = desc[b * (1 + G)];
        const int l = hd.x, np = hd.y;
        const int4* slot = desc + b * (1 + G) + 1;  // per query: (query, first-row position, k_sel, t0)
        const int len = __ldg(ix.list_len + l);
        const uint8_t* codes = ix.codes + __ldg(ix.list_beg + l) * (int64_t)M;
        const int nbytes = (len * M + 15) & ~15;  // the code array is padded to whole 16-byte groups
        const int ntiles = (nbytes + LC_TILE - 1) / LC_TILE;
        if (tid == 0 && !pre) {  // (normally copied already, during the previous item's last tile)
            const int st = tc & 1;
            mbar_expect_tx(&bar[st], (uint32_t)min(nbytes, LC_TILE));
            bulk_load(stage + st * TILE_GROUPS, codes, (uint32_t)min(nbytes, LC_TILE), &bar[st]);
            armed[st] = true;
        }
        pre = false;
        if (tid < 32) {
            // the queries' current bounds (the 16-byte pair holding each, from L2: other SMs lower them)
            // and the next item's descriptor
            if (lane < np) lc_cp_async16(s_taup + 2 * lane, w.tau + (slot[lane].x & ~1));
            if (it + istep < nitems) fetch_desc(b ^ 1, it + istep);
            else lc_cp_async_commit();
        }
        // residuals r = x_q - y_l (bsxfunMINUS, ivf_search.cpp:155-172) and their sub-norms ||r_s||^2 in
        // the reference's float order (nn.c:129-135): one thread per (query, sub-quantizer), once per
        // item instead of once per table thread
        if (tid < G * M) {
            const int g = tid / M, sq = tid % M;
            float r[DS];
#pragma unroll
            for (int t = 0; t < DS; t++)
                r[t] = g < np ? __fsub_rn(xs[(b * G + g) * D + sq * DS + t], ys[b * D + sq * DS + t]) : 0.0f;
#pragma unroll
            for (int t = 0; t < DS; t += 4)
                *reinterpret_cast<float4*>(rr + g * D + sq * DS + t) = make_float4(r[t], r[t + 1], r[t + 2], r[t + 3]);
            rn[tid] = norm_f_seq(r, DS);
        }
        __syncthreads();
        // the G interleaved tables from the register codebook
        if constexpr (MIXED) {
            // ||r_s - c||^2 / 4 = ||r_s||^2 / 4 + ||c||^2 / 4 - <r_s, c> / 2 by packed fused multiply-adds, in FP16
            uint32_t hw[G][EM];
#pragma unroll
            for (int g = 0; g < G; g++) {
                if (g < np) {
                    float rs[DS];
                    const float4* r4 = reinterpret_cast<const float4*>(rr + g * D + my_s * DS);
#pragma unroll
                    for (int v4 = 0; v4 < DS / 4; v4++) {
                        const float4 x = r4[v4];
                        rs[4 * v4] = x.x;
                        rs[4 * v4 + 1] = x.y;
                        rs[4 * v4 + 2] = x.z;
                        rs[4 * v4 + 3] = x.w;
                    }
                    f2_t rs2[DS];
#pragma unroll
                    for (int t = 0; t < DS; t++) rs2[t] = f2_pack(rs[t], rs[t]);
                    const float f4 = 0.25f * rn[g * M + my_s];
                    const f2_t f42 = f2_pack(f4, f4), mh2 = f2_pack(-0.5f, -0.5f);
#pragma unroll
                    for (int p = 0; p < EM; p++) {
                        f2_t dt = f2_pack(0.0f, 0.0f);
#pragma unroll
                        for (int t = 0; t < DS; t++) dt = f2_fma(rs2[t], cen2[p][t], dt);
                        float e0, e1;
                        f2_unpack(f2_fma(mh2, dt, f2_add(f42, cn2[p])), e0, e1);
                        uint32_t r;
                        asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(e1), "f"(e0));
                        hw[g][p] = r;  // (entry 2p, entry 2p+1) of query g
                    }
                } else {
#pragma unroll
                    for (int p = 0; p < EM; p++) hw[g][p] = 0u;
                }
            }
            // entry-major words: the 8 queries' FP16 values of one entry in one 16-byte word
#pragma unroll
            for (int p = 0; p < EM; p++) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint32_t sel = h ? 0x7632u : 0x5410u;
                    const uint4 v = make_uint4(__byte_perm(hw[0][p], hw[1][p], sel), __byte_perm(hw[2][p], hw[3][p], sel),
                                               __byte_perm(hw[4][p], hw[5][p], sel), __byte_perm(hw[6][p], hw[7][p], sel));
                    const int c = my_cl + TPS * (2 * p + h);
                    *reinterpret_cast<uint4*>(tab + ((c * M + my_s) << 4)) = v;
                }
            }
        } else {
            // the reference's entry: -2 <r_s, c> + (float)(||c||^2 + ||r_s||^2) (nn.c:113-150), the dot
            // product's products as fma(r, c, -0) (one rounding, never fused with the add); entry pairs
            // outermost, so that the G queries' values of an entry are stored as one 16-byte word
            const f2_t m2 = f2_pack(-2.0f, -2.0f), nz2 = f2_pack(a.neg_zero, a.neg_zero);
            float fq[G];
#pragma unroll
            for (int g = 0; g < G; g++) fq[g] = g < np ? rn[g * M + my_s] : 0.0f;
#pragma unroll
            for (int i = 0; i < E; i += 2) {
                float o0[G], o1[G];
                const int e = my_s * KS + my_cl + TPS * i;
#pragma unroll
                for (int g = 0; g < G; g++) {
                    if (g < np) {
                        float rs[DS];
                        const float4* r4 = reinterpret_cast<const float4*>(rr + g * D + my_s * DS);
#pragma unroll
                        for (int v4 = 0; v4 < DS / 4; v4++) {
                            const float4 x = r4[v4];
                            rs[4 * v4] = x.x;
                            rs[4 * v4 + 1] = x.y;
                            rs[4 * v4 + 2] = x.z;
                            rs[4 * v4 + 3] = x.w;
                        }
                        const float f = fq[g];
                        const f2_t f2 = f2_pack(f, f);
                        f2_t d2 = f2_pack(0.0f, 0.0f);
#pragma unroll
                        for (int t = 0; t < DS; t++)
                            d2 = f2_add(d2, f2_fma(f2_pack(rs[t], rs[t]), f2_pack(cen[i][t], cen[i + 1][t]), nz2));
                        float d0, d1;
                        f2_unpack(d2, d0, d1);
                        const f2_t hi2 = f2_pack(nhi[i], nhi[i + 1]);
                        const f2_t S2 = f2_add(hi2, f2);
                        const f2_t bb = f2_sub(S2, hi2);
                        const f2_t e1 = f2_add(f2_sub(hi2, f2_sub(S2, bb)), f2_sub(f2, bb));
                        const f2_t t2 = f2_add(e1, f2_pack(nlo[i], nlo[i + 1]));
                        float Sa, Sb, ta, tb;
                        f2_unpack(S2, Sa, Sb);
                        f2_unpack(t2, ta, tb);
                        const f2_t c02 = f2_pack(add_norms_finish(ix.pq_norm + e, Sa, ta, f),
                                                 add_norms_finish(ix.pq_norm + e + TPS, Sb, tb, f));
                        f2_unpack(f2_add(f2_mul(m2, f2_pack(d0, d1)), c02), o0[g], o1[g]);
                    } else {
                        o0[g] = o1[g] = 0.0f;
                    }
                }
                const int c = my_cl + TPS * i;
                *reinterpret_cast<float4*>(tab + ((my_s * KS + c) << 4)) = make_float4(o0[0], o0[1], o0[2], o0[3]);
                *reinterpret_cast<float4*>(tab + ((my_s * KS + c + TPS) << 4)) = make_float4(o1[0], o1[1], o1[2], o1[3]);
            }
        }
        if (tid < 32) {
            lc_cp_async_wait_all();  // the bounds (each lane waits for its own copy) and the next descriptor
            if (lane < G) s_tau[lane] = lane < np ? s_taup[2 * lane + (slot[lane].x & 1)] : 0ull;  // 0: nothing passes
        }
        __syncthreads();  // tables written; bounds in
        if (it + istep < nitems) fetch_vectors(b ^ 1);  // they arrive during this item's scan
        const u64* tau = s_tau;

        for (int t = 0; t < ntiles; t++, tc++) {
            const int st = tc & 1;
            const bool ok = mbar_wait(&bar[st], (phase >> st) & 1u);
            if (__syncthreads_or(!ok)) {  // a copy did not land in time: report, drain, stop
                if (tid == 0) {
                    s_abort = 1;
                    atomicOr(w.err, 1);
                }
                goto done;
            }
            phase ^= 1u << st;
            armed[st] = false;
            if (tid == 0) {
                // the tile after this one: this item's next, or the next item's first (its descriptor
                // has been in since the table barrier)
                const uint8_t* src = nullptr;
                int nb = 0;
                if (t + 1 < ntiles) {
                    src = codes + (int64_t)(t + 1) * LC_TILE;
                    nb = min(LC_TILE, nbytes - (t + 1) * LC_TILE);
                } else if (it + istep < nitems) {
                    const int nl = desc[(b ^ 1) * (1 + G)].x;
                    src = ix.codes + __ldg(ix.list_beg + nl) * (int64_t)M;
                    nb = min(LC_TILE, (__ldg(ix.list_len + nl) * M + 15) & ~15);
                    pre = true;
                }
                if (src) {
                    mbar_expect_tx(&bar[st ^ 1], (uint32_t)nb);
                    bulk_load(stage + (st ^ 1) * TILE_GROUPS, src, (uint32_t)nb, &bar[st ^ 1]);
                    armed[st ^ 1] = true;
                }
            }
            const uint4* sg = stage + st * TILE_GROUPS;
            const int row0 = t * TILE_ROWS;
            const int ngt = min(TILE_GROUPS, (min(TILE_ROWS, len - row0) * M + 15) / 16);
#pragma unroll 1
            for (int r0 = 0; r0 < RS; r0 += RB) {
                if ((r0 / GR) * NT + (tid & ~31) >= ngt) break;  // warp-uniform: no rows left for this warp
                // rows r0 .. r0 + RB - 1 of this thread: row slot r is row r % GR of group u = r / GR, read
                // from the stage here (only the groups of this batch are held in registers)
                float acc[RB][G];
                int rowv[RB];
                uint4 cb[RB];
#pragma unroll
                for (int rb = 0; rb < RB; rb++) {
                    const int r = r0 + rb, gl = (r / GR) * NT + tid;
                    rowv[rb] = row0 + gl * GR + r % GR;
                    cb[rb] = gl < ngt ? sg[gl] : make_uint4(0, 0, 0, 0);
                }
                if constexpr (MIXED) {
                    // row-rotated order (rot_codes.cuh): the lanes of a quarter-warp, consecutive rows, read
                    // different sub-quantizers, i.e. different bank quads of the [c][s] table
                    float s8[RB][G];
                    uint4 rc[RB];
#pragma unroll
                    for (int rb = 0; rb < RB; rb++) {
#pragma unroll
                        for (int g = 0; g < G; g++) s8[rb][g] = 0.0f;
                        const int r = r0 + rb, rr = r % GR;
                        const uint4 c = cb[rb];
                        const int rot = row_rot<M>(rowv[rb]);
                        if constexpr (M == 16) {
                            rc[rb] = rot_bytes(c, rot);
                        } else if constexpr (M == 8) {
                            const uint2 v = rot_bytes(rr == 0 ? make_uint2(c.x, c.y) : make_uint2(c.z, c.w), rot);
                            rc[rb] = make_uint4(v.x, v.y, 0u, 0u);
                        } else {
                            rc[rb] = make_uint4(rot_bytes(row_word(c, rr), rot), 0u, 0u, 0u);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < M; k++) {
#pragma unroll
                        for (int rb = 0; rb < RB; rb++) {
                            const int sk = (k + row_rot<M>(rowv[rb])) & (M - 1);
                            const uint32_t bidx = lc_byte(row_word(rc[rb], k >> 2), k & 3);
                            const uint4 v = *reinterpret_cast<const uint4*>(tab + ((bidx * M + sk) << 4));
                            const uint32_t vw[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                            for (int g = 0; g < G; g++) s8[rb][g] = lc_add_h(s8[rb][g], vw[g >> 1], g & 1);
                        }
                    }
#pragma unroll
                    for (int rb = 0; rb < RB; rb++)
#pragma unroll
                        for (int g = 0; g < G; g++) acc[rb][g] = s8[rb][g] * 4.0f;
                } else {
                    f2_t a01[RB], a23[RB];
#pragma unroll
                    for (int rb = 0; rb < RB; rb++) a01[rb] = a23[rb] = f2_pack(0.0f, 0.0f);
#pragma unroll
                    for (int s = 0; s < M; s++) {
#pragma unroll
                        for (int rb = 0; rb < RB; rb++) {
                            const int rr = (r0 + rb) % GR;
                            const uint4 c = cb[rb];
                            const uint32_t cw = (rr * M + s) >> 2 == 0 ? c.x
                                              : (rr * M + s) >> 2 == 1 ? c.y
                                              : (rr * M + s) >> 2 == 2 ? c.z : c.w;
                            const uint32_t bidx = lc_byte(cw, (rr * M + s) & 3);
                            const float4 v = *reinterpret_cast<const float4*>(tab + ((s * KS + bidx) << 4));
                            a01[rb] = f2_add(a01[rb], f2_pack(v.x, v.y));
                            a23[rb] = f2_add(a23[rb], f2_pack(v.z, v.w));
                        }
                    }
#pragma unroll
                    for (int rb = 0; rb < RB; rb++) {
                        f2_unpack(a01[rb], acc[rb][0], acc[rb][1]);
                        f2_unpack(a23[rb], acc[rb][2], acc[rb][3]);
                    }
                }
                uint32_t pass = 0;
#pragma unroll
                for (int rb = 0; rb < RB; rb++) {
                    const int gl = ((r0 + rb) / GR) * NT + tid;
                    const bool valid = gl < ngt && rowv[rb] < len;
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        const u64 key = make_key(acc[rb][g], (uint32_t)slot[g].y + (uint32_t)rowv[rb]);
                        if (valid && key < tau[g]) pass |= 1u << (g * RB + rb);
                    }
                }
                if (__any_sync(0xffffffffu, pass != 0)) {
                    const unsigned lt = (1u << lane) - 1u;
                    // each query's survivors in this batch; lane g reserves query g's slots, all queries in
                    // one round trip to L2
                    int mytot = 0;
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        int tot = 0;
#pragma unroll
                        for (int rb = 0; rb < RB; rb++) tot += __popc(__ballot_sync(0xffffffffu, (pass >> (g * RB + rb)) & 1u));
                        if (lane == g) mytot = tot;
                    }
                    int mybase = 0;
                    if (lane < G && mytot > 0) mybase = atomicAdd(&w.ecnt[slot[lane].x], mytot);
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        const int tot = __shfl_sync(0xffffffffu, mytot, g);
                        if (tot == 0) continue;  // warp-uniform
                        const int q = slot[g].x;
                        int base = __shfl_sync(0xffffffffu, mybase, g);
                        const int base0 = base;
                        u64* out = w.ebuf + (int64_t)q * w.ecap;
                        unsigned int* hq = w.hist + (int64_t)q * LC_HIST_BUCKETS;
#pragma unroll
                        for (int rb = 0; rb < RB; rb++) {
                            const unsigned msk = __ballot_sync(0xffffffffu, (pass >> (g * RB + rb)) & 1u);
                            if ((pass >> (g * RB + rb)) & 1u) {
                                const int idx = base + __popc(msk & lt);
                                const u64 key = make_key(acc[rb][g], (uint32_t)slot[g].y + (uint32_t)rowv[rb]);
                                if (idx < w.ecap) out[idx] = key;
                                const uint32_t below = (uint32_t)slot[g].w - (uint32_t)(key >> 32);
                                atomicAdd(hq + min(LC_HIST_BUCKETS - 1, (int)(below >> LC_HIST_SHIFT)), 1u);
                            }
                            base += __popc(msk);
                        }
                        // past a multiple of k_sel / 4 emitted keys: a tighter bound from the histogram
                        const int step = max(slot[g].z / 4, 32);
                        if (base0 / step != (base0 + tot) / step)
                            lc_lower_bound(w, q, (uint32_t)slot[g].w, slot[g].z, lane);
                    }
                }
            }
            __syncthreads();  // this stage is free again
        }
    }
done:
    // let every copy in flight land before the CTA's shared memory goes away (bounded waits)
    if (tid == 0)
        for (int s = 0; s < 2; s++)
            if (armed[s]) mbar_wait(&bar[s], (phase >> s) & 1u);
}

// ---------------------------------------------------------------------------
// selection: the first pass's best keys and the emitted keys -> the finalize hand-off
// ---------------------------------------------------------------------------

template <bool ROWS_OUT>
__global__ void __launch_bounds__(LC_SEL_NT) lc_select_kernel(DevIndex ix, ScanArgs a, ListScanWork w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int q = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    const int na = w.cntA[q], ne = w.ecnt[q];
    if (ne > w.ecap) {  // the buffer overflowed: the query-centric kernel scans this query again
        if (tid == 0) w.ovf[atomicAdd(&w.counters[2], 1)] = q;
        return;
    }
    const int stride = a.cand_stride, wq = query_w(a, q), n = na + ne;
    u64* stage = reinterpret_cast<u64*>(smem);                                // LC_SEL_STAGE keys
    uint32_t* prefix = reinterpret_cast<uint32_t*>(stage + LC_SEL_STAGE);     // wq + 1
    int* plist = reinterpret_cast<int*>(prefix + a.w + 1);                    // wq
    unsigned char* work = reinterpret_cast<unsigned char*>(plist + a.w + 1);
    work = reinterpret_cast<unsigned char*>(((uintptr_t)work + 15) & ~(uintptr_t)15);
    __shared__ int s_cnt;
    TopKSmem s{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0, 0, work};
    // the pool: staged in shared memory when it fits, else read in place (the radix passes then go
    // to L2); a small stage keeps several CTAs per SM
    const u64* A = w.keysA + (int64_t)q * stride;
    const u64* B = w.ebuf + (int64_t)q * w.ecap;
    int nA = na, nB = ne;
    if (n <= LC_SEL_STAGE) {
        for (int i = tid; i < na; i += LC_SEL_NT) stage[i] = A[i];
        for (int i = tid; i < ne; i += LC_SEL_NT) stage[na + i] = B[i];
        A = stage;
        nA = n;
        nB = 0;
    }
    for (int j = tid; j < wq; j += LC_SEL_NT) {
        const int l = __ldg(a.probes + (int64_t)q * a.w + j);
        plist[j] = l;
        prefix[j] = l >= 0 ? (uint32_t)__ldg(ix.list_len + l) : 0u;
    }
    if (tid == 0) {
        s_cnt = 0;
        s.slots()[0] = 0;
    }
    __syncthreads();
    if (tid < 32) {  // exclusive prefix of the probe lengths
        uint32_t carry = 0;
        for (int j0 = 0; j0 < wq; j0 += 32) {
            const int j = j0 + lane;
            const uint32_t len = j < wq ? prefix[j] : 0u;
            uint32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (j < wq) prefix[j] = carry + incl - len;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) prefix[wq] = carry;
    }
    const int K = min(lc_ksel(a, q), n);
    u64 T = KEY_MAX;
    if (n > K && K > 0) T = block_kth(s, A, nA, B, nB, K);  // the K-th smallest key
    __syncthreads();
    const int64_t o0 = (int64_t)q * stride;
    for (int i0 = 0; i0 < n; i0 += LC_SEL_NT) {
        const int i = i0 + tid;
        const u64 key = i < nA ? A[i] : (i < n ? B[i - nA] : KEY_MAX);
        const bool keep = i < n && key <= T && K > 0;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (!m) continue;
        int base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(&s_cnt, __popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (keep) {
            const int slot = base + __popc(m & ((1u << lane) - 1u));
            const uint32_t pos = key_payload(key);
            const int j = probe_of(prefix, wq, pos);
            const int l = plist[j];
            const int64_t row = ix.list_beg[l] + (int64_t)(pos - prefix[j]);
            a.cand_key[o0 + slot] = key;
            if (ROWS_OUT) {
                a.cand_id[o0 + slot] = (int32_t)row;
                a.cand_list[o0 + slot] = l;
            } else {
                a.cand_id[o0 + slot] = ix.ids[row];
            }
        }
    }
    // (slots K .. stride - 1 stay unwritten: the finalize kernels read the first cand_cnt only)
    if (tid == 0) a.cand_cnt[q] = K;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

bool list_scan_supported(const DevIndex& ix, const ScanArgs& a) {
    return scan_persistent_supported(ix, a) && !(a.flags & (SCAN_TABLE_DIRECT | SCAN_SRC_RESIDUAL | SCAN_OUT_PACKED));
}

// Keys a query may emit below its threshold. The first pass's k-th key ranks well beyond k over all
// probes for large k (measured at the 100M workload: with 2 k + 2048 slots about one query in seven
// overflowed), so the buffer holds 8 k + 2048; untouched slots cost nothing.
int list_scan_ecap(const ScanArgs& a) { return 8 * scan_persistent_stride(a) + 2048; }

template <int M, bool MIXED>
static cudaError_t launch_lc(const DevIndex& ix, const ScanArgs& a, const ListScanWork& w, int num_sms,
                             cudaStream_t st, cudaEvent_t* ev) {
    constexpr int G = LcShape<MIXED>::G;
    const int C = ix.C, nq = a.nq;
    cudaError_t e;
    auto rec = [&](int i) { return ev && ev[i] ? cudaEventRecord(ev[i], st) : cudaSuccess; };
    if ((e = cudaMemsetAsync(w.pcnt, 0, sizeof(int) * C, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(w.counters, 0, sizeof(int) * 3, st)) != cudaSuccess) return e;
    const int wblocks = (nq * 32 + 255) / 256;
    lc_plan_kernel<<<wblocks, 256, 0, st>>>(ix, a, w, std::max(1, w.beta));
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // first pass: the query-centric kernel over each query's leading probes, keys only
    ScanArgs pa = a;
    pa.flags |= SCAN_KEYS_ONLY;
    pa.w_per_q = w.w0;
    pa.cand_key = w.keysA;
    pa.cand_cnt = w.cntA;
    pa.cand_id = nullptr;
    pa.cand_list = nullptr;
    pa.tau_out = w.tau0;
    pa.queue = w.queue_a;
    if ((e = rec(0)) != cudaSuccess) return e;
    if ((e = launch_scan_persistent(ix, pa, num_sms, 512, st, nullptr, false)) != cudaSuccess) return e;
    if ((e = rec(1)) != cudaSuccess) return e;
    const int pblocks = (C + LC_PFX - 1) / LC_PFX;
    lc_prefix_sums_kernel<G><<<pblocks, 1024, 0, st>>>(C, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    lc_prefix_kernel<G><<<pblocks, 1024, 0, st>>>(C, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    lc_fill_kernel<<<wblocks, 256, 0, st>>>(ix, a, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    lc_groups_kernel<G><<<(C + 255) / 256, 256, 0, st>>>(ix, a, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = rec(2)) != cudaSuccess) return e;
    const size_t smem = 2 * LC_TILE + (size_t)M * 256 * 16 + sizeof(float) * (3 * G * 128 + 2 * 128) +
                        sizeof(int4) * 2 * (1 + G) + sizeof(float) * G * M;
    auto kern = lc_scan_kernel<M, MIXED>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    kern<<<num_sms, LC_NT, smem, st>>>(ix, a, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = rec(3)) != cudaSuccess) return e;
    const bool rows_out = (a.flags & (SCAN_MIXED | SCAN_REFINE)) != 0;
    const size_t ssm = sizeof(u64) * LC_SEL_STAGE + sizeof(int) * (2 * (size_t)a.w + 2) + 16 + TOPK_WORK_BYTES;
    void (*sel)(DevIndex, ScanArgs, ListScanWork) = rows_out ? lc_select_kernel<true> : lc_select_kernel<false>;
    if ((e = cudaFuncSetAttribute(sel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm)) != cudaSuccess)
        return e;
    sel<<<nq, LC_SEL_NT, ssm, st>>>(ix, a, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // queries whose buffer overflowed: the query-centric kernel, all their probes, full hand-off
    ScanArgs fa = a;
    fa.qlist = w.ovf;
    fa.nqlist = w.counters + 2;
    fa.queue = w.queue_b;
    if ((e = rec(4)) != cudaSuccess) return e;
    return launch_scan_persistent(ix, fa, num_sms, 512, st, nullptr, false);
}

cudaError_t launch_list_scan(const DevIndex& ix, const ScanArgs& a, const ListScanWork& w, int num_sms,
                             cudaStream_t st, cudaEvent_t* ev) {
    if (a.nq <= 0) return cudaSuccess;
    if (!list_scan_supported(ix, a) || ix.C > (1 << 24)) return cudaErrorNotSupported;
    if (w.ecap < 1 || w.ecap > list_scan_ecap(a)) return cudaErrorInvalidValue;
    const bool mixed = a.flags & SCAN_MIXED;
    switch (ix.m) {
        case 4: return mixed ? launch_lc<4, true>(ix, a, w, num_sms, st, ev) : launch_lc<4, false>(ix, a, w, num_sms, st, ev);
        case 8: return mixed ? launch_lc<8, true>(ix, a, w, num_sms, st, ev) : launch_lc<8, false>(ix, a, w, num_sms, st, ev);
        case 16:
            return mixed ? launch_lc<16, true>(ix, a, w, num_sms, st, ev) : launch_lc<16, false>(ix, a, w, num_sms, st, ev);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace gbivf
