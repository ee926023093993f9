// Filtered coarse stage for large coarse quantizers.
//
// knn_full over C centroids (sequential/ivf_pq/ivf_search.cpp:37-38) keeps the
// w nearest of C per query. Writing the whole nq x C distance block and
// selecting from it costs 8 bytes of HBM traffic per (query, centroid) and a
// long latency-bound selection per query; at C = 262,144 that is most of a
// search. For large C the stage runs as:
//
//   1. a sample: distances (exact for the plain form, approximate for the
//      tensor-core form) to the first S ~ C/8 centroids;
//   2. per query, T = the r-th smallest of the sample (upper bounds approx +
//      eps in the mixed form), r about twice w * S / C, so that about 2w
//      centroids of the whole set fall below T;
//   3. the full distance pass (SIMT or tcgen05) appends every centroid that
//      can fall below T (exact <= T; approx - eps <= T) to the query's
//      candidate slots and, in the mixed form, counts the centroids that
//      certainly do (approx + eps <= T);
//   4. per query, if at least w centroids certainly fall below T, the true w
//      nearest are among the candidates: their exact distances (the
//      reference's FP32 arithmetic, nn.c:143-145 and 85-86) and the keyed
//      top-w give the plain path's result bit for bit. Otherwise (too few
//      below T, or more candidates than slots) the query takes all C
//      centroids exactly -- slow, rare and still exact.
//
// The result never depends on the sample: T only decides how much work the
// candidate set takes.
#include <algorithm>
#include <cmath>

#include "block_topk.cuh"
#include "kernels.cuh"

namespace gbivf {

constexpr int KT_NT = 128, KT_ITEMS = 8;  // sample selection
constexpr int CC_NT = 128, CC_KC = 32;    // candidate selection: batch of rows, staged dimensions

static int pow2_ge(int x) {
    int p = 2;
    while (p < x) p <<= 1;
    return p;
}

constexpr int CC_MAX_REGIONS = 512;  // survivor regions per query (2 x the GEMM's centroid ranges)

static size_t cand_select_smem(int w, int cap, int d) {
    const int kcap = pow2_ge(std::max(w, 2));
    const int bcap = std::max(std::max(cap, 2 * CC_NT), kcap);
    return sizeof(u64) * (2 * (size_t)kcap + bcap + 1) + TOPK_WORK_BYTES + 2 * sizeof(int) + sizeof(float) * d +
           sizeof(int) * CC_NT + sizeof(float) * CC_NT * (CC_KC + 1) + sizeof(int) * (2 * CC_MAX_REGIONS + 5);
}

bool coarse_filter_shape(int C, int w, int d, int* S, int* r, int* cap) {
    if (C < 16384 || w < 1 || w > 1024) return false;
    int s = std::max(4096, (C / 8 + 127) / 128 * 128);
    s = std::min(s, C);
    const int rr = std::min(s, (int)std::ceil(2.0 * w * (double)s / (double)C) + 8);
    const int cp = pow2_ge(std::max(1024, 8 * w));
    if (cand_select_smem(w, cp, d) > 200 * 1024) return false;
    *S = s;
    *r = rr;
    *cap = cp;
    return true;
}

// the sample rank of a query that takes wq of the batch's w probes: the batch's rank r scaled down
// (about twice the centroids the query needs below its bound), never above r
__device__ __forceinline__ int sample_rank(const SampleRank& sr, int r, int q) {
    if (!sr.w_per_q) return r;
    const int wq = min(max(sr.w_per_q[q], 1), sr.w);
    return max(1, min(r, (int)ceil(sr.scale * wq) + 8));
}

// thr[q] = r_q-th smallest of row q (plus mixed_eps when clen != NULL)
__global__ void __launch_bounds__(KT_NT) coarse_sample_kth_kernel(const float* __restrict__ vals, int S, int r,
                                                                  const double* __restrict__ qnorm,
                                                                  const float* __restrict__ cnorm,
                                                                  const float* __restrict__ clen, int kcap, int bcap,
                                                                  SampleRank sr, float* __restrict__ thr) {
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem);
    u64* tmp = best + kcap;
    u64* buf = tmp + kcap;
    u64* thresh = buf + bcap;
    unsigned char* work = reinterpret_cast<unsigned char*>(thresh + 1);
    int* cnt = reinterpret_cast<int*>(work + TOPK_WORK_BYTES);
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, bcap, work};
    const int q = blockIdx.x, tid = threadIdx.x;
    const float* row = vals + (int64_t)q * S;
    const float qn = (float)qnorm[q];
    const float qlen = sqrtf(qn);
    topk_init(s, r);
    for (int i0 = 0; i0 < S; i0 += KT_NT * KT_ITEMS) {
#pragma unroll
        for (int it = 0; it < KT_ITEMS; it++) {
            const int c = i0 + it * KT_NT + tid;
            const bool valid = c < S;
            float v = valid ? row[c] : 0.0f;
            if (clen && valid) v = v + mixed_eps(qn, qlen, cnorm[c], clen[c]);
            topk_offer(s, make_key(v, (uint32_t)c), valid);
        }
        topk_round_end(s, KT_NT * KT_ITEMS);
    }
    topk_finish(s);
    if (tid == 0) thr[q] = key_dist(best[min(sample_rank(sr, r, q), *s.nbest) - 1]);
}

cudaError_t launch_coarse_sample_kth(const float* vals, int nq, int S, int r, const double* qnorm,
                                     const float* cnorm, const float* clen, float* thr, cudaStream_t st,
                                     SampleRank sr) {
    if (nq <= 0) return cudaSuccess;
    if (r < 1 || r > S) return cudaErrorInvalidValue;
    const int kcap = pow2_ge(std::max(r, 2));
    const int bcap = pow2_ge(std::max(2 * KT_NT * KT_ITEMS, kcap));
    const size_t sm = sizeof(u64) * (2 * (size_t)kcap + bcap + 1) + TOPK_WORK_BYTES + 2 * sizeof(int);
    if (sm > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(coarse_sample_kth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    coarse_sample_kth_kernel<<<nq, KT_NT, sm, st>>>(vals, S, r, qnorm, cnorm, clen, kcap, bcap, sr, thr);
    return cudaGetLastError();
}

constexpr int KB_NT = 512;  // sample bound: groups per query

// thr[q] = r_q-th smallest of the minima of KB_NT interleaved groups of row q
__global__ void __launch_bounds__(KB_NT) coarse_sample_bound_kernel(const float* __restrict__ vals, int L, int64_t ld,
                                                                    int r, SampleRank sr, float* __restrict__ thr) {
    __shared__ u64 keys[KB_NT];
    __shared__ __align__(8) unsigned char work[TOPK_WORK_BYTES];
    const int q = blockIdx.x, tid = threadIdx.x;
    const float* row = vals + (int64_t)q * ld;
    float m = __int_as_float(0x7f800000);
#pragma unroll 8
    for (int c = tid; c < L; c += KB_NT) m = fminf(m, row[c]);
    keys[tid] = make_key(m, (uint32_t)tid);
    TopKSmem s{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, r, 0, 0, work};
    if (tid == 0) s.slots()[0] = 0;
    __syncthreads();
    const u64 kth = block_kth(s, keys, KB_NT, keys, 0, sample_rank(sr, r, q));
    if (tid == 0) thr[q] = key_dist(kth);
}

cudaError_t launch_coarse_sample_bound(const float* vals, int nq, int L, int64_t ld, int r, float* thr,
                                       cudaStream_t st, SampleRank sr) {
    if (nq <= 0) return cudaSuccess;
    if (r < 1 || r > KB_NT / 4 || r > L || ld < L) return cudaErrorInvalidValue;
    coarse_sample_bound_kernel<<<nq, KB_NT, 0, st>>>(vals, L, ld, r, sr, thr);
    return cudaGetLastError();
}

// Per query: exact keyed top-w over its candidates, or over all C centroids
// when the candidates cannot be trusted to hold the w nearest. Candidates go
// in batches of CC_NT, one per thread; their centroid rows are staged through
// shared memory CC_KC dimensions at a time with row-contiguous (coalesced)
// loads, and each thread keeps its own sequential dot product (l = 0..d-1,
// the reference's order) across the chunks.
__global__ void __launch_bounds__(CC_NT) coarse_cand_select_kernel(const float* __restrict__ X, int d,
                                                                   const float* __restrict__ coa, int C,
                                                                   const double* __restrict__ qnorm,
                                                                   const float* __restrict__ cnorm, int w,
                                                                   CoarseFilter f, int kcap, int bcap,
                                                                   int32_t* __restrict__ coaidx,
                                                                   float* __restrict__ coadis, int* __restrict__ stats) {
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem);
    u64* tmp = best + kcap;
    u64* buf = tmp + kcap;
    u64* thresh = buf + bcap;
    unsigned char* work = reinterpret_cast<unsigned char*>(thresh + 1);
    int* cnt = reinterpret_cast<int*>(work + TOPK_WORK_BYTES);
    float* xq = reinterpret_cast<float*>(cnt + 2);
    int* ids = reinterpret_cast<int*>(xq + d);
    float* rows = reinterpret_cast<float*>(ids + CC_NT);  // [CC_NT][CC_KC + 1]
    int* rcnt = reinterpret_cast<int*>(rows + CC_NT * (CC_KC + 1));  // [CC_MAX_REGIONS] survivor counts
    int* tally = rcnt + CC_MAX_REGIONS;                               // candidates, below, overflow
    int* rpre = tally + 4;                                            // [CC_MAX_REGIONS + 1] prefix of rcnt
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, bcap, work};
    const int q = blockIdx.x, tid = threadIdx.x;
    for (int l = tid; l < d; l += CC_NT) xq[l] = X[(int64_t)q * d + l];
    const double qn = qnorm[q];
    int n, below;
    bool overflow = false;
    if (f.surv) {
        // mixed form: the exact candidate (a - eps <= T) and count (a + eps <= T) tests on the
        // GEMM's pre-test survivors; candidates go to this query's slots of f.cand
        const int G = 2 * f.nsplit;
        if (tid < 3) tally[tid] = 0;
        for (int g = tid; g < G; g += CC_NT) {
            int c = f.scnt[(int64_t)q * G + g];
            if (c > f.sreg) {
                tally[2] = 1;
                c = f.sreg;
            }
            rcnt[g] = c;
        }
        __syncthreads();
        // exclusive prefix of the region counts (thread t sums regions 4t .. 4t + 3), so that the loop
        // below visits the survivors only, not every slot of the regions (sized for the batch's
        // largest nprobe)
        {
            constexpr int PER = CC_MAX_REGIONS / CC_NT;
            static_assert(PER * CC_NT == CC_MAX_REGIONS, "regions per thread");
            int v[PER], sum = 0;
#pragma unroll
            for (int j = 0; j < PER; j++) {
                const int g = tid * PER + j;
                v[j] = g < G ? rcnt[g] : 0;
                sum += v[j];
            }
            const int lane = tid & 31, warp = tid >> 5;
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int x = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += x;
            }
            __shared__ int wsum[CC_NT / 32];
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            int base = incl - sum;
            for (int w2 = 0; w2 < warp; w2++) base += wsum[w2];
#pragma unroll
            for (int j = 0; j < PER; j++) {
                const int g = tid * PER + j;
                if (g < G) rpre[g] = base;
                base += v[j];
            }
            if (tid == CC_NT - 1) rpre[G] = base;
            __syncthreads();
        }
        const int nsurv = rpre[G];
        const float qf = (float)qn, qlen = sqrtf(qf), T = f.thr[q];
        const int2* sq = f.surv + (int64_t)q * G * f.sreg;
        int mine = 0;
#pragma unroll 4
        for (int i = tid; i < nsurv; i += CC_NT) {
            int lo = 0, hi = G;  // the region of survivor i: rpre[lo] <= i < rpre[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (rpre[mid] <= i) lo = mid;
                else hi = mid;
            }
            const int2 v = sq[(int64_t)lo * f.sreg + (i - rpre[lo])];
            const int c = v.x;
            const float cn = cnorm[c];
            const float a = qf + cn - 2.0f * __int_as_float(v.y);
            const float ee = mixed_eps(qf, qlen, cn, f.clen[c]);
            mine += (a + ee <= T) ? 1 : 0;
            if (a - ee <= T) {
                const int slot = atomicAdd(&tally[0], 1);
                if (slot < f.cap) f.cand[(int64_t)q * f.cap + slot] = c;
            }
        }
        if (mine) atomicAdd(&tally[1], mine);
        __syncthreads();
        n = tally[0];
        below = tally[1];
        overflow = tally[2] != 0;
    } else {
        n = f.ncand[q];
        below = f.cnt ? f.cnt[q] : n;
    }
    // the query's own probe count (an uneven batch): its top-wq is the prefix of its top-w
    const int wq = f.w_per_q ? min(max(f.w_per_q[q], 1), w) : w;
    const bool all = overflow || n > f.cap || below < wq;
    const int total = all ? C : n;  // without the fallback n <= cap <= bcap: no flush until the end
    const int32_t* cq = f.cand + (int64_t)q * f.cap;
    topk_init(s, wq);  // (its barrier also publishes xq)
    for (int i0 = 0; i0 < total; i0 += CC_NT) {
        const int i = i0 + tid;
        const bool valid = i < total;
        const int c = valid ? (all ? i : cq[i]) : -1;
        __syncthreads();  // the previous batch is done with ids / rows
        ids[tid] = c;
        __syncthreads();
        float t = 0.0f;
        for (int l0 = 0; l0 < d; l0 += CC_KC) {
            const int lw = min(CC_KC, d - l0);
            // all CC_KC loads of this thread in flight at once (warp = one row, lanes along it)
            float v[CC_KC];
#pragma unroll
            for (int k = 0; k < CC_KC; k++) {
                const int e = tid + k * CC_NT, rr = e / CC_KC, col = e % CC_KC;
                const int cid = ids[rr];
                v[k] = (cid >= 0 && col < lw) ? __ldg(coa + (int64_t)cid * d + l0 + col) : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < CC_KC; k++) {
                const int e = tid + k * CC_NT, rr = e / CC_KC, col = e % CC_KC;
                rows[rr * (CC_KC + 1) + col] = v[k];
            }
            __syncthreads();
            for (int l = 0; l < lw; l++) t = __fadd_rn(t, __fmul_rn(rows[tid * (CC_KC + 1) + l], xq[l0 + l]));
            __syncthreads();
        }
        const u64 key = valid ? make_key(expansion_from(qn, cnorm[c], t), (uint32_t)c) : 0;
        topk_offer(s, key, valid);
        if (all) topk_round_end(s, CC_NT);
    }
    topk_finish(s);
    const int nb = min(*s.nbest, wq);
    for (int j = tid; j < w; j += CC_NT) {
        coaidx[(int64_t)q * w + j] = j < nb ? (int32_t)key_payload(best[j]) : -1;
        coadis[(int64_t)q * w + j] = j < nb ? key_dist(best[j]) : __int_as_float(0x7f800000);
    }
    if (tid == 0 && stats) {
        atomicAdd(&stats[0], total);
        if (all) atomicAdd(&stats[1], 1);
    }
}

cudaError_t launch_coarse_cand_select(const DevIndex& ix, const float* q, const double* qnorm, int nq, int w,
                                      const CoarseFilter& f, int32_t* coaidx, float* coadis, int* stats,
                                      cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    if (!f.cand || f.cap <= 0 || (!f.surv && !f.ncand)) return cudaErrorInvalidValue;
    if (f.surv && (!f.scnt || !f.thr || !f.clen || f.sreg <= 0 || 2 * f.nsplit > CC_MAX_REGIONS))
        return cudaErrorInvalidValue;
    const int kcap = pow2_ge(std::max(w, 2));
    const int bcap = std::max(std::max(f.cap, 2 * CC_NT), kcap);
    if (bcap & (bcap - 1)) return cudaErrorInvalidValue;  // the buffer is a power of two
    const size_t sm = cand_select_smem(w, f.cap, ix.d);
    if (sm > 200 * 1024) return cudaErrorNotSupported;
    if (sm > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(coarse_cand_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    coarse_cand_select_kernel<<<nq, CC_NT, sm, st>>>(q, ix.d, ix.coa, ix.C, qnorm, ix.coa_norm, w, f, kcap, bcap,
                                                      coaidx, coadis, stats);
    return cudaGetLastError();
}

}  // namespace gbivf
