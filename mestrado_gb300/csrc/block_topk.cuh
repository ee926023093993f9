// Block-wide exact streaming top-k over unique 64-bit keys.
//
// Replaces the reference's selections -- yael's heap (binheap.c:102-170),
// its quickselect + qsort (sorting.c:143-194) and the GPU path's per-thread
// sub-heaps with a single-thread merge (parallel2/ivf_pq/topk.cu:223-337) --
// by a threshold filter in front of a shared-memory candidate buffer:
//
//   * every thread offers keys; a key below the current k-th best is
//     appended to the buffer (one shared atomic per warp, ballot-aggregated);
//   * when the buffer could overflow on the next round, the block sorts it
//     (bitonic network in shared memory) and merges it with the sorted best
//     list (each element finds its output rank by binary search in the other
//     list), keeping the k smallest; the threshold drops to the new k-th key.
//
// Keys are unique (the low 32 bits carry a unique payload), so the result is
// exactly the k smallest keys, ascending.
//
// Protocol (all threads of the block, uniform control flow):
//   topk_init(s, k)  ->  per round: offer() from every thread of every warp,
//   then round_end(s, incoming) ...  ->  topk_finish(s)  -> best[0..nbest)
#pragma once
#include "common.cuh"

namespace gbivf {

struct TopKSmem {
    u64* best;    // [kcap] sorted ascending, nbest valid
    u64* tmp;     // [kcap] merge output
    u64* buf;     // [bcap] unsorted candidates, bcap a power of two
    int* nbuf;    // shared counters
    int* nbest;
    u64* thresh;  // current k-th best key (KEY_MAX until k are known)
    int k, kcap, bcap;
};

__device__ __forceinline__ void topk_init(TopKSmem& s, int k) {
    s.k = k;
    if (threadIdx.x == 0) {
        *s.nbuf = 0;
        *s.nbest = 0;
        *s.thresh = KEY_MAX;
    }
    __syncthreads();
}

// Warp-collective: every lane of the warp calls it (valid=false to abstain).
__device__ __forceinline__ void topk_offer(TopKSmem& s, u64 key, bool valid) {
    bool pass = valid && key < *s.thresh;
    unsigned mask = __ballot_sync(0xffffffffu, pass);
    if (mask == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(s.nbuf, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pass) s.buf[base + __popc(mask & ((1u << lane) - 1u))] = key;
}

__device__ __forceinline__ int lower_bound_u64(const u64* a, int n, u64 x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ inline void bitonic_sort_smem(u64* a, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < (n >> 1); i += nt) {
                int lo = 2 * i - (i & (stride - 1));
                int hi = lo + stride;
                bool asc = (lo & size) == 0;
                u64 x = a[lo], y = a[hi];
                if ((x > y) == asc) {
                    a[lo] = y;
                    a[hi] = x;
                }
            }
            __syncthreads();
        }
    }
}

// Merge the nb buffered keys into best. nb is the block-uniform count.
__device__ inline void topk_flush(TopKSmem& s, int nb) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if (nb <= 0) return;
    int n = 2;
    while (n < nb) n <<= 1;
    for (int i = nb + tid; i < n; i += nt) s.buf[i] = KEY_MAX;
    __syncthreads();
    bitonic_sort_smem(s.buf, n);
    const int na = *s.nbest, k = s.k;
    for (int i = tid; i < na; i += nt) {
        int r = i + lower_bound_u64(s.buf, nb, s.best[i]);
        if (r < k) s.tmp[r] = s.best[i];
    }
    for (int j = tid; j < nb; j += nt) {
        int r = j + lower_bound_u64(s.best, na, s.buf[j]);
        if (r < k) s.tmp[r] = s.buf[j];
    }
    __syncthreads();
    const int nn = min(k, na + nb);
    for (int i = tid; i < nn; i += nt) s.best[i] = s.tmp[i];
    __syncthreads();
    if (tid == 0) {
        *s.nbest = nn;
        *s.nbuf = 0;
        *s.thresh = (nn == k) ? s.best[k - 1] : KEY_MAX;
    }
    __syncthreads();
}

// End of a round: flush if the next round (at most `incoming` keys) could
// overflow the buffer. Two barriers: everyone reads the counter, then acts.
__device__ __forceinline__ void topk_round_end(TopKSmem& s, int incoming) {
    __syncthreads();
    int nb = *s.nbuf;
    __syncthreads();
    if (nb + incoming > s.bcap) topk_flush(s, nb);
}

__device__ __forceinline__ void topk_finish(TopKSmem& s) {
    __syncthreads();
    int nb = *s.nbuf;
    __syncthreads();
    topk_flush(s, nb);
}

}  // namespace gbivf
