// Block-wide exact streaming top-k over unique 64-bit keys.
//
// Replaces the reference's selections -- yael's heap (binheap.c:102-170),
// its quickselect + qsort (sorting.c:143-194) and the GPU path's per-thread
// sub-heaps with a single-thread merge (parallel2/ivf_pq/topk.cu:223-337) --
// by a threshold filter in front of a shared-memory candidate buffer:
//
//   * every thread offers keys; a key below the current k-th best is
//     appended to the buffer (one shared atomic per warp, ballot-aggregated);
//   * a flush finds the exact k-th smallest key of (best u buffer) with a
//     block radix select (8-bit digits, starting at the highest bit in which
//     the pool's keys differ), keeps the keys <= it as the new best set
//     (unordered) and lowers the threshold to it;
//   * the final call sorts the k survivors (by rank up to 256 keys, else a
//     bitonic network).
//
// Keys are unique (the low 32 bits carry a unique payload), so the result is
// exactly the k smallest keys, ascending.
//
// Protocol (all threads of the block, uniform control flow):
//   topk_init(s, k)  ->  offer() from every thread of every warp, with
//   topk_round_end(s, incoming) or explicit topk_flush(s, nb) between rounds
//   ->  topk_finish(s)  ->  best[0..nbest) ascending
#pragma once
#include "common.cuh"

namespace gbivf {

constexpr int TOPK_WORK_BYTES = 2 * 256 * 4 + 16 * 4 + 4 * 8;  // two histograms, ints, u64 slots

struct TopKSmem {
    u64* best;    // [kcap] best set (unordered until topk_finish), nbest valid
    u64* tmp;     // [kcap] compaction output
    u64* buf;     // [bcap] unsorted candidates, bcap a power of two
    int* nbuf;    // shared counters
    int* nbest;
    u64* thresh;  // current k-th best key (KEY_MAX until k are known)
    int k, kcap, bcap;
    unsigned char* work;  // TOPK_WORK_BYTES, 8-byte aligned
    // radix-select pass p uses histogram p & 1 and result ints info() + 8 (p & 1) (info()[4] is
    // the flush's compaction counter)
    __device__ int* hist(int p = 0) const { return reinterpret_cast<int*>(work + 1024 * (p & 1)); }
    __device__ int* info() const { return reinterpret_cast<int*>(work + 2048); }
    __device__ u64* slots() const { return reinterpret_cast<u64*>(work + 2112); }
};

__device__ __forceinline__ void topk_init(TopKSmem& s, int k) {
    s.k = k;
    if (threadIdx.x == 0) {
        *s.nbuf = 0;
        *s.nbest = 0;
        *s.thresh = KEY_MAX;
        s.slots()[0] = 0;
        s.info()[4] = 0;
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

// Warp-collective append of keys that already passed the caller's filter.
__device__ __forceinline__ void topk_push(TopKSmem& s, u64 key, bool pass) {
    unsigned mask = __ballot_sync(0xffffffffu, pass);
    if (mask == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(s.nbuf, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pass) s.buf[base + __popc(mask & ((1u << lane) - 1u))] = key;
}

// Warp-collective append of R keys per lane (row r of every lane, then row r + 1, ...) with one
// shared atomic for all of them; the caller has checked that some lane passes.
template <int R>
__device__ __forceinline__ void topk_push_rows(TopKSmem& s, const u64 (&key)[R], const bool (&pass)[R]) {
    const int lane = threadIdx.x & 31;
    unsigned msk[R], all = 0;
    int total = 0;
#pragma unroll
    for (int r = 0; r < R; r++) {
        msk[r] = __ballot_sync(0xffffffffu, pass[r]);
        all |= msk[r];
        total += __popc(msk[r]);
    }
    if (all == 0) return;
    const int leader = __ffs(all) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(s.nbuf, total);
    base = __shfl_sync(0xffffffffu, base, leader);
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (pass[r]) s.buf[base + __popc(msk[r] & lt)] = key[r];
        base += __popc(msk[r]);
    }
}

// Ascending order of n unique keys a[0..n) (with their ids b[0..n) when b is not NULL), for
// n <= 2 * blockDim.x: every element's final position is the number of smaller keys, found by one
// pass over the keys; two block barriers in all, where a bitonic network of n = 128 takes 28.
__device__ inline void rank_sort(u64* a, int32_t* b, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const bool h0 = tid < n, h1 = tid + nt < n;
    u64 k0 = h0 ? a[tid] : KEY_MAX, k1 = h1 ? a[tid + nt] : KEY_MAX;
    int32_t i0 = 0, i1 = 0;
    if (b) {
        if (h0) i0 = b[tid];
        if (h1) i1 = b[tid + nt];
    }
    int r0 = 0, r1 = 0;
    if (h0)
        for (int j = 0; j < n; j++) {
            const u64 x = a[j];
            r0 += x < k0;
            r1 += x < k1;
        }
    __syncthreads();
    if (h0) a[r0] = k0;
    if (h1) a[r1] = k1;
    if (b) {
        if (h0) b[r0] = i0;
        if (h1) b[r1] = i1;
    }
    __syncthreads();
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

// The K-th smallest (1-based) key of A[0..na) u B[0..nb), 1 <= K <= na+nb.
// Expects slots()[0] == 0 on entry and leaves it 0.
// Two barriers per 8-bit digit: the passes alternate between two histograms and two result
// slots, so the next pass's histogram is cleared while this one is filled, and a pass's result
// is read after the barrier that publishes it without a second barrier before it is reused.
__device__ inline u64 block_kth(TopKSmem& s, const u64* A, int na, const u64* B, int nb, int K) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    u64* slot = s.slots();
    for (int i = tid; i < 256; i += nt) s.hist(0)[i] = 0;  // the first pass's histogram
    const u64 ref = na > 0 ? A[0] : B[0];
    u64 acc = 0;
    for (int i = tid; i < na; i += nt) acc |= A[i] ^ ref;
    for (int i = tid; i < nb; i += nt) acc |= B[i] ^ ref;
    unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)acc);
    unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(acc >> 32));
    if (lane == 0 && (lo | hi)) atomicOr(&slot[0], ((u64)hi << 32) | lo);
    __syncthreads();
    const u64 diff = slot[0];
    __syncthreads();
    if (tid == 0) slot[0] = 0;
    if (diff == 0) return ref;  // a single distinct key
    int hib = 63 - __clzll((long long)diff);
    u64 kmask = hib == 63 ? 0ull : (~0ull << (hib + 1));
    u64 kval = ref & kmask;
    int want = K;
    for (int p = 0;; p++) {
        int* hist = s.hist(p);
        int* info = s.info() + 8 * (p & 1);
        const int lob = max(hib - 7, 0);
        const int width = hib - lob + 1;
        const u64 dmask = ((1ull << width) - 1ull);
        for (int i = tid; i < na; i += nt)
            if ((A[i] & kmask) == kval) atomicAdd(&hist[(A[i] >> lob) & dmask], 1);
        for (int i = tid; i < nb; i += nt)
            if ((B[i] & kmask) == kval) atomicAdd(&hist[(B[i] >> lob) & dmask], 1);
        // clear the next pass's histogram: its last reader, the previous pass's scan, finished
        // before that pass's second barrier
        for (int i = tid; i < 256; i += nt) s.hist(p + 1)[i] = 0;
        __syncthreads();
        if (tid < 32) {
            // lane owns bins 8*lane .. 8*lane+7
            int c[8], sum = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                c[j] = hist[8 * lane + j];
                sum += c[j];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            int before = incl - sum;
            if (before < want && want <= incl) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (before < want && want <= before + c[j]) {
                        info[0] = 8 * lane + j;
                        info[1] = want - before;
                        info[2] = c[j];
                    }
                    before += c[j];
                }
            }
        }
        __syncthreads();
        const int dig = info[0], cnt = info[2];
        want = info[1];
        kmask |= dmask << lob;
        kval |= (u64)dig << lob;
        if (lob == 0) return kval;  // all 64 bits known
        if (cnt == 1) {
            for (int i = tid; i < na; i += nt)
                if ((A[i] & kmask) == kval) slot[1] = A[i];
            for (int i = tid; i < nb; i += nt)
                if ((B[i] & kmask) == kval) slot[1] = B[i];
            __syncthreads();
            const u64 r = slot[1];
            __syncthreads();
            return r;
        }
        hib = lob - 1;
    }
}

// The K-th smallest (1-based, 1 <= K <= their count) of the unique keys A[i], i < n, whose bit i is
// set in flags (every key when flags is NULL), by the same radix select as block_kth: 8-bit digits
// from the highest bit in which those keys differ, until one key is left in the digit's bucket.
// All threads of the block call it; it ends with a barrier.
static __device__ __noinline__ u64 block_kth_flagged(const u64* A, int n, const unsigned* flags, int K) {
    __shared__ int hist[2][256];
    __shared__ int info[2][4];
    __shared__ u64 red[3];  // the smallest key, the OR of the differences to it, the last survivor
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    auto in = [&](int i) { return !flags || ((flags[i >> 5] >> (i & 31)) & 1u); };
    if (tid == 0) {
        red[0] = KEY_MAX;
        red[1] = 0;
    }
    for (int i = tid; i < 256; i += nt) hist[0][i] = 0;
    __syncthreads();
    u64 lo = KEY_MAX;
    for (int i = tid; i < n; i += nt)
        if (in(i)) lo = A[i] < lo ? A[i] : lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const u64 x = __shfl_xor_sync(0xffffffffu, lo, o);
        lo = x < lo ? x : lo;
    }
    if (lane == 0) atomicMin(&red[0], lo);
    __syncthreads();
    const u64 ref = red[0];
    u64 acc = 0;
    for (int i = tid; i < n; i += nt)
        if (in(i)) acc |= A[i] ^ ref;
    const unsigned alo = __reduce_or_sync(0xffffffffu, (unsigned)acc);
    const unsigned ahi = __reduce_or_sync(0xffffffffu, (unsigned)(acc >> 32));
    if (lane == 0 && (alo | ahi)) atomicOr(&red[1], ((u64)ahi << 32) | alo);
    __syncthreads();
    const u64 diff = red[1];
    if (diff == 0) return ref;  // a single key
    int hib = 63 - __clzll((long long)diff);
    u64 kmask = hib == 63 ? 0ull : (~0ull << (hib + 1));
    u64 kval = ref & kmask;
    int want = K;
    for (int p = 0;; p++) {
        int* h = hist[p & 1];
        int* inf = info[p & 1];
        const int lob = max(hib - 7, 0);
        const int width = hib - lob + 1;
        const u64 dmask = (1ull << width) - 1ull;
        for (int i = tid; i < n; i += nt)
            if (in(i) && (A[i] & kmask) == kval) atomicAdd(&h[(A[i] >> lob) & dmask], 1);
        // the next pass's histogram: its last reader, the previous pass's scan, finished before the
        // previous pass's second barrier
        for (int i = tid; i < 256; i += nt) hist[(p + 1) & 1][i] = 0;
        __syncthreads();
        if (tid < 32) {
            int c[8], sum = 0;  // lane owns bins 8 lane .. 8 lane + 7
#pragma unroll
            for (int j = 0; j < 8; j++) {
                c[j] = h[8 * lane + j];
                sum += c[j];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            int before = incl - sum;
            if (before < want && want <= incl) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (before < want && want <= before + c[j]) {
                        inf[0] = 8 * lane + j;
                        inf[1] = want - before;
                        inf[2] = c[j];
                    }
                    before += c[j];
                }
            }
        }
        __syncthreads();
        const int dig = inf[0], cnt = inf[2];
        want = inf[1];
        kmask |= dmask << lob;
        kval |= (u64)dig << lob;
        if (lob == 0) return kval;  // all 64 bits known
        if (cnt == 1) {
            for (int i = tid; i < n; i += nt)
                if (in(i) && (A[i] & kmask) == kval) red[2] = A[i];
            __syncthreads();
            const u64 r = red[2];
            __syncthreads();
            return r;
        }
        hib = lob - 1;
    }
}

// Ascending order of q <= NT * PER unique keys sk[0..q) with their payloads ss[0..q), by a bitonic
// network over NT * PER elements (KEY_MAX padding) held in registers, PER consecutive elements per
// thread: partners within a thread are exchanged in registers, within a warp by shuffles, and only
// the stages across warps go through shared memory (sk, ss). blockDim.x == NT. Ends with a barrier.
template <int NT, int PER>
__device__ __noinline__ void block_sort_regs(u64* sk, int32_t* ss, int q) {
    constexpr int CAP = NT * PER;
    static_assert((CAP & (CAP - 1)) == 0 && (PER & (PER - 1)) == 0 && PER >= 2 && NT % 32 == 0, "powers of two");
    const int tid = threadIdx.x;
    u64 k[PER];
    int32_t v[PER];
#pragma unroll
    for (int e = 0; e < PER; e++) {
        const int i = tid * PER + e;
        k[e] = i < q ? sk[i] : KEY_MAX;
        v[e] = i < q ? ss[i] : 0;
    }
    // one compare-exchange of registers e < e2 in the direction of merge size `size` (selects, no
    // branches: the lanes of a warp disagree on the swap)
    auto cx = [&](int e, int e2, int size) {
        const bool asc = ((tid * PER + e) & size) == 0;
        const u64 a = k[e], b = k[e2];
        const int32_t va = v[e], vb = v[e2];
        const bool sw = (a > b) == asc;
        k[e] = sw ? b : a;
        k[e2] = sw ? a : b;
        v[e] = sw ? vb : va;
        v[e2] = sw ? va : vb;
    };
    // the stages of one merge with partners PER / 2, ..., 1 apart: within the thread
    auto local_stages = [&](int size) {
#pragma unroll
        for (int j = PER / 2; j > 0; j >>= 1) {
            if (j < size) {
#pragma unroll
                for (int e = 0; e < PER; e++)
                    if ((e & j) == 0) cx(e, e | j, size);
            }
        }
    };
    for (int size = 2; size <= CAP; size <<= 1) {
        for (int j = size >> 1; j >= PER; j >>= 1) {  // partners in other threads
            const bool cross = j >= 32 * PER;
            if (cross) {
                __syncthreads();  // the previous cross stage's readers are done
#pragma unroll
                for (int e = 0; e < PER; e++) {
                    sk[tid * PER + e] = k[e];
                    ss[tid * PER + e] = v[e];
                }
                __syncthreads();
            }
            const bool lower = ((tid * PER) & j) == 0;
#pragma unroll
            for (int e = 0; e < PER; e++) {
                const bool asc = ((tid * PER + e) & size) == 0;
                u64 ok;
                int32_t ov;
                if (cross) {
                    ok = sk[(tid * PER + e) ^ j];
                    ov = ss[(tid * PER + e) ^ j];
                } else {
                    ok = __shfl_xor_sync(0xffffffffu, k[e], j / PER);
                    ov = __shfl_xor_sync(0xffffffffu, v[e], j / PER);
                }
                const bool take = (lower == asc) ? ok < k[e] : ok > k[e];
                k[e] = take ? ok : k[e];
                v[e] = take ? ov : v[e];
            }
        }
        local_stages(size);
    }
    __syncthreads();  // the last cross stage's readers are done
#pragma unroll
    for (int e = 0; e < PER; e++) {
        const int i = tid * PER + e;
        if (i < q) {
            sk[i] = k[e];
            ss[i] = v[e];
        }
    }
    __syncthreads();
}

// Merge the nb buffered keys into the best set. nb is block-uniform.
__device__ inline void topk_flush(TopKSmem& s, int nb) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    if (nb <= 0) return;
    const int na = *s.nbest, k = s.k;
    if (na + nb < k) {
        for (int i = tid; i < nb; i += nt) s.best[na + i] = s.buf[i];
        __syncthreads();
        if (tid == 0) {
            *s.nbest = na + nb;
            *s.nbuf = 0;
        }
        __syncthreads();
        return;
    }
    const u64 T = block_kth(s, s.best, na, s.buf, nb, k);
    int* ctr = s.info() + 4;  // zero on entry (topk_init / previous flush)
    for (int i0 = 0; i0 < na + nb; i0 += nt) {
        const int i = i0 + tid;
        u64 x = 0;
        bool keep = false;
        if (i < na + nb) {
            x = i < na ? s.best[i] : s.buf[i - na];
            keep = x <= T;
        }
        unsigned m = __ballot_sync(0xffffffffu, keep);
        if (m) {
            int leader = __ffs(m) - 1, base = 0;
            if (lane == leader) base = atomicAdd(ctr, __popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (keep) s.tmp[base + __popc(m & ((1u << lane) - 1u))] = x;
        }
    }
    __syncthreads();
    for (int i = tid; i < k; i += nt) s.best[i] = s.tmp[i];
    __syncthreads();
    if (tid == 0) {
        *s.nbest = k;
        *s.nbuf = 0;
        *s.thresh = T;
        *ctr = 0;
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

// Final flush, then sort the survivors ascending.
__device__ __forceinline__ void topk_finish(TopKSmem& s) {
    __syncthreads();
    int nb = *s.nbuf;
    __syncthreads();
    topk_flush(s, nb);
    const int n = *s.nbest;
    if (n > 1 && n <= 256 && n <= 2 * (int)blockDim.x) {
        rank_sort(s.best, nullptr, n);  // (the flush's last barrier published the best set)
    } else if (n > 1) {
        int p = 2;
        while (p < n) p <<= 1;
        for (int i = n + threadIdx.x; i < p; i += blockDim.x) s.best[i] = KEY_MAX;
        __syncthreads();
        bitonic_sort_smem(s.best, p);
    }
}

}  // namespace gbivf
