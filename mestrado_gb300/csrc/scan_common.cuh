// Pieces shared by the two scan kernels (one CTA per query, and the
// persistent register-codebook kernel): the shared-memory layout, the ADC
// row sum, position -> id mapping and the output / re-rank epilogue.
#pragma once
#include <algorithm>

#include "block_topk.cuh"
#include "kernels.cuh"

namespace gbivf {

struct ScanSmem {
    size_t off_best, off_tmp, off_buf, off_thresh, off_table, off_xq, off_r, off_rn, off_prefix,
        off_plist, off_cand, off_cnt, off_misc, off_work, off_stage, total;
};

// tables: number of m x ks table buffers of table_elem bytes per entry; rrows: residual rows held
// at once; stage_bytes: staging area for code rows copied ahead (16-byte aligned)
inline ScanSmem scan_smem_layout(int m, int ks, int d, int w, int kcap, int bcap, int tables = 1, int rrows = 1,
                                 int table_elem = 4, size_t stage_bytes = 0) {
    ScanSmem L;
    size_t o = 0;
    auto take = [&](size_t bytes, size_t align) {
        o = (o + align - 1) / align * align;
        size_t r = o;
        o += bytes;
        return r;
    };
    L.off_best = take(sizeof(u64) * kcap, 16);
    L.off_tmp = take(sizeof(u64) * kcap, 16);
    L.off_buf = take(sizeof(u64) * bcap, 16);
    L.off_thresh = take(sizeof(u64), 8);
    L.off_table = take((size_t)table_elem * m * ks * tables, 16);
    L.off_xq = take(sizeof(float) * d, 16);
    L.off_r = take(sizeof(float) * d * rrows, 16);
    L.off_rn = take(sizeof(float) * m * rrows, 16);
    L.off_prefix = take(sizeof(uint32_t) * (w + 1), 16);
    L.off_plist = take(sizeof(int) * w, 16);
    L.off_cand = take(sizeof(int) * kcap, 16);
    L.off_cnt = take(sizeof(int) * 2, 8);
    L.off_misc = take(sizeof(int) * 4, 8);
    L.off_work = take(TOPK_WORK_BYTES, 16);
    L.off_stage = take(stage_bytes, 16);
    L.total = (o + 15) / 16 * 16;
    return L;
}

inline int pow2_at_least(int x) {
    int n = 1;
    while (n < x) n <<= 1;
    return n;
}

// ADC sum of one code row: acc = 0; acc += T[s][code[s]] in s order
// (sumidxtab2, sequential/ivf_pq/ivf_search.cpp:189-200)
template <int M>
__device__ __forceinline__ float adc_row(const uint8_t* __restrict__ row, const float* __restrict__ T, int m,
                                         int ks) {
    float acc = 0.0f;
    if constexpr (M == 4) {
        uint32_t v = __ldg(reinterpret_cast<const uint32_t*>(row));
#pragma unroll
        for (int s = 0; s < 4; s++) acc = __fadd_rn(acc, T[s * ks + ((v >> (8 * s)) & 0xff)]);
    } else if constexpr (M == 8) {
        uint2 v = __ldg(reinterpret_cast<const uint2*>(row));
#pragma unroll
        for (int s = 0; s < 4; s++) acc = __fadd_rn(acc, T[s * ks + ((v.x >> (8 * s)) & 0xff)]);
#pragma unroll
        for (int s = 0; s < 4; s++) acc = __fadd_rn(acc, T[(s + 4) * ks + ((v.y >> (8 * s)) & 0xff)]);
    } else if constexpr (M == 16) {
        uint4 v = __ldg(reinterpret_cast<const uint4*>(row));
        const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int g = 0; g < 4; g++)
#pragma unroll
            for (int s = 0; s < 4; s++) acc = __fadd_rn(acc, T[(4 * g + s) * ks + ((w4[g] >> (8 * s)) & 0xff)]);
    } else {
        for (int s = 0; s < m; s++) acc = __fadd_rn(acc, T[s * ks + row[s]]);
    }
    return acc;
}

// last j with prefix[j] <= pos
__device__ __forceinline__ int probe_of(const uint32_t* prefix, int w, uint32_t pos) {
    int lo = 0, hi = w;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int32_t pos_to_id(const DevIndex& ix, const uint32_t* prefix, const int* plist, int w,
                                             uint32_t pos) {
    int j = probe_of(prefix, w, pos);
    int l = plist[j];
    return ix.ids[ix.list_beg[l] + (int64_t)(pos - prefix[j])];
}

// After the ADC top-k (best[0..nbest) sorted): write the results, or run the
// exact re-rank of the kl candidates (ivf_search.cpp:113-134) and write k.
// xq holds the query (re-rank needs it). Uniform control flow.
__device__ inline void scan_epilogue(const DevIndex& ix, const ScanArgs& a, TopKSmem& s, int q, const uint32_t* prefix,
                              const int* plist, int* cand, const float* xq, int w) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int kq = query_k(a, q);
    const int64_t oq = query_out(a, q);
    const int nb = *s.nbest;
    const float inf = __int_as_float(0x7f800000);
    if (!(a.flags & SCAN_RERANK)) {
        if (a.flags & SCAN_OUT_PACKED) {
            const int64_t o = a.out_start[q];
            for (int c = tid; c < nb; c += nt) {
                a.out_ids[o + c] = pos_to_id(ix, prefix, plist, w, key_payload(s.best[c]));
                a.out_dis[o + c] = key_dist(s.best[c]);
            }
        } else {
            for (int c = tid; c < kq; c += nt) {
                a.out_ids[oq + c] = c < nb ? pos_to_id(ix, prefix, plist, w, key_payload(s.best[c])) : -1;
                a.out_dis[oq + c] = c < nb ? key_dist(s.best[c]) : inf;
            }
        }
        return;
    }
    for (int c = tid; c < nb; c += nt) cand[c] = pos_to_id(ix, prefix, plist, w, key_payload(s.best[c]));
    __syncthreads();
    const int kr = min(kq, nb);
    if (kr > 0) {
        topk_init(s, kr);
        const double qn = a.qnorm[q];
        const int d = ix.d;
        for (int c0 = 0; c0 < nb; c0 += nt) {
            const int c = c0 + tid;
            const bool valid = c < nb;
            float dist = 0.0f;
            if (valid) {
                const int32_t id = cand[c];
                const float* v = ix.base + (int64_t)id * d;
                float dot = 0.0f;
                if ((d & 3) == 0) {  // rows are 16-byte aligned: vector loads, same order
                    const float4* v4 = reinterpret_cast<const float4*>(v);
                    for (int l = 0; l < d / 4; l++) {
                        const float4 b = __ldg(v4 + l);
                        dot = __fadd_rn(dot, __fmul_rn(b.x, xq[4 * l]));
                        dot = __fadd_rn(dot, __fmul_rn(b.y, xq[4 * l + 1]));
                        dot = __fadd_rn(dot, __fmul_rn(b.z, xq[4 * l + 2]));
                        dot = __fadd_rn(dot, __fmul_rn(b.w, xq[4 * l + 3]));
                    }
                } else {
                    dot = dot_seq(v, xq, d);
                }
                dist = expansion_from(qn, ix.base_norm[id], dot);
            }
            topk_offer(s, make_key(dist, (uint32_t)c), valid);
            topk_round_end(s, nt);
        }
        topk_finish(s);
    }
    for (int c = tid; c < kq; c += nt) {
        a.out_ids[oq + c] = c < kr ? cand[key_payload(s.best[c])] : -1;
        a.out_dis[oq + c] = c < kr ? key_dist(s.best[c]) : inf;
    }
}

}  // namespace gbivf
