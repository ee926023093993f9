// Persistent, register-codebook IVF-PQ scan for d = 128, ks = 256 and
// m in {4, 8, 16} (the shapes of the reference's runs: SIFT-like d = 128,
// 256-centroid sub-quantizers, sequential/pq-utils/pq_new.cpp:35).
//
// One CTA of 512 threads per SM pulls queries from a device work counter.
// The whole PQ codebook (m x 256 x ds = 32768 floats) lives in registers:
// thread t owns table entries e = t + 512 i (i < m/2), i.e. 64 centroid
// floats, loaded once per launch. For each probed list of a query the block
//   1. forms the residual r = x - c_list in shared memory (bsxfunMINUS),
//   2. computes the m sub-norms of r,
//   3. builds the m x 256 table from registers -- per entry a sequential
//      float dot product and the reference's norm sum (exact_round.cuh),
//      no memory traffic for the centroids,
//   4. streams the list's codes (8/16-byte vector loads) through the ADC sum
//      and the threshold filter of the block top-k.
// The top-k buffer is sized so that a whole list fits: the capacity check is
// made once per list at a barrier that exists anyway, and the scan loop runs
// without block barriers. Results and the optional re-rank are shared with
// the general kernel (scan_common.cuh).
#include "exact_round.cuh"
#include "scan_common.cuh"

namespace gbivf {

constexpr int SP_NT = 512;
constexpr int SP_UNROLL = 4;
constexpr int SP_BCAP = 8192;   // candidate buffer (64 KB)
constexpr int SP_EARLY = 2048;  // flush once this many are buffered before k are known

template <int M, bool DIRECT>
__global__ void __launch_bounds__(SP_NT, 1) ivf_scan_persistent_kernel(DevIndex ix, ScanArgs a, ScanSmem L, int kcap) {
    constexpr int D = 128, KS = 256, DS = D / M, E = M * KS / SP_NT;
    static_assert(E * SP_NT == M * KS, "entries must divide evenly");
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem + L.off_best);
    u64* tmp = reinterpret_cast<u64*>(smem + L.off_tmp);
    u64* buf = reinterpret_cast<u64*>(smem + L.off_buf);
    u64* thresh = reinterpret_cast<u64*>(smem + L.off_thresh);
    float* table = reinterpret_cast<float*>(smem + L.off_table);
    float* xq = reinterpret_cast<float*>(smem + L.off_xq);
    float* r = reinterpret_cast<float*>(smem + L.off_r);
    float* rn = reinterpret_cast<float*>(smem + L.off_rn);
    uint32_t* prefix = reinterpret_cast<uint32_t*>(smem + L.off_prefix);
    int* plist = reinterpret_cast<int*>(smem + L.off_plist);
    int* cand = reinterpret_cast<int*>(smem + L.off_cand);
    int* cnt = reinterpret_cast<int*>(smem + L.off_cnt);
    int* qslot = reinterpret_cast<int*>(smem + L.off_misc);
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, SP_BCAP};

    const int tid = threadIdx.x, w = a.w;
    const bool src_res = a.flags & SCAN_SRC_RESIDUAL;
    const int kk = (a.flags & SCAN_RERANK) ? a.kl : a.k;

    // this thread's slice of the codebook
    float cen[E][DS];
    float nhi[E], nlo[E];
#pragma unroll
    for (int i = 0; i < E; i++) {
        const int e = tid + i * SP_NT;
        const float4* src = reinterpret_cast<const float4*>(ix.pq + (int64_t)e * DS);
#pragma unroll
        for (int v = 0; v < DS / 4; v++) {
            float4 x = __ldg(src + v);
            cen[i][4 * v] = x.x;
            cen[i][4 * v + 1] = x.y;
            cen[i][4 * v + 2] = x.z;
            cen[i][4 * v + 3] = x.w;
        }
        if (!DIRECT) {
            nhi[i] = __ldg(ix.pq_hi + e);
            nlo[i] = __ldg(ix.pq_lo + e);
        }
    }

    for (;;) {
        if (tid == 0) *qslot = atomicAdd(a.queue, 1);
        __syncthreads();
        const int q = *qslot;
        if (q >= a.nq) break;
        if (!src_res && tid < D) xq[tid] = a.queries[(int64_t)q * D + tid];
        if (tid == 0) {
            uint32_t acc = 0;
            for (int j = 0; j < w; j++) {
                int l = a.probes[(int64_t)q * w + j];
                plist[j] = l;
                prefix[j] = acc;
                acc += (l >= 0) ? (uint32_t)ix.list_len[l] : 0u;
            }
            prefix[w] = acc;
        }
        topk_init(s, kk);

        for (int j = 0; j < w; j++) {
            const int l = plist[j];
            if (l < 0) continue;
            // 1. residual
            if (tid < D)
                r[tid] = src_res ? a.residual[((int64_t)q * w + j) * D + tid]
                                 : __fsub_rn(xq[tid], ix.coa[(int64_t)l * D + tid]);
            __syncthreads();
            // 2. sub-norms; everyone reads the buffer count (all appends of the
            //    previous list happened before the barrier above)
            if (!DIRECT && tid < M) rn[tid] = norm_f_seq(r + tid * DS, DS);
            const int nb = *s.nbuf;
            __syncthreads();
            // 3. table from the register codebook
#pragma unroll
            for (int i = 0; i < E; i++) {
                const int e = tid + i * SP_NT;
                const int sq = e / KS;
                const float* rs = r + sq * DS;
                float v;
                if (DIRECT) {
                    v = 0.0f;
#pragma unroll
                    for (int t = 0; t < DS; t++) {
                        float df = __fsub_rn(rs[t], cen[i][t]);
                        v = __fadd_rn(v, __fmul_rn(df, df));
                    }
                } else {
                    float dot = 0.0f;
#pragma unroll
                    for (int t = 0; t < DS; t++) dot = __fadd_rn(dot, __fmul_rn(rs[t], cen[i][t]));
                    const float c0 = add_norms_rn(ix.pq_norm + e, nhi[i], nlo[i], rn[sq]);
                    v = __fadd_rn(__fmul_rn(-2.0f, dot), c0);
                }
                table[e] = v;
            }
            const int len = ix.list_len[l];
            const bool flush_now = (nb + len > SP_BCAP) || (*s.nbest < kk && nb >= SP_EARLY);
            __syncthreads();
            if (flush_now) topk_flush(s, nb);
            // 4. ADC scan of the list
            const uint8_t* codes = ix.codes + ix.list_beg[l] * (int64_t)M;
            const uint32_t pos0 = prefix[j];
            const bool fits = len <= SP_BCAP - (flush_now ? 0 : nb);
            for (int i0 = 0; i0 < len; i0 += SP_NT * SP_UNROLL) {
                float dist[SP_UNROLL];
#pragma unroll
                for (int u = 0; u < SP_UNROLL; u++) {
                    const int i = i0 + u * SP_NT + tid;
                    dist[u] = i < len ? adc_row<M>(codes + (int64_t)i * M, table, M, KS) : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < SP_UNROLL; u++) {
                    const int i = i0 + u * SP_NT + tid;
                    topk_offer(s, make_key(dist[u], pos0 + (uint32_t)i), i < len);
                }
                if (!fits) topk_round_end(s, SP_NT * SP_UNROLL);
            }
        }
        topk_finish(s);
        scan_epilogue(ix, a, s, q, prefix, plist, cand, xq);
        __syncthreads();
    }
}

bool scan_persistent_supported(const DevIndex& ix, const ScanArgs& a) {
    const int kk = (a.flags & SCAN_RERANK) ? a.kl : a.k;
    const bool m_ok = ix.m == 4 || ix.m == 8 || ix.m == 16;
    return ix.d == 128 && ix.ks == 256 && m_ok && std::max(kk, a.k) <= 1024 && a.queue != nullptr &&
           ix.pq_hi != nullptr && !((a.flags & SCAN_SRC_RESIDUAL) && (a.flags & SCAN_RERANK));
}

template <int M, bool DIRECT>
static cudaError_t launch_sp(const DevIndex& ix, const ScanArgs& a, int num_sms, cudaStream_t st) {
    const int kk = (a.flags & SCAN_RERANK) ? a.kl : a.k;
    const int kcap = pow2_at_least(std::max(std::max(kk, a.k), 2));
    ScanSmem L = scan_smem_layout(M, 256, 128, a.w, kcap, SP_BCAP);
    auto kern = ivf_scan_persistent_kernel<M, DIRECT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SP_NT, L.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = std::min(a.nq, num_sms * per_sm);
    e = cudaMemsetAsync(a.queue, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, SP_NT, L.total, st>>>(ix, a, L, kcap);
    return cudaGetLastError();
}

cudaError_t launch_scan_persistent(const DevIndex& ix, const ScanArgs& a, int num_sms, cudaStream_t st) {
    if (a.nq <= 0) return cudaSuccess;
    if (!scan_persistent_supported(ix, a)) return cudaErrorNotSupported;
    const bool direct = a.flags & SCAN_TABLE_DIRECT;
    switch (ix.m) {
        case 4: return direct ? launch_sp<4, true>(ix, a, num_sms, st) : launch_sp<4, false>(ix, a, num_sms, st);
        case 8: return direct ? launch_sp<8, true>(ix, a, num_sms, st) : launch_sp<8, false>(ix, a, num_sms, st);
        default: return direct ? launch_sp<16, true>(ix, a, num_sms, st) : launch_sp<16, false>(ix, a, num_sms, st);
    }
}

}  // namespace gbivf
