// GB300 (sm_103a) kernels of the plain FP32 IVF-PQ search path.
//
// Reference path (rafaelms101/mestrado, sequential/ivf_pq/ivf_search.cpp:9-203):
//   knn_full (coarse, k = w)           -> coarse_dist_kernel + coarse_select_kernel
//   bsxfunMINUS + compute_cross_distances (m x ks tables)
//   + sumidxtab2 (ADC) + k_min (kl)     -> ivf_scan_kernel (fused, one CTA per query)
//   RERANK knn_full over kl candidates  -> tail of ivf_scan_kernel
// and parallel2's core_gpu (parallel2/ivf_pq/mycuda.cu:28-188) through the
// SCAN_SRC_RESIDUAL | SCAN_TABLE_DIRECT | SCAN_OUT_PACKED mode.
//
// All arithmetic mirrors the reference rounding (see common.cuh); ties are
// broken by (distance, payload) keys (block_topk.cuh).
#include <algorithm>

#include "exact_round.cuh"
#include "f32x2.cuh"
#include "scan_common.cuh"

namespace gbivf {

// ---------------------------------------------------------------------------
// norms
// ---------------------------------------------------------------------------

__global__ void norm_d_kernel(const float* __restrict__ x, int64_t n, int d, double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = x + i * d;
    double s = 0.0;
    for (int l = 0; l < d; l++) s = __dadd_rn(s, (double)__fmul_rn(r[l], r[l]));
    out[i] = s;
}

__global__ void norm_f_kernel(const float* __restrict__ x, int64_t n, int d, float* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = norm_f_seq(x + i * d, d);
}

cudaError_t launch_norm_d(const float* x, int64_t n, int d, double* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    norm_d_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(x, n, d, out);
    return cudaGetLastError();
}

cudaError_t launch_norm_f(const float* x, int64_t n, int d, float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    norm_f_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(x, n, d, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// coarse distances: 128 x 128 output tile per CTA, 8 x 8 per thread (rows
// 4ty..4ty+3 and 64+4ty.., columns likewise with tx), K chunks of 16 staged in
// shared memory (the next chunk is loaded into registers while the current one
// is used). Every output is one sequential dot product over l = 0..d-1 (the
// netlib sgemm order), two outputs per instruction: each product is
// fma(q, c, -0) with a -0 the compiler cannot see (so it rounds once, like the
// reference's multiply, and is not fused into the add), each sum a packed add.
// Epilogue: the reference's constant term (float)(double ||q||^2 + float
// ||c||^2) by the exact FP32 form of that sum (exact_round.cuh; GB300's FP64
// rate is a small fraction of FP32), then -2 dot + c.
// ---------------------------------------------------------------------------

constexpr int CD_TILE = 128, CD_K = 16;

__global__ void __launch_bounds__(256) coarse_dist_kernel(
    const float* __restrict__ X, int nq, const float* __restrict__ Cc, int C, int d,
    const double* __restrict__ qnorm, const float* __restrict__ cnorm, float* __restrict__ out,
    CoarseFilter flt, float neg_zero) {
    __shared__ __align__(16) float Xs[CD_K][CD_TILE];
    __shared__ __align__(16) float Cs[CD_K][CD_TILE];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int q0 = blockIdx.y * CD_TILE, c0 = blockIdx.x * CD_TILE;
    // 16-byte loads where every row starts on a 16-byte boundary
    const bool vec = (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(Cc)) & 15) == 0;
    const f2_t nz2 = f2_pack(neg_zero, neg_zero);
    f2_t acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = f2_pack(0.0f, 0.0f);

    // staging: element (row r, 4 columns from l0 + 4v) for e = tid + 256 h, r = e % 128, v = e / 128
    float4 px[2], pc[2];
    auto fetch = [&](int l0) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int e = tid + 256 * h, r = e & 127, l = l0 + 4 * (e >> 7);
            const int qr = q0 + r, cr = c0 + r;
            float4 x = make_float4(0.0f, 0.0f, 0.0f, 0.0f), c = x;
            if (vec) {
                if (qr < nq && l < d) x = __ldg(reinterpret_cast<const float4*>(X + (int64_t)qr * d + l));
                if (cr < C && l < d) c = __ldg(reinterpret_cast<const float4*>(Cc + (int64_t)cr * d + l));
            } else {
                float xv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, cv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (qr < nq && l + k < d) xv[k] = X[(int64_t)qr * d + l + k];
                    if (cr < C && l + k < d) cv[k] = Cc[(int64_t)cr * d + l + k];
                }
                x = make_float4(xv[0], xv[1], xv[2], xv[3]);
                c = make_float4(cv[0], cv[1], cv[2], cv[3]);
            }
            px[h] = x;
            pc[h] = c;
        }
    };
    fetch(0);
    for (int l0 = 0; l0 < d; l0 += CD_K) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int e = tid + 256 * h, r = e & 127, k = 4 * (e >> 7);
            Xs[k][r] = px[h].x;
            Xs[k + 1][r] = px[h].y;
            Xs[k + 2][r] = px[h].z;
            Xs[k + 3][r] = px[h].w;
            Cs[k][r] = pc[h].x;
            Cs[k + 1][r] = pc[h].y;
            Cs[k + 2][r] = pc[h].z;
            Cs[k + 3][r] = pc[h].w;
        }
        __syncthreads();
        if (l0 + CD_K < d) fetch(l0 + CD_K);
        const int lmax = min(CD_K, d - l0);
        for (int l = 0; l < lmax; l++) {
            const float4 a0 = reinterpret_cast<const float4*>(Xs[l])[ty];
            const float4 a1 = reinterpret_cast<const float4*>(Xs[l])[16 + ty];
            const float4 b0 = reinterpret_cast<const float4*>(Cs[l])[tx];
            const float4 b1 = reinterpret_cast<const float4*>(Cs[l])[16 + tx];
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const f2_t b[4] = {f2_pack(b0.x, b0.y), f2_pack(b0.z, b0.w), f2_pack(b1.x, b1.y), f2_pack(b1.z, b1.w)};
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const f2_t aa = f2_pack(a[i], a[i]);
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = f2_add(acc[i][j], f2_fma(aa, b[j], nz2));
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int q = q0 + (i < 4 ? 4 * ty + i : 64 + 4 * ty + i - 4);
        if (q >= nq) continue;
        const double qn = qnorm[q];
        float qhi, qlo;
        split_norm_dev(qn, &qhi, &qlo);
        const float T = flt.thr ? flt.thr[q] : 0.0f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float dot[2];
            f2_unpack(acc[i][j], dot[0], dot[1]);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int c = c0 + (j < 2 ? 4 * tx + 2 * j + h : 64 + 4 * tx + 2 * (j - 2) + h);
                if (c >= C) continue;
                const float cst = add_norms_rn(qnorm + q, qhi, qlo, cnorm[c]);
                const float dist = __fadd_rn(__fmul_rn(-2.0f, dot[h]), cst);
                if (flt.thr) {
                    // filtered: append the centroids within the query's bound
                    if (dist <= T) {
                        const int slot = atomicAdd(&flt.ncand[q], 1);
                        if (slot < flt.cap) flt.cand[(int64_t)q * flt.cap + slot] = c;
                    }
                } else {
                    out[(int64_t)q * C + c] = dist;
                }
            }
        }
    }
}

cudaError_t launch_coarse_dist(const DevIndex& ix, const float* q, const double* qnorm, int nq,
                               float* out, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    dim3 grid((ix.C + CD_TILE - 1) / CD_TILE, (nq + CD_TILE - 1) / CD_TILE);
    coarse_dist_kernel<<<grid, 256, 0, st>>>(q, nq, ix.coa, ix.C, ix.d, qnorm, ix.coa_norm, out, CoarseFilter{},
                                             -0.0f);
    return cudaGetLastError();
}

cudaError_t launch_coarse_dist_filter(const DevIndex& ix, const float* q, const double* qnorm, int nq,
                                      const CoarseFilter& f, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    if (!f.thr || !f.ncand || !f.cand || f.cap <= 0) return cudaErrorInvalidValue;
    dim3 grid((ix.C + CD_TILE - 1) / CD_TILE, (nq + CD_TILE - 1) / CD_TILE);
    coarse_dist_kernel<<<grid, 256, 0, st>>>(q, nq, ix.coa, ix.C, ix.d, qnorm, ix.coa_norm, nullptr, f, -0.0f);
    return cudaGetLastError();
}

__global__ void id_range_kernel(const int32_t* __restrict__ ids, int64_t n, int* __restrict__ range) {
    int lo = 0x7fffffff, hi = (int)0x80000000;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        lo = min(lo, ids[i]);
        hi = max(hi, ids[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&range[0], lo);
        atomicMax(&range[1], hi);
    }
}

cudaError_t launch_id_range(const int32_t* ids, int64_t n, int* range, cudaStream_t st) {
    int* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 2 * sizeof(int));
    if (e != cudaSuccess) return e;
    const int init[2] = {0x7fffffff, (int)0x80000000};
    e = cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        id_range_kernel<<<1024, 256, 0, st>>>(ids, n, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(range, d, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    return e;
}

// one CTA per list: copy its rows from the caller's order into the padded row layout
__global__ void scatter_rows_kernel(const uint8_t* __restrict__ src, const int64_t* __restrict__ off,
                                    const int64_t* __restrict__ beg, int width, uint8_t* __restrict__ dst) {
    const int l = blockIdx.x;
    const int64_t n = (off[l + 1] - off[l]) * width;
    const uint8_t* s = src + off[l] * width;
    uint8_t* d = dst + beg[l] * width;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
}

cudaError_t launch_scatter_rows(const uint8_t* src, const int64_t* off, const int64_t* beg, int C, int width,
                                uint8_t* dst, cudaStream_t st) {
    if (C <= 0) return cudaSuccess;
    scatter_rows_kernel<<<C, 256, 0, st>>>(src, off, beg, width, dst);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// coarse k-min: one CTA per query over its row of C distances
// ---------------------------------------------------------------------------

constexpr int CS_NT = 128, CS_ITEMS = 8;

__global__ void __launch_bounds__(CS_NT) coarse_select_kernel(
    const float* __restrict__ dist, int C, int w, int kcap, int bcap,
    int32_t* __restrict__ coaidx, float* __restrict__ coadis) {
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem);
    u64* tmp = best + kcap;
    u64* buf = tmp + kcap;
    u64* thresh = buf + bcap;
    unsigned char* work = reinterpret_cast<unsigned char*>(thresh + 1);
    int* cnt = reinterpret_cast<int*>(work + TOPK_WORK_BYTES);
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, bcap, work};
    const int q = blockIdx.x, tid = threadIdx.x;
    const float* row = dist + (int64_t)q * C;
    topk_init(s, w);
    for (int i0 = 0; i0 < C; i0 += CS_NT * CS_ITEMS) {
#pragma unroll
        for (int it = 0; it < CS_ITEMS; it++) {
            int c = i0 + it * CS_NT + tid;
            bool valid = c < C;
            float v = valid ? row[c] : 0.0f;
            topk_offer(s, make_key(v, (uint32_t)c), valid);
        }
        topk_round_end(s, CS_NT * CS_ITEMS);
    }
    topk_finish(s);
    const int nb = *s.nbest;
    for (int j = tid; j < w; j += CS_NT) {
        coaidx[(int64_t)q * w + j] = j < nb ? (int32_t)key_payload(best[j]) : -1;
        coadis[(int64_t)q * w + j] = j < nb ? key_dist(best[j]) : __int_as_float(0x7f800000);
    }
}

cudaError_t launch_coarse_select(const float* dist, int nq, int C, int w, int32_t* coaidx,
                                 float* coadis, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    int kcap = pow2_at_least(std::max(w, 2));
    int bcap = pow2_at_least(std::max(2 * CS_NT * CS_ITEMS, kcap));
    size_t sm = sizeof(u64) * (2 * kcap + bcap + 1) + TOPK_WORK_BYTES + 2 * sizeof(int);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(coarse_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    coarse_select_kernel<<<nq, CS_NT, sm, st>>>(dist, C, w, kcap, bcap, coaidx, coadis);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fused scan: per query (one CTA), for each probed list: residual, m x ks
// table in shared memory, ADC over the list's codes, streaming top-k; then
// the optional exact re-rank of the kl best. General shapes (any d, m, ks).
// ---------------------------------------------------------------------------

constexpr int SC_NT = 256, SC_ITEMS = 4;

template <int M>
__global__ void __launch_bounds__(SC_NT) ivf_scan_kernel(DevIndex ix, ScanArgs a, ScanSmem L, int kcap, int bcap) {
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
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, bcap, smem + L.off_work};

    const int q = blockIdx.x, tid = threadIdx.x;
    const int d = ix.d, m = ix.m, ks = ix.ks, ds = ix.ds, w = a.w;
    const bool src_res = a.flags & SCAN_SRC_RESIDUAL;
    const bool direct = a.flags & SCAN_TABLE_DIRECT;
    const bool rerank = a.flags & SCAN_RERANK;

    if (!src_res)
        for (int i = tid; i < d; i += SC_NT) xq[i] = a.queries[(int64_t)q * d + i];
    const int wq = query_w(a, q);  // probes used by this query (w is the row stride)
    if (tid == 0) {
        uint32_t acc = 0;
        for (int j = 0; j < wq; j++) {
            int l = a.probes[(int64_t)q * w + j];
            plist[j] = l;
            prefix[j] = acc;
            acc += (l >= 0) ? (uint32_t)ix.list_len[l] : 0u;
        }
        prefix[wq] = acc;
    }
    const int kk = rerank ? a.kl : query_k(a, q);
    topk_init(s, kk);

    for (int j = 0; j < wq; j++) {
        const int l = plist[j];
        if (l < 0) continue;
        // residual (bsxfunMINUS) or given residual row
        if (src_res) {
            const float* src = a.residual + ((int64_t)q * w + j) * d;
            for (int i = tid; i < d; i += SC_NT) r[i] = src[i];
        } else {
            const float* cen = ix.coa + (int64_t)l * d;
            for (int i = tid; i < d; i += SC_NT) r[i] = __fsub_rn(xq[i], cen[i]);
        }
        __syncthreads();
        if (!direct)
            for (int sq = tid; sq < m; sq += SC_NT) rn[sq] = norm_f_seq(r + sq * ds, ds);
        __syncthreads();
        // m x ks table (compute_cross_distances(ds, 1, ks, r_s, C_s))
        for (int e = tid; e < m * ks; e += SC_NT) {
            const int sq = e / ks;
            const float* cen = ix.pq + (int64_t)e * ds;
            const float* rs = r + sq * ds;
            table[e] = direct ? direct_seq(rs, cen, ds) : expansion_from(ix.pq_norm[e], rn[sq], dot_seq(rs, cen, ds));
        }
        __syncthreads();
        // ADC scan (sumidxtab2) with streaming top-k
        const int len = ix.list_len[l];
        const uint8_t* codes = ix.codes + ix.list_beg[l] * (int64_t)m;
        const uint32_t pos0 = prefix[j];
        for (int i0 = 0; i0 < len; i0 += SC_NT * SC_ITEMS) {
#pragma unroll
            for (int it = 0; it < SC_ITEMS; it++) {
                const int i = i0 + it * SC_NT + tid;
                const bool valid = i < len;
                float dist = 0.0f;
                if (valid) dist = adc_row<M>(codes + (int64_t)i * m, table, m, ks);
                topk_offer(s, make_key(dist, pos0 + (uint32_t)i), valid);
            }
            topk_round_end(s, SC_NT * SC_ITEMS);
        }
        __syncthreads();
    }
    topk_finish(s);
    scan_epilogue(ix, a, s, q, prefix, plist, cand, xq, wq);
}

template <int M>
static cudaError_t launch_scan_m(const DevIndex& ix, const ScanArgs& a, cudaStream_t st) {
    const bool rerank = a.flags & SCAN_RERANK;
    const int kk = rerank ? a.kl : a.k;
    int kcap = pow2_at_least(std::max(std::max(kk, a.k), 2));
    int bcap = pow2_at_least(std::max(2048, kcap));
    ScanSmem L = scan_smem_layout(ix.m, ix.ks, ix.d, a.w, kcap, bcap);
    auto kern = ivf_scan_kernel<M>;
    if (L.total > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
        if (e != cudaSuccess) return e;
    }
    kern<<<a.nq, SC_NT, L.total, st>>>(ix, a, L, kcap, bcap);
    return cudaGetLastError();
}

cudaError_t launch_scan(const DevIndex& ix, const ScanArgs& a, cudaStream_t st) {
    if (a.nq <= 0) return cudaSuccess;
    switch (ix.m) {
        case 4: return launch_scan_m<4>(ix, a, st);
        case 8: return launch_scan_m<8>(ix, a, st);
        case 16: return launch_scan_m<16>(ix, a, st);
        default: return launch_scan_m<0>(ix, a, st);
    }
}

}  // namespace gbivf
