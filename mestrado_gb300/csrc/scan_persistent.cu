// Persistent, register-codebook IVF-PQ scan for d = 128, ks = 256 and
// m in {4, 8, 16} (the shapes of the reference's runs: SIFT-like d = 128,
// 256-centroid sub-quantizers, sequential/pq-utils/pq_new.cpp:35).
//
// One CTA of 512 threads per SM pulls queries from a device work counter.
// The whole PQ codebook (m x 256 x ds = 32768 floats) lives in registers:
// thread t owns the E = m*256/512 consecutive table entries of one
// sub-quantizer, i.e. 64 centroid floats, loaded once per launch. For each
// probed list of a query the block
//   1. forms the residual r = x - c_list in shared memory (bsxfunMINUS),
//   2. computes the m sub-norms of r,
//   3. builds the m x 256 table from registers, two entries per packed
//      instruction -- exact form: per entry a sequential float dot product and
//      the reference's norm sum (exact_round.cuh); precision form: FP16
//      entries by fused multiply-adds -- with no memory traffic for centroids,
//   4. streams the list's codes (16-byte groups of rows) through the ADC sum
//      and the threshold filter of the block top-k.
// The top-k buffer is sized so that a whole list fits: the capacity check is
// made once per list at a barrier that exists anyway, and the scan loop runs
// without block barriers. Results and the optional re-rank are shared with
// the general kernel (scan_common.cuh).
#include <cuda_fp16.h>

#include "exact_round.cuh"
#include "f32x2.cuh"
#include "scan_common.cuh"


namespace gbivf {

constexpr int SP_BCAP = 8192;   // candidate buffer (64 KB)
constexpr int SP_SOFT = 2048;   // flush at a list boundary once this many are buffered
constexpr int SP_RCH = 16;      // residuals formed per chunk of probes
// Precision form: the first chunk of each probe's code rows is copied into shared memory
// SP_AHEAD probes ahead (cp.async, per thread: a thread copies exactly the 16-byte groups it later
// scans, so it only waits for its own copies, with no barrier), in SP_NS rotating stages. Its
// probes are short (most probed lists are, and its tables take a few instructions), often shorter
// than a memory round trip: one probe of lead left the copy exposed at the start of the scan. The
// exact form loads its first chunk into registers at the start of its (long) table build instead.
constexpr int SP_AHEAD = 2;
constexpr int SP_NS = SP_AHEAD + 1;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most n of this thread's committed groups are still in flight
template <int n>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(n) : "memory"); }

// one code row as a vector load
template <int M> struct CodeRow;
template <> struct CodeRow<4> { using T = uint32_t; };
template <> struct CodeRow<8> { using T = uint2; };
template <> struct CodeRow<16> { using T = uint4; };

template <int M>
__device__ __forceinline__ typename CodeRow<M>::T load_row(const uint8_t* p) {
    return __ldg(reinterpret_cast<const typename CodeRow<M>::T*>(p));
}

// byte s of v, zero-extended (one byte-permute)
__device__ __forceinline__ uint32_t byte_of(uint32_t v, int s) { return __byte_perm(v, 0u, 0x4440u | (uint32_t)s); }

__device__ __forceinline__ float adc4(float acc, uint32_t v, const float* T) {
#pragma unroll
    for (int s = 0; s < 4; s++) acc = __fadd_rn(acc, T[s * 256 + byte_of(v, s)]);
    return acc;
}

// acc = 0; acc += T[s][code[s]] in s order (sumidxtab2, ivf_search.cpp:189-200)
__device__ __forceinline__ float adc_sum(uint32_t v, const float* T) { return adc4(0.0f, v, T); }
__device__ __forceinline__ float adc_sum(uint2 v, const float* T) { return adc4(adc4(0.0f, v.x, T), v.y, T + 1024); }
__device__ __forceinline__ float adc_sum(uint4 v, const float* T) {
    return adc4(adc4(adc4(adc4(0.0f, v.x, T), v.y, T + 1024), v.z, T + 2048), v.w, T + 3072);
}

// Precision form of the scan: approximate tables held in FP16 (scaled by 2^-2
// so that partial distances up to 2^18 fit; saturating), summed in FP32 with the
// mixed-precision add (add.rn.f32.f16, sm_100 and later), scaled back by 4.
constexpr float SP_T16_SCALE = 0.25f;

__device__ __forceinline__ float add_f16(float acc, const __half* p) {
    const unsigned short h = *reinterpret_cast<const unsigned short*>(p);
    asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(acc) : "h"(h));
    return acc;
}
__device__ __forceinline__ float adc4h(float acc, uint32_t v, const __half* T) {
#pragma unroll
    for (int s = 0; s < 4; s++) acc = add_f16(acc, T + s * 256 + byte_of(v, s));
    return acc;
}
__device__ __forceinline__ float adc_sum16(uint32_t v, const __half* T) { return adc4h(0.0f, v, T) * 4.0f; }
__device__ __forceinline__ float adc_sum16(uint2 v, const __half* T) {
    return adc4h(adc4h(0.0f, v.x, T), v.y, T + 1024) * 4.0f;
}
__device__ __forceinline__ float adc_sum16(uint4 v, const __half* T) {
    return adc4h(adc4h(adc4h(adc4h(0.0f, v.x, T), v.y, T + 1024), v.z, T + 2048), v.w, T + 3072) * 4.0f;
}
// The ADC loop reads code rows in 16-byte groups (G = 16 / M rows: 4 at m = 4, 2 at m = 8, 1 at
// m = 16), so that a thread's bounds checks, filter vote and loop control are paid once per group,
// not once per row. List starts and the end of the code array are padded to whole groups.
__device__ __forceinline__ uint4 load_group(const uint8_t* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// ADC distance of row r (0 <= r < 16 / M) of a group
template <int M, bool MIXED>
__device__ __forceinline__ float group_row_dist(const uint4& c, int r, const float* T, const __half* T16) {
    if constexpr (M == 16) {
        return MIXED ? adc_sum16(c, T16) : adc_sum(c, T);
    } else if constexpr (M == 8) {
        const uint2 v = r == 0 ? make_uint2(c.x, c.y) : make_uint2(c.z, c.w);
        return MIXED ? adc_sum16(v, T16) : adc_sum(v, T);
    } else {
        const uint32_t v = r == 0 ? c.x : (r == 1 ? c.y : (r == 2 ? c.z : c.w));
        return MIXED ? adc_sum16(v, T16) : adc_sum(v, T);
    }
}

// two FP32 values as an FP16 pair (lo in the low half, the lower address), saturating
__device__ __forceinline__ uint32_t f16x2_sat(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

template <int M, bool DIRECT, int NT, bool MIXED = false>
__global__ void __launch_bounds__(NT, 1) ivf_scan_persistent_kernel(DevIndex ix, ScanArgs a, ScanSmem L, int kcap) {
    constexpr int D = 128, KS = 256, DS = D / M, E = M * KS / NT;
    constexpr int TPS = NT / M;  // threads per sub-quantizer
    constexpr int G = 16 / M;              // code rows per 16-byte group
    constexpr int U = M == 4 ? 1 : 2;      // groups per thread per chunk
    constexpr int CH = NT * U * G;         // code rows per chunk
    // staged groups per thread (precision form; at most 1024 per probe)
    constexpr int US = !MIXED ? 0 : NT * U > 1024 ? 1024 / NT : U;
    static_assert(E * NT == M * KS && E * TPS == KS, "entries must divide evenly");
    static_assert(G * M == 16, "m must be 4, 8 or 16");
    extern __shared__ __align__(16) unsigned char smem[];
    u64* best = reinterpret_cast<u64*>(smem + L.off_best);
    u64* tmp = reinterpret_cast<u64*>(smem + L.off_tmp);
    u64* buf = reinterpret_cast<u64*>(smem + L.off_buf);
    u64* thresh = reinterpret_cast<u64*>(smem + L.off_thresh);
    float* tables = reinterpret_cast<float*>(smem + L.off_table);  // 2 buffers
    float* xq = reinterpret_cast<float*>(smem + L.off_xq);
    float* rr = reinterpret_cast<float*>(smem + L.off_r);    // SP_RCH x D residuals
    float* rn = reinterpret_cast<float*>(smem + L.off_rn);   // SP_RCH x M sub-norms
    uint4* stage = reinterpret_cast<uint4*>(smem + L.off_stage);  // SP_NS x (US x NT) code groups
    uint32_t* prefix = reinterpret_cast<uint32_t*>(smem + L.off_prefix);
    int* plist = reinterpret_cast<int*>(smem + L.off_plist);
    int* cnt = reinterpret_cast<int*>(smem + L.off_cnt);
    int* qslot = reinterpret_cast<int*>(smem + L.off_misc);  // [1] = next query
    TopKSmem s{best, tmp, buf, cnt, cnt + 1, thresh, 0, kcap, SP_BCAP, smem + L.off_work};

    const int tid = threadIdx.x, lane = tid & 31, w = a.w;  // w: the probes row stride
    const bool src_res = a.flags & SCAN_SRC_RESIDUAL;
    const bool rows_out = MIXED || (a.flags & SCAN_REFINE);  // hand off code rows and lists

    // this thread's slice of the codebook: sub-quantizer my_s, centroids
    // my_c0 .. my_c0+E-1 (consecutive, so the table row is one vector store)
    const int my_s = tid / TPS, my_c0 = (tid % TPS) * E;
    // The precision form keeps the same slice as packed pairs of entries (i, i+1) for packed
    // fused multiply-adds, with ||c||^2 / 4 of each entry (a single entry, E = 1, is paired with
    // itself and stored once).
    constexpr int EP = MIXED ? 1 : E, EM = MIXED ? (E + 1) / 2 : 1;
    float cen[EP][DS];
    float nhi[EP], nlo[EP];
    f2_t cen2[EM][DS], cn2[EM];
#pragma unroll
    for (int i = 0; i < (MIXED ? 0 : E); i++) {
        const int e = my_s * KS + my_c0 + i;
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
#pragma unroll
    for (int i = 0; i < (MIXED ? E : 0); i += 2) {
        const int e = my_s * KS + my_c0 + i;
        const float4* s0 = reinterpret_cast<const float4*>(ix.pq + (int64_t)e * DS);
        const int e1 = i + 1 < E ? e + 1 : e;
        const float4* s1 = reinterpret_cast<const float4*>(ix.pq + (int64_t)e1 * DS);
#pragma unroll
        for (int v = 0; v < DS / 4; v++) {
            const float4 x = __ldg(s0 + v), y = __ldg(s1 + v);
            cen2[i / 2][4 * v] = f2_pack(x.x, y.x);
            cen2[i / 2][4 * v + 1] = f2_pack(x.y, y.y);
            cen2[i / 2][4 * v + 2] = f2_pack(x.z, y.z);
            cen2[i / 2][4 * v + 3] = f2_pack(x.w, y.w);
        }
        // exact: a power-of-two scale
        cn2[i / 2] = f2_pack(0.25f * __ldg(ix.pq_hi + e), 0.25f * __ldg(ix.pq_hi + e1));
    }

    if (tid == 0) qslot[1] = atomicAdd(a.queue, 1);
    // the batch, or the subset of it that a.qlist names (its count written by an earlier kernel)
    const int nwork = a.qlist ? *a.nqlist : a.nq;
    for (;;) {
        __syncthreads();
        const int qi = qslot[1];
        if (qi >= nwork) break;
        const int q = a.qlist ? a.qlist[qi] : qi;
        // this query's probe count and result count (uneven batches)
        const int wq = query_w(a, q);
        // its probe lists and their lengths, loaded by all threads at once (one memory round trip
        // instead of two dependent ones per 32 probes); the prefix sums follow, in one warp
        for (int j = tid; j < wq; j += NT) {
            const int l = __ldg(a.probes + (int64_t)q * w + j);
            plist[j] = l;
            prefix[j] = l >= 0 ? (uint32_t)__ldg(ix.list_len + l) : 0u;
        }
        if (!src_res && tid < D) xq[tid] = __ldg(a.queries + (int64_t)q * D + tid);
        __syncthreads();
        if (tid == 0) qslot[1] = atomicAdd(a.queue, 1);  // next query, in flight meanwhile
        const int kq0 = (a.flags & (SCAN_RERANK | SCAN_REFINE)) ? a.kl : query_k(a, q);
        // the precision form keeps alpha * k approximate candidates for the exact re-score
        const int kq = MIXED ? mixed_sel(a, kq0) : kq0;
        // prefix sums of the probe lengths (each lane reads, then overwrites, its own slot)
        if (tid < 32) {
            uint32_t carry = 0;
            for (int j0 = 0; j0 < wq; j0 += 32) {
                const int j = j0 + lane;
                const uint32_t len = j < wq ? prefix[j] : 0u;
                uint32_t incl = len;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                if (j < wq) prefix[j] = carry + incl - len;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (lane == 0) prefix[wq] = carry;
        }
        topk_init(s, kq);
        // buffered keys that trigger a flush at a list boundary: a flush selects among the best kq
        // and the buffer, so with a large kq (the precision form's 4k) a larger buffer amortises it
        const int soft = max(SP_SOFT, min(kq, SP_BCAP / 2));
        // copy probe jj's first chunk of code groups into its stage (one commit group per probe,
        // empty past the last probe, so that the group count stays in step with the probes)
        auto stage_probe = [&](int jj) {
            if constexpr (!MIXED) return;
            const int ll = jj < wq ? plist[jj] : -1;
            if (ll >= 0) {
                const int ngp = (__ldg(ix.list_len + ll) + G - 1) / G;
                const uint8_t* cp = ix.codes + __ldg(ix.list_beg + ll) * (int64_t)M;
                uint4* dst = stage + (jj % SP_NS) * (US * NT);
#pragma unroll
                for (int u = 0; u < US; u++) {
                    const int g = u * NT + tid;
                    if (g < ngp) cp_async16(dst + g, cp + (int64_t)g * 16);
                }
            }
            cp_async_commit();
        };
#pragma unroll
        for (int jj = 0; jj < SP_AHEAD; jj++) stage_probe(jj);


        for (int j = 0; j < wq; j++) {
            const int jr = j % SP_RCH;
            if (jr == 0) {
                // residuals of probes j .. j+SP_RCH-1 (bsxfunMINUS) and their
                // sub-norms (the a-operand norm of compute_cross_distances)
                const int nr = min(SP_RCH, wq - j);
                for (int e = tid; e < nr * D; e += NT) {
                    const int p = e / D, x = e % D, l = plist[j + p];
                    float v = 0.0f;
                    if (l >= 0)
                        v = src_res ? __ldg(a.residual + ((int64_t)q * w + j + p) * D + x)
                                    : __fsub_rn(xq[x], __ldg(ix.coa + (int64_t)l * D + x));
                    rr[p * D + x] = v;
                }
                __syncthreads();
                if (!DIRECT)
                    for (int e = tid; e < nr * M; e += NT) rn[e] = norm_f_seq(rr + e * DS, DS);
                __syncthreads();
            }
            stage_probe(j + SP_AHEAD);
            const int l = plist[j];
            if (l < 0) continue;
            const int len = __ldg(ix.list_len + l);
            const int ng = (len + G - 1) / G;  // 16-byte groups of code rows
            const uint8_t* codes = ix.codes + __ldg(ix.list_beg + l) * (int64_t)M;
            uint4 cur[U];
            if constexpr (!MIXED) {
                // first chunk of codes in flight during the table build
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int g = u * NT + tid;
                    cur[u] = g < ng ? load_group(codes + (int64_t)g * 16) : make_uint4(0, 0, 0, 0);
                }
            }
            float* table = tables + (j & 1) * (M * KS);
            __half* table16 = reinterpret_cast<__half*>(tables) + (j & 1) * (M * KS);
            if constexpr (MIXED) {
                // approximate entry, scaled: ||r_s - c||^2 / 4 = ||r_s||^2 / 4 + ||c||^2 / 4 - <r_s, c> / 2,
                // the dot product by packed fused multiply-adds over the register codebook (two
                // entries per instruction), converted to FP16 in pairs with saturation
                f2_t rs2[DS];
                const float4* r4 = reinterpret_cast<const float4*>(rr + jr * D + my_s * DS);
#pragma unroll
                for (int v4 = 0; v4 < DS / 4; v4++) {
                    const float4 x = r4[v4];
                    rs2[4 * v4] = f2_pack(x.x, x.x);
                    rs2[4 * v4 + 1] = f2_pack(x.y, x.y);
                    rs2[4 * v4 + 2] = f2_pack(x.z, x.z);
                    rs2[4 * v4 + 3] = f2_pack(x.w, x.w);
                }
                const float f4 = SP_T16_SCALE * rn[jr * M + my_s];
                const f2_t f42 = f2_pack(f4, f4), mh2 = f2_pack(-2.0f * SP_T16_SCALE, -2.0f * SP_T16_SCALE);
                uint32_t hw[EM];
#pragma unroll
                for (int i = 0; i < EM; i++) {
                    f2_t dt = f2_pack(0.0f, 0.0f);
#pragma unroll
                    for (int t = 0; t < DS; t++) dt = f2_fma(rs2[t], cen2[i][t], dt);
                    float e0, e1;
                    f2_unpack(f2_fma(mh2, dt, f2_add(f42, cn2[i])), e0, e1);
                    hw[i] = f16x2_sat(e0, e1);
                }
                uint32_t* dst = reinterpret_cast<uint32_t*>(table16 + my_s * KS + my_c0);
                if constexpr (E == 8) {
                    *reinterpret_cast<uint4*>(dst) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                } else if constexpr (E == 4) {
                    *reinterpret_cast<uint2*>(dst) = make_uint2(hw[0], hw[1]);
                } else if constexpr (E == 2) {
                    dst[0] = hw[0];
                } else {
                    *reinterpret_cast<unsigned short*>(dst) = (unsigned short)(hw[0] & 0xffffu);
                }
            } else
            // table row segment from the register codebook
            {
                float rs[DS];
                const float4* r4 = reinterpret_cast<const float4*>(rr + jr * D + my_s * DS);
#pragma unroll
                for (int v4 = 0; v4 < DS / 4; v4++) {
                    const float4 x = r4[v4];
                    rs[4 * v4] = x.x;
                    rs[4 * v4 + 1] = x.y;
                    rs[4 * v4 + 2] = x.z;
                    rs[4 * v4 + 3] = x.w;
                }
                const float f = DIRECT ? 0.0f : rn[jr * M + my_s];
                float out[E];
                if constexpr (E % 2 == 0 && !DIRECT) {
                    // Two entries per instruction. The dot products' products are fma(r, c, -0) with
                    // a -0 known only at run time: ptxas contracts a packed multiply feeding a packed
                    // add into a fused multiply-add (measured), which rounds differently from the
                    // reference's separate operations, but it cannot merge two FMAs. The TwoSum of the
                    // norm sum and the final -2 dot + c (-2 dot is exact, so fusing it changes
                    // nothing) need no such guard.
                    const f2_t f2 = f2_pack(f, f), m2 = f2_pack(-2.0f, -2.0f), nz2 = f2_pack(a.neg_zero, a.neg_zero);
#pragma unroll
                    for (int i = 0; i < E; i += 2) {
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
                        const int e = my_s * KS + my_c0 + i;
                        const f2_t c02 = f2_pack(add_norms_finish(ix.pq_norm + e, Sa, ta, f),
                                                 add_norms_finish(ix.pq_norm + e + 1, Sb, tb, f));
                        f2_unpack(f2_add(f2_mul(m2, f2_pack(d0, d1)), c02), out[i], out[i + 1]);
                    }
                } else
#pragma unroll
                for (int i = 0; i < E; i++) {
                    if (DIRECT) {
                        float v = 0.0f;
#pragma unroll
                        for (int t = 0; t < DS; t++) {
                            float df = __fsub_rn(rs[t], cen[i][t]);
                            v = __fadd_rn(v, __fmul_rn(df, df));
                        }
                        out[i] = v;
                    } else {
                        float dot = 0.0f;
#pragma unroll
                        for (int t = 0; t < DS; t++) dot = __fadd_rn(dot, __fmul_rn(rs[t], cen[i][t]));
                        const int e = my_s * KS + my_c0 + i;
                        const float c0 = add_norms_rn(ix.pq_norm + e, nhi[i], nlo[i], f);
                        out[i] = __fadd_rn(__fmul_rn(-2.0f, dot), c0);
                    }
                }
                float* dst = table + my_s * KS + my_c0;
                if constexpr (E % 4 == 0) {
#pragma unroll
                    for (int i = 0; i < E; i += 4)
                        *reinterpret_cast<float4*>(dst + i) = make_float4(out[i], out[i + 1], out[i + 2], out[i + 3]);
                } else if constexpr (E % 2 == 0) {
#pragma unroll
                    for (int i = 0; i < E; i += 2) *reinterpret_cast<float2*>(dst + i) = make_float2(out[i], out[i + 1]);
                } else {
#pragma unroll
                    for (int i = 0; i < E; i++) dst[i] = out[i];
                }
            }
            // all appends of the previous list are done at this barrier; the
            // count is read between it and the next one, before new appends
            __syncthreads();
            const int nb = *s.nbuf;
            const bool flush_now = (nb + len > SP_BCAP) || (*s.nbest < kq && nb >= kq) || nb >= soft;
            __syncthreads();
            if (flush_now) topk_flush(s, nb);
            // ADC scan of the list, software-pipelined one chunk ahead; the
            // filter compares floats first; warps past the end skip the chunk
            // this probe's first chunk, from its stage (the thread's own copies: probes up to j
            // have landed once at most SP_AHEAD groups remain in flight); groups past the staged
            // 1024 (1024-thread blocks) come from global memory
            if constexpr (MIXED) {
                cp_async_wait<SP_AHEAD>();
                const uint4* src = stage + (j % SP_NS) * (US * NT);
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int g = u * NT + tid;
                    cur[u] = g >= ng ? make_uint4(0, 0, 0, 0) : (u < US ? src[g] : load_group(codes + (int64_t)g * 16));
                }
            }
            const uint32_t pos0 = prefix[j];
            const bool fits = len <= SP_BCAP - (flush_now ? 0 : nb);
            u64 tk = *s.thresh;
            float td = tk == KEY_MAX ? __int_as_float(0x7f800000) : key_dist(tk);
            uint32_t tp = key_payload(tk);
            // two chunk buffers used in turn (unrolled by two, so nothing is copied between them)
            auto load_chunk = [&](uint4(&dst)[U], int g0) {
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int g = g0 + u * NT + tid;
                    dst[u] = g < ng ? load_group(codes + (int64_t)g * 16) : make_uint4(0, 0, 0, 0);
                }
            };
            auto scan_chunk = [&](const uint4(&c)[U], int g0) {
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int gw = g0 + u * NT + (tid & ~31);
                    if (gw < ng) {
                        const int i0 = (g0 + u * NT + tid) * G;  // first row of this thread's group
                        float dist[G];
                        bool pass[G], any = false;
#pragma unroll
                        for (int r = 0; r < G; r++) {
                            dist[r] = group_row_dist<M, MIXED>(c[u], r, table, table16);
                            const uint32_t pos = pos0 + (uint32_t)(i0 + r);
                            pass[r] = i0 + r < len && (dist[r] < td || (dist[r] == td && pos < tp));
                            any |= pass[r];
                        }
                        if (__any_sync(0xffffffffu, any)) {
                            u64 key[G];
#pragma unroll
                            for (int r = 0; r < G; r++) key[r] = make_key(dist[r], pos0 + (uint32_t)(i0 + r));
                            topk_push_rows<G>(s, key, pass);
                        }
                    }
                }
                if (!fits) {
                    topk_round_end(s, CH);
                    tk = *s.thresh;
                    td = tk == KEY_MAX ? __int_as_float(0x7f800000) : key_dist(tk);
                    tp = key_payload(tk);
                }
            };
            for (int g0 = 0; g0 < ng; g0 += 2 * NT * U) {
                uint4 nxt[U];
                load_chunk(nxt, g0 + NT * U);
                scan_chunk(cur, g0);
                if (g0 + NT * U >= ng) break;
                load_chunk(cur, g0 + 2 * NT * U);
                scan_chunk(nxt, g0 + NT * U);
            }
        }
        // final merge; hand the unsorted best set (keys and base ids) over
        {
            __syncthreads();
            const int nb = *s.nbuf;
            __syncthreads();
            topk_flush(s, nb);
        }
        const int nbest = *s.nbest;
        if (a.flags & SCAN_KEYS_ONLY) {
            // the best keys, unordered, their count, and the k-th best key (the bound of the rows not
            // scanned here: the list-centric pass keeps only rows below it)
            for (int c = tid; c < nbest; c += NT) a.cand_key[(int64_t)q * a.cand_stride + c] = best[c];
            if (tid == 0) {
                a.cand_cnt[q] = nbest;
                a.tau_out[q] = nbest == kq ? *s.thresh : KEY_MAX;
            }
            continue;
        }
        if (rows_out) {
            // The code row and its list of each candidate, for the exact re-score or the refinement
            // re-rank, grouped by probe (a counting sort on probe & 255): neighbouring threads of the
            // finalize kernel then read the same list centroid and nearby code rows. The finalize
            // orders candidates by (distance, position) keys, so the slot order is free.
            int* cnt = s.hist(0);
            for (int i = tid; i < 256; i += NT) cnt[i] = 0;
            __syncthreads();
            for (int c = tid; c < nbest; c += NT) atomicAdd(&cnt[probe_of(prefix, wq, key_payload(best[c])) & 255], 1);
            __syncthreads();
            if (tid < 32) {  // exclusive prefix over the 256 bins, 8 per lane
                int v[8], sum = 0;
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    v[b] = cnt[8 * lane + b];
                    sum += v[b];
                }
                int incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                int run = incl - sum;
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    cnt[8 * lane + b] = run;
                    run += v[b];
                }
            }
            __syncthreads();
            for (int c = tid; c < nbest; c += NT) {
                const uint32_t pos = key_payload(best[c]);
                const int jj = probe_of(prefix, wq, pos);
                const int ll = plist[jj];
                const int64_t o = (int64_t)q * a.cand_stride + atomicAdd(&cnt[jj & 255], 1);
                a.cand_key[o] = best[c];
                a.cand_id[o] = (int32_t)(ix.list_beg[ll] + (int64_t)(pos - prefix[jj]));
                a.cand_list[o] = ll;
            }
            for (int c = nbest + tid; c < a.cand_stride; c += NT) {
                const int64_t o = (int64_t)q * a.cand_stride + c;
                a.cand_key[o] = KEY_MAX;
                a.cand_id[o] = -1;
                a.cand_list[o] = 0;
            }
        } else {
            for (int c = tid; c < a.cand_stride; c += NT) {
                const int64_t o = (int64_t)q * a.cand_stride + c;
                if (c < nbest) {
                    a.cand_key[o] = best[c];
                    a.cand_id[o] = pos_to_id(ix, prefix, plist, wq, key_payload(best[c]));
                } else {
                    a.cand_key[o] = KEY_MAX;
                    a.cand_id[o] = -1;
                }
            }
        }
        if (tid == 0) a.cand_cnt[q] = nbest;
    }
}

// Per query (one CTA): sort the hand-off set, then write it, or re-rank it by
// exact L2 (ivf_search.cpp:113-134) and write the k best.
// finalize threads per query: 128 (sort, RERANK by raw vectors, the precision form's re-score:
// one candidate per thread), 512 for the refinement re-rank of the exact form (eight lanes per
// candidate)
constexpr int FIN_NT = 128;
// finalize sets of at most this many keys are ordered by rank_sort (one pass over the keys per
// element, two barriers), larger ones by a bitonic network (log^2 barriers, fewer operations)
constexpr int RANK_SORT_MAX = 256;
constexpr int FIN_NT_BIG = 512;
// the precision form's error bound (rs_second_kernel): relative, then absolute per unit of
// ||r||^2 + sum_s max_c ||c_s||^2, then absolute (FP16 subnormals)
constexpr double MIX_DELTA = 0x1p-9;
constexpr double MIX_EPS_REL = 0x1p-12;
constexpr double MIX_EPS_ABS = 0x1p-12;
// the largest second re-score set that the order kernel merges without a second select
constexpr int FIN_XTRA = 256;

__device__ inline void bitonic_sort_pairs(u64* a, int32_t* b, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < (n >> 1); i += nt) {
                const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const u64 x = a[lo], y = a[hi];
                if ((x > y) == asc) {
                    a[lo] = y;
                    a[hi] = x;
                    const int32_t t = b[lo];
                    b[lo] = b[hi];
                    b[hi] = t;
                }
            }
            __syncthreads();
        }
    }
}

// The reference's ADC distance of one code row of list l (d = 128, m = M), recomputed from scratch
// in its arithmetic: per sub-quantizer the residual r_s = x_s - y_{l,s}, its float
// norm, the sequential dot with the code's centroid, the norm sum and -2 dot + c
// (compute_cross_distances, nn.c:113-150), summed in s order (sumidxtab2,
// ivf_search.cpp:189-200). Bit-identical to the scan's exact table entries.
template <int M>
__device__ __forceinline__ float exact_adc(const DevIndex& ix, const float* xq, int l, int64_t row) {
    constexpr int DS = 128 / M, H = M >= 8 ? M / 4 : M;  // sub-quantizers per batch of loads
    using CT = typename CodeRow<M>::T;
    const CT cr = load_row<M>(ix.codes + row * M);
    const uint32_t* cw = reinterpret_cast<const uint32_t*>(&cr);
    const float4* y4 = reinterpret_cast<const float4*>(ix.coa + (int64_t)l * 128);
    float dist = 0.0f;
#pragma unroll
    for (int s0 = 0; s0 < M; s0 += H) {
        // every load of this batch of sub-quantizers first, then the arithmetic
        float4 yv[H * DS / 4], cv[H * DS / 4];
        float hi[H], lo[H];
        int ent[H];
#pragma unroll
        for (int h = 0; h < H; h++) {
            const int s = s0 + h;
            ent[h] = s * 256 + ((cw[s >> 2] >> (8 * (s & 3))) & 0xff);
            const float4* c4 = reinterpret_cast<const float4*>(ix.pq + (int64_t)ent[h] * DS);
#pragma unroll
            for (int v = 0; v < DS / 4; v++) {
                yv[h * (DS / 4) + v] = __ldg(y4 + s * (DS / 4) + v);
                cv[h * (DS / 4) + v] = __ldg(c4 + v);
            }
            hi[h] = __ldg(ix.pq_hi + ent[h]);
            lo[h] = __ldg(ix.pq_lo + ent[h]);
        }
#pragma unroll
        for (int h = 0; h < H; h++) {
            const int s = s0 + h;
            float r[DS], cc[DS];
#pragma unroll
            for (int v = 0; v < DS / 4; v++) {
                const float4 y = yv[h * (DS / 4) + v], c = cv[h * (DS / 4) + v];
                r[4 * v] = __fsub_rn(xq[s * DS + 4 * v], y.x);
                r[4 * v + 1] = __fsub_rn(xq[s * DS + 4 * v + 1], y.y);
                r[4 * v + 2] = __fsub_rn(xq[s * DS + 4 * v + 2], y.z);
                r[4 * v + 3] = __fsub_rn(xq[s * DS + 4 * v + 3], y.w);
                cc[4 * v] = c.x;
                cc[4 * v + 1] = c.y;
                cc[4 * v + 2] = c.z;
                cc[4 * v + 3] = c.w;
            }
            float f = 0.0f, dot = 0.0f;
#pragma unroll
            for (int t = 0; t < DS; t++) f = __fadd_rn(f, __fmul_rn(r[t], r[t]));
#pragma unroll
            for (int t = 0; t < DS; t++) dot = __fadd_rn(dot, __fmul_rn(r[t], cc[t]));
            const float c0 = add_norms_rn(ix.pq_norm + ent[h], hi[h], lo[h], f);
            dist = __fadd_rn(dist, __fadd_rn(__fmul_rn(-2.0f, dot), c0));
        }
    }
    return dist;
}

// Refinement re-rank of candidates 0 .. n-1 (in ADC order; ids[c] is the hand-off slot of
// candidate c): keys[c] = (||x - y_l - c1(codes) - c2(codes2)||^2, c). FP32; eight lanes take one
// candidate, lane b the 16 dimensions 16b .. 16b+15: e_t = ((x_t - y_t) - c1_t) - c2_t, the lane's
// partial sum of e_t^2 in dimension order from 0, then the eight partials summed in b order from 0.
// (The refinement codes have no counterpart in the reference; this order is the definition.)
template <int M>
__device__ __forceinline__ void refine_rerank(const DevIndex& ix, const ScanArgs& a, int64_t hb, const float* xq,
                                              const int32_t* ids, u64* keys, int n) {
    constexpr int DS = 128 / M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int b = lane & 7, grp = lane >> 3, t0 = 16 * b;
    const int m2 = ix.m2, sh2 = __ffs(ix.ds2) - 1;  // ds2 = 128 / m2, a power of two >= 4
    for (int c0 = warp * 4; c0 < n; c0 += (blockDim.x >> 5) * 4) {  // warp-uniform bound
        const int c = c0 + grp;
        float p = 0.0f;
        if (c < n) {
            const int64_t slot = hb + ids[c];
            const int64_t row = a.cand_id[slot];
            const int l = a.cand_list[slot];
            const float4* y4 = reinterpret_cast<const float4*>(ix.coa + (int64_t)l * 128 + t0);
            const uint8_t* c1 = ix.codes + row * M;
            const uint8_t* c2 = ix.codes2 + row * m2;
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const int t = t0 + 4 * v, s = t / DS, s2 = t >> sh2;
                const float4 y = __ldg(y4 + v);
                const float4 av = __ldg(reinterpret_cast<const float4*>(ix.pq + ((int64_t)s * 256 + c1[s]) * DS + (t - s * DS)));
                const float4 bv = __ldg(reinterpret_cast<const float4*>(
                    ix.pq2 + (((int64_t)s2 * 256 + c2[s2]) << sh2) + (t - (s2 << sh2))));
                const float e0 = __fsub_rn(__fsub_rn(__fsub_rn(xq[t], y.x), av.x), bv.x);
                const float e1 = __fsub_rn(__fsub_rn(__fsub_rn(xq[t + 1], y.y), av.y), bv.y);
                const float e2 = __fsub_rn(__fsub_rn(__fsub_rn(xq[t + 2], y.z), av.z), bv.z);
                const float e3 = __fsub_rn(__fsub_rn(__fsub_rn(xq[t + 3], y.w), av.w), bv.w);
                p = __fadd_rn(p, __fmul_rn(e0, e0));
                p = __fadd_rn(p, __fmul_rn(e1, e1));
                p = __fadd_rn(p, __fmul_rn(e2, e2));
                p = __fadd_rn(p, __fmul_rn(e3, e3));
            }
        }
        float dist = 0.0f;
#pragma unroll
        for (int t = 0; t < 8; t++) dist = __fadd_rn(dist, __shfl_sync(0xffffffffu, p, grp * 8 + t));
        if (c < n && b == 0) keys[c] = make_key(dist, (uint32_t)c);
    }
}

// Per query (one CTA): order the hand-off set, then write it, or re-rank it and write the k best.
// The sort carries the keys and, with them, either base ids (the exact form) or hand-off slots
// (precision form, refinement re-rank: the slot leads to the candidate's code row and list).
// The results of one query from its ordered set: keys[0 .. n) ascending with ids[0 .. n) (base ids,
// or hand-off slots when `slots`), written out, or re-ranked first (RERANK by the raw vectors,
// REFINE by the refinement codes). keys[] holds room for the next power of two >= n; xq is the
// query (shared memory) when re-ranking. All NT threads of the block call it.
template <int M, int NT>
__device__ void fin_output(const DevIndex& ix, const ScanArgs& a, int q, int64_t hb, u64* keys, int32_t* ids, int n,
                           const float* xq, bool slots) {
    constexpr int FIN_NT = NT;
    const int tid = threadIdx.x;
    const bool rerank = a.flags & SCAN_RERANK, refine = a.flags & SCAN_REFINE;
    auto base_id = [&](int c) { return slots ? ix.ids[a.cand_id[hb + ids[c]]] : ids[c]; };
    const float inf = __int_as_float(0x7f800000);
    if (!rerank && !refine) {
        if (a.flags & SCAN_OUT_PACKED) {
            const int64_t o = a.out_start[q];
            for (int c = tid; c < n; c += FIN_NT) {
                a.out_ids[o + c] = base_id(c);
                a.out_dis[o + c] = key_dist(keys[c]);
            }
        } else {
            const int kq = query_k(a, q);
            const int64_t o = query_out(a, q);
            for (int c = tid; c < kq; c += FIN_NT) {
                a.out_ids[o + c] = c < n ? base_id(c) : -1;
                a.out_dis[o + c] = c < n ? key_dist(keys[c]) : inf;
            }
        }
        return;
    }
    // re-rank the n candidates in ADC order: exact L2 to the raw vector (ivf_search.cpp:113-134)
    // or the refined distance, keyed by the ADC rank
    const double qn = a.qnorm[q];
    const int d = ix.d;
    int pr = 2;
    while (pr < n) pr <<= 1;
    if (refine) {
        // keys[c] for c < n: every lane reads ids[] and keys[] of its own candidate only
        refine_rerank<M>(ix, a, hb, xq, ids, keys, n);
        for (int c = n + tid; c < pr; c += FIN_NT) keys[c] = KEY_MAX;
    } else
    for (int c = tid; c < pr; c += FIN_NT) {
        u64 key = KEY_MAX;
        if (c < n) {
            float dist;
            {
                const int32_t id = base_id(c);
                const float4* v4 = reinterpret_cast<const float4*>(ix.base + (int64_t)id * d);
                float dot = 0.0f;
                for (int l = 0; l < d / 4; l++) {
                    const float4 b = __ldg(v4 + l);
                    dot = __fadd_rn(dot, __fmul_rn(b.x, xq[4 * l]));
                    dot = __fadd_rn(dot, __fmul_rn(b.y, xq[4 * l + 1]));
                    dot = __fadd_rn(dot, __fmul_rn(b.z, xq[4 * l + 2]));
                    dot = __fadd_rn(dot, __fmul_rn(b.w, xq[4 * l + 3]));
                }
                dist = expansion_from(qn, ix.base_norm[id], dot);
            }
            key = make_key(dist, (uint32_t)c);
        }
        keys[c] = key;  // (ids[] keeps the ADC order the payload refers to)
    }
    __syncthreads();
    if (n <= RANK_SORT_MAX) rank_sort(keys, nullptr, n);
    else bitonic_sort_smem(keys, pr);
    const int kq = query_k(a, q);
    const int64_t o = query_out(a, q);
    const int kr = min(kq, n);
    for (int c = tid; c < kq; c += FIN_NT) {
        a.out_ids[o + c] = c < kr ? base_id(key_payload(keys[c])) : -1;
        a.out_dis[o + c] = c < kr ? key_dist(keys[c]) : inf;
    }
}

// Per query (one CTA): sort the hand-off set, then write it, or re-rank it by
// exact L2 (ivf_search.cpp:113-134) and write the k best. (The precision form's hand-off goes
// through the re-score kernels below instead.)
template <int M, int NT>
__global__ void __launch_bounds__(NT) finalize_kernel(DevIndex ix, ScanArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    constexpr int FIN_NT = NT;
    const int n2 = a.cand_stride;  // power of two
    u64* keys = reinterpret_cast<u64*>(fsm);
    int32_t* ids = reinterpret_cast<int32_t*>(keys + n2);
    float* xq = reinterpret_cast<float*>(ids + n2);
    const int q = blockIdx.x, tid = threadIdx.x;
    const bool rerank = a.flags & SCAN_RERANK, refine = a.flags & SCAN_REFINE;
    const bool slots = refine;  // ids[] holds hand-off slots, not base ids
    const int64_t hb = (int64_t)q * n2;  // this query's hand-off slots
    const int n = a.cand_cnt[q];
    // only this query's candidates are sorted: the smallest power of two holding them (the
    // hand-off pads with KEY_MAX), not the batch-wide stride
    int p2 = 2;
    while (p2 < n) p2 <<= 1;
    for (int c = tid; c < p2; c += FIN_NT) {
        keys[c] = c < n ? a.cand_key[hb + c] : KEY_MAX;
        ids[c] = slots ? c : a.cand_id[hb + c];
    }
    if (rerank || slots)
        for (int x = tid; x < ix.d; x += FIN_NT) xq[x] = a.queries[(int64_t)q * ix.d + x];
    __syncthreads();
    if (n <= RANK_SORT_MAX) rank_sort(keys, ids, n);
    else bitonic_sort_pairs(keys, ids, p2);
    fin_output<M, NT>(ix, a, q, hb, keys, ids, n, xq, slots);
}

bool scan_persistent_supported(const DevIndex& ix, const ScanArgs& a) {
    const int kk = (a.flags & (SCAN_RERANK | SCAN_REFINE)) ? a.kl : a.k;
    const bool m_ok = ix.m == 4 || ix.m == 8 || ix.m == 16;
    const bool mixed_ok = !(a.flags & SCAN_MIXED) ||
                          !(a.flags & (SCAN_TABLE_DIRECT | SCAN_SRC_RESIDUAL | SCAN_OUT_PACKED));
    const bool refine_ok = !(a.flags & SCAN_REFINE) ||
                           !(a.flags & (SCAN_RERANK | SCAN_SRC_RESIDUAL | SCAN_OUT_PACKED));
    return ix.d == 128 && ix.ks == 256 && m_ok && std::max(kk, a.k) <= 1024 && a.queue != nullptr &&
           ix.pq_hi != nullptr && !((a.flags & SCAN_SRC_RESIDUAL) && (a.flags & SCAN_RERANK)) && mixed_ok &&
           refine_ok;
}

int scan_persistent_stride(const ScanArgs& a) {
    const int kk = (a.flags & (SCAN_RERANK | SCAN_REFINE)) ? a.kl : a.k;
    const int sel = (a.flags & SCAN_MIXED) ? mixed_sel(a, kk) : kk;
    return pow2_at_least(std::max(std::max(sel, a.k), 2));
}

// ---------------------------------------------------------------------------
// The precision form's exact re-score.
//
// Every approximate distance A bounds the exact one E (the reference's FP32 arithmetic) from
// below: E >= A (1 - MIX_DELTA) - eps_q. MIX_DELTA covers the FP16 rounding of the table entries
// (2^-11 relative, a saturated entry only lowers A) and the FP32 accumulation; eps_q the FP32
// rounding of both forms' expansions (at most ~2^-16 (||r||^2 + sum_s max ||c_s||^2)), with
// margins of 4 and 16. So, with T0 the largest exact distance of the kk best approximate
// candidates, no candidate with A >= tau = (T0 + eps_q) / (1 - MIX_DELTA) can enter the exact
// top-kk: the kk best and those below tau are re-scored, no other. Five launches:
//   rs_first_kernel   per query: the kk-th approximate key (radix select), the kk best listed
//                     (the first set), the residual bound r2;
//   rs_rescore_kernel flat: one lane per listed candidate, 32-candidate chunks from a queue; the
//                     exact key replaces the approximate one in the hand-off; T0 by atomicMax;
//   rs_second_kernel  per query: tau, the other candidates below it listed (the second set), the proof;
//   rs_rescore_kernel on the second set;
//   rs_order_kernel   per query: the two sets sorted (registers / by rank) and merged, then the
//                     results written (or re-ranked) by fin_output.
// Only the re-score kernel holds the exact arithmetic's registers; the per-query kernels run at
// the occupancy their shared memory allows.
// ---------------------------------------------------------------------------

constexpr int RS_NT = 128;        // per-query kernels
// the order kernel's threads and keys per thread of its register sort (1,024 keys): 256 x 4, or
// 512 x 2 with the refinement re-rank, whose gathers want more loads in flight
constexpr int RS_ORDER_KEYS = 1024;
constexpr int RS_CHUNK = 32;      // candidates per queue entry (one warp)

// queue the chunks [i0, i1) of query q's list in the queue of set `set` (0: first, 1: second)
__device__ __forceinline__ void rs_enqueue(const ScanArgs& a, int set, int q, int i0, int i1) {
    const int nch = (i1 - i0 + RS_CHUNK - 1) / RS_CHUNK;
    __shared__ int s_base;
    if (threadIdx.x == 0) s_base = nch > 0 ? atomicAdd(a.rw.qcount + set, nch) : 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nch; j += blockDim.x) {
        const int slot = s_base + j;
        if (slot < a.rw.qcap) a.rw.queue[(int64_t)set * a.rw.qcap + slot] = make_int4(q, i0 + j * RS_CHUNK, i1, 0);
    }
}

// warp-uniform gather of the candidates c < n passing pred(c) into list[*cnt ..); returns the
// warp's ballot word for the 32 candidates from c0
template <class Pred>
__device__ __forceinline__ unsigned rs_gather_word(int c0, int n, int32_t* list, int* cnt, Pred pred) {
    const int lane = threadIdx.x & 31, c = c0 + lane;
    const bool in = c < n && pred(c);
    const unsigned mk = __ballot_sync(0xffffffffu, in);
    int base = 0;
    if (lane == 0 && mk) base = atomicAdd(cnt, __popc(mk));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (in) list[base + __popc(mk & ((1u << lane) - 1u))] = c;
    return mk;
}

template <int M>
__global__ void __launch_bounds__(RS_NT) rs_first_kernel(DevIndex ix, ScanArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    u64* keys = reinterpret_cast<u64*>(fsm);   // [cand_stride] the approximate keys
    float* xq = reinterpret_cast<float*>(keys + a.cand_stride);
    __shared__ u64 s_amax;
    __shared__ unsigned s_r2;
    __shared__ int s_cnt;
    const int q = blockIdx.x, tid = threadIdx.x, stride = a.cand_stride;
    const int64_t hb = (int64_t)q * stride;
    const int n = a.cand_cnt[q];
    const bool rr = a.flags & (SCAN_RERANK | SCAN_REFINE);
    const int kk = min(n, rr ? a.kl : query_k(a, q));
    if (tid == 0) {
        s_amax = 0;
        s_r2 = 0u;
        s_cnt = 0;
    }
    u64 amax = 0;
    for (int c = tid; c < n; c += RS_NT) {
        keys[c] = a.cand_key[hb + c];
        amax = keys[c] > amax ? keys[c] : amax;
    }
    for (int x = tid; x < 128; x += RS_NT) xq[x] = a.queries[(int64_t)q * 128 + x];
    __syncthreads();
    atomicMax(&s_amax, amax);
    const u64 th = n > kk ? block_kth_flagged(keys, n, nullptr, kk) : KEY_MAX;
    int32_t* list = a.rw.list + hb;
    unsigned* marks = a.rw.marks + (int64_t)q * (stride / 32);
    for (int c0 = tid & ~31; c0 < n; c0 += RS_NT) {
        const unsigned mk = rs_gather_word(c0, n, list, &s_cnt, [&](int c) { return keys[c] <= th; });
        if ((tid & 31) == 0) marks[c0 >> 5] = mk;
    }
    // the largest squared residual norm over the query's probes (a bound on ||r||^2 for every
    // candidate, handed off or not): four threads per probe, 32 dimensions each
    float r2 = 0.0f;
    const int wq = query_w(a, q);
    for (int j0 = 0; j0 < wq; j0 += RS_NT / 4) {  // block-uniform trip count (shuffles below)
        const int j = j0 + tid / 4, part = tid & 3;
        float sq = 0.0f;
        const int l = j < wq ? a.probes[(int64_t)q * a.w + j] : -1;
        if (l >= 0 && l < ix.C) {
            const float4* y4 = reinterpret_cast<const float4*>(ix.coa + (int64_t)l * 128 + 32 * part);
            const float* xp = xq + 32 * part;
            float4 y[8];
#pragma unroll
            for (int v = 0; v < 8; v++) y[v] = __ldg(y4 + v);
#pragma unroll
            for (int v = 0; v < 8; v++) {
                const float d0 = xp[4 * v] - y[v].x, d1 = xp[4 * v + 1] - y[v].y, d2 = xp[4 * v + 2] - y[v].z,
                            d3 = xp[4 * v + 3] - y[v].w;
                sq = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, fmaf(d3, d3, sq))));
            }
        }
        sq += __shfl_xor_sync(0xffffffffu, sq, 1);
        sq += __shfl_xor_sync(0xffffffffu, sq, 2);
        r2 = fmaxf(r2, sq);
    }
    atomicMax(&s_r2, __float_as_uint(r2));  // (non-negative floats order as their bits)
    __syncthreads();
    const int m0 = s_cnt;
    if (tid == 0) {
        a.rw.cnt[2 * q] = m0;
        a.rw.cnt[2 * q + 1] = m0;
        a.rw.t0[q] = 0;
        a.rw.amax[q] = s_amax;
        a.rw.r2[q] = __uint_as_float(s_r2);
    }
    rs_enqueue(a, 0, q, 0, m0);
}

// one lane per listed candidate: its exact ADC distance (exact_adc: the reference's arithmetic, the
// exact form's table entries bit for bit) keyed (distance, position) in place of its approximate key
template <int M>
__global__ void __launch_bounds__(RS_NT, M == 4 ? 2 : 6) rs_rescore_kernel(DevIndex ix, ScanArgs a, int set) {
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (RS_NT / 32);
    const int nch = min(a.rw.qcount[set], a.rw.qcap);
    const int4* queue = a.rw.queue + (int64_t)set * a.rw.qcap;
    for (int ch = blockIdx.x * (RS_NT / 32) + (threadIdx.x >> 5); ch < nch; ch += nwarps) {
        const int4 e = queue[ch];  // (query, first, end, 0)
        const int q = e.x, i = e.y + lane;
        const int64_t hb = (int64_t)q * a.cand_stride;
        u64 key = 0;
        if (i < e.z) {
            const int c = a.rw.list[hb + i];
            key = make_key(exact_adc<M>(ix, a.queries + (int64_t)q * 128, a.cand_list[hb + c], a.cand_id[hb + c]),
                           key_payload(a.cand_key[hb + c]));
            a.cand_key[hb + c] = key;
        }
        if (set == 0) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const u64 x = __shfl_xor_sync(0xffffffffu, key, o);
                key = x > key ? x : key;
            }
            if (lane == 0) atomicMax(a.rw.t0 + q, key);
        }
    }
}

template <int M>
__global__ void __launch_bounds__(RS_NT) rs_second_kernel(DevIndex ix, ScanArgs a) {
    __shared__ int s_cnt;
    const int q = blockIdx.x, tid = threadIdx.x, stride = a.cand_stride;
    const int64_t hb = (int64_t)q * stride;
    const int n = a.cand_cnt[q];
    const bool rr = a.flags & (SCAN_RERANK | SCAN_REFINE);
    const int ksel = mixed_sel(a, rr ? a.kl : query_k(a, q));
    const int m0 = a.rw.cnt[2 * q];
    const double T0 = fmax(0.0, (double)key_dist(a.rw.t0[q]));
    const double eps = MIX_EPS_REL * ((double)a.rw.r2[q] * (1.0 + 0x1p-10) + (double)ix.pq_cmax) + MIX_EPS_ABS;
    const double tau = (T0 + eps) / (1.0 - MIX_DELTA) * (1.0 + 0x1p-20);
    if (tid == 0) s_cnt = m0;
    __syncthreads();
    int32_t* list = a.rw.list + hb;
    const unsigned* marks = a.rw.marks + (int64_t)q * (stride / 32);
    for (int c0 = tid & ~31; c0 < n; c0 += RS_NT) {
        const unsigned mw = marks[c0 >> 5];
        rs_gather_word(c0, n, list, &s_cnt, [&](int c) {
            return !((mw >> (c & 31)) & 1u) && (double)key_dist(a.cand_key[hb + c]) < tau;
        });
    }
    __syncthreads();
    const int m = s_cnt;
    if (tid == 0) {
        a.rw.cnt[2 * q + 1] = m;
        // not proven: the hand-off is full (candidates may lie beyond it) and all of it is below tau
        if (a.unproven && n >= ksel && (double)key_dist(a.rw.amax[q]) < tau) atomicAdd(a.unproven, 1);
    }
    rs_enqueue(a, 1, q, m0, m);
}

// The kk best exact keys of the re-scored set, in order: the first set (min(n, kk) keys)
// sorted in registers, the second (usually a few) by rank, the two merged -- each key's place is
// its rank in its own set plus the number of smaller keys in the other; a large second set goes
// through a radix select of the kk-th key and one sort instead. Then the results.
template <int M, int RS_ORDER_NT, int RS_ORDER_PER>
__global__ void __launch_bounds__(RS_ORDER_NT) rs_order_kernel(DevIndex ix, ScanArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    constexpr int META = RS_ORDER_NT * RS_ORDER_PER;
    const int stride = a.cand_stride;
    u64* keys = reinterpret_cast<u64*>(fsm);                       // [stride] ordered keys, then scratch
    int32_t* ids = reinterpret_cast<int32_t*>(keys + stride);      // [stride] their hand-off slots
    float* xq = reinterpret_cast<float*>(ids + stride);            // [128] the query
    u64* sk = reinterpret_cast<u64*>(xq + 128);                    // staging: META + FIN_XTRA keys ...
    int32_t* ss = reinterpret_cast<int32_t*>(sk + META + FIN_XTRA);  // ... and slots
    u64* xk = sk + META;
    int32_t* xs = ss + META;
    __shared__ int s_cnt2;
    const int q = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    const int64_t hb = (int64_t)q * stride;
    const bool rr = a.flags & (SCAN_RERANK | SCAN_REFINE);
    const int kk0 = rr ? a.kl : query_k(a, q);
    const int m0 = a.rw.cnt[2 * q], m = a.rw.cnt[2 * q + 1], m1 = m - m0;
    const int32_t* list = a.rw.list + hb;
    if (rr)
        for (int x = tid; x < 128; x += RS_ORDER_NT) xq[x] = a.queries[(int64_t)q * 128 + x];
    if (tid == 0) s_cnt2 = 0;
    int nout;
    if (m1 <= FIN_XTRA) {
        for (int i = tid; i < m0; i += RS_ORDER_NT) {
            const int c = list[i];
            sk[i] = a.cand_key[hb + c];
            ss[i] = c;
        }
        for (int i = tid; i < m1; i += RS_ORDER_NT) {
            const int c = list[m0 + i];
            xk[i] = a.cand_key[hb + c];
            xs[i] = c;
        }
        __syncthreads();
        if (m0 <= RANK_SORT_MAX) rank_sort(sk, ss, m0);
        else block_sort_regs<RS_ORDER_NT, RS_ORDER_PER>(sk, ss, m0);
        if (m1 > 1) rank_sort(xk, xs, m1);
        __syncthreads();
        nout = min(m, kk0);
        for (int i = tid; i < m0; i += RS_ORDER_NT) {
            const u64 key = sk[i];
            int lo = 0, hi = m1;  // smaller keys of the second set
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (xk[mid] < key) lo = mid + 1;
                else hi = mid;
            }
            if (i + lo < nout) {
                keys[i + lo] = key;
                ids[i + lo] = ss[i];
            }
        }
        for (int i = tid; i < m1; i += RS_ORDER_NT) {
            const u64 key = xk[i];
            int lo = 0, hi = m0;  // smaller keys of the first set
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (sk[mid] < key) lo = mid + 1;
                else hi = mid;
            }
            if (i + lo < nout) {
                keys[i + lo] = key;
                ids[i + lo] = xs[i];
            }
        }
    } else {
        // all m exact keys (m <= n <= stride) in keys[] / ids[], the kk0-th by a radix select
        for (int i = tid; i < m; i += RS_ORDER_NT) {
            const int c = list[i];
            keys[i] = a.cand_key[hb + c];
            ids[i] = c;
        }
        __syncthreads();
        const u64 th2 = m > kk0 ? block_kth_flagged(keys, m, nullptr, kk0) : KEY_MAX;
        for (int c0 = tid & ~31; c0 < m; c0 += RS_ORDER_NT) {
            const int c = c0 + lane;
            const bool in = c < m && keys[c] <= th2;
            const unsigned mk = __ballot_sync(0xffffffffu, in);
            int base = 0;
            if (lane == 0 && mk) base = atomicAdd(&s_cnt2, __popc(mk));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (in) {
                const int o = base + __popc(mk & ((1u << lane) - 1u));
                sk[o] = keys[c];
                ss[o] = ids[c];
            }
        }
        __syncthreads();
        nout = s_cnt2;  // min(m, kk0): the keys are unique
        if (nout <= RANK_SORT_MAX) rank_sort(sk, ss, nout);
        else block_sort_regs<RS_ORDER_NT, RS_ORDER_PER>(sk, ss, nout);
        for (int c = tid; c < nout; c += RS_ORDER_NT) {
            keys[c] = sk[c];
            ids[c] = ss[c];
        }
    }
    __syncthreads();
    fin_output<M, RS_ORDER_NT>(ix, a, q, hb, keys, ids, nout, xq, true);
}

template <int M>
static cudaError_t launch_rescore(const DevIndex& ix, const ScanArgs& a, cudaStream_t st) {
    const RescoreWork& w = a.rw;
    if (!w.list || !w.cnt || !w.marks || !w.t0 || !w.amax || !w.r2 || !w.queue || !w.qcount || w.qcap <= 0 ||
        ix.d != 128 || a.cand_stride > 4096 || a.cand_stride < 32)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(w.qcount, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const size_t sm1 = (size_t)a.cand_stride * 8 + 512;
    if (sm1 > 48 * 1024 &&
        (e = cudaFuncSetAttribute(rs_first_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1)) != cudaSuccess)
        return e;
    rs_first_kernel<M><<<a.nq, RS_NT, sm1, st>>>(ix, a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    // persistent, as many CTAs as fit: the queues' lengths are known on the device only
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rs_rescore_kernel<M>, RS_NT, 0)) != cudaSuccess)
        return e;
    const int rgrid = sms * std::max(per_sm, 1);
    rs_rescore_kernel<M><<<rgrid, RS_NT, 0, st>>>(ix, a, 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    rs_second_kernel<M><<<a.nq, RS_NT, 0, st>>>(ix, a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    rs_rescore_kernel<M><<<rgrid, RS_NT, 0, st>>>(ix, a, 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const size_t sm4 = (size_t)a.cand_stride * 12 + 512 + (size_t)(RS_ORDER_KEYS + FIN_XTRA) * 12;
    const bool refine = a.flags & SCAN_REFINE;
    void (*ord)(DevIndex, ScanArgs) = refine ? rs_order_kernel<M, 512, RS_ORDER_KEYS / 512>
                                             : rs_order_kernel<M, 256, RS_ORDER_KEYS / 256>;
    if (sm4 > 48 * 1024 &&
        (e = cudaFuncSetAttribute(ord, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4)) != cudaSuccess)
        return e;
    ord<<<a.nq, refine ? 512 : 256, sm4, st>>>(ix, a);
    return cudaGetLastError();
}

// the re-score workspace's queue capacity for a batch (chunks of either set, per set)
int rescore_queue_cap(int nq, int stride) { return nq * (stride / RS_CHUNK + 1); }

template <int M, bool MIXED>
static cudaError_t launch_fin(const DevIndex& ix, const ScanArgs& a, cudaStream_t st) {
    if constexpr (MIXED) {
        return launch_rescore<M>(ix, a, st);
    } else {
        const size_t fsm = (size_t)a.cand_stride * 12 + 512;  // keys, ids, the query
        const bool big = a.flags & SCAN_REFINE;
        void (*fin)(DevIndex, ScanArgs) = big ? finalize_kernel<M, FIN_NT_BIG> : finalize_kernel<M, FIN_NT>;
        if (fsm > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm);
            if (e != cudaSuccess) return e;
        }
        fin<<<a.nq, big ? FIN_NT_BIG : FIN_NT, fsm, st>>>(ix, a);
        return cudaGetLastError();
    }
}

cudaError_t launch_finalize(const DevIndex& ix, const ScanArgs& a, cudaStream_t st) {
    if (a.nq <= 0) return cudaSuccess;
    const bool mixed = a.flags & SCAN_MIXED;
    switch (ix.m) {
        case 4: return mixed ? launch_fin<4, true>(ix, a, st) : launch_fin<4, false>(ix, a, st);
        case 8: return mixed ? launch_fin<8, true>(ix, a, st) : launch_fin<8, false>(ix, a, st);
        case 16: return mixed ? launch_fin<16, true>(ix, a, st) : launch_fin<16, false>(ix, a, st);
        default: return cudaErrorNotSupported;
    }
}

template <int M, bool DIRECT, int NT, bool MIXED = false>
static cudaError_t launch_sp(const DevIndex& ix, const ScanArgs& a, int num_sms, cudaStream_t st, cudaEvent_t mid,
                             bool finalize) {
    const int kcap = scan_persistent_stride(a);
    const bool keys_only = a.flags & SCAN_KEYS_ONLY;
    if (a.cand_stride != kcap || !a.cand_key || (!a.cand_id && !keys_only) || !a.cand_cnt) return cudaErrorInvalidValue;
    if (MIXED && ((!a.cand_list && !keys_only) || a.sel_mult < 1 || a.sel_cap < 1)) return cudaErrorInvalidValue;
    if ((a.flags & SCAN_REFINE) && ((!a.cand_list && !keys_only) || !ix.codes2 || !ix.pq2)) return cudaErrorInvalidValue;
    if (a.qlist && !a.nqlist) return cudaErrorInvalidValue;
    ScanSmem L = scan_smem_layout(M, 256, 128, a.w, kcap, SP_BCAP, 2, SP_RCH, MIXED ? 2 : 4,
                                  MIXED ? (size_t)SP_NS * std::min((M == 4 ? 1 : 2) * NT, 1024) * 16 : 0);
    auto kern = ivf_scan_persistent_kernel<M, DIRECT, NT, MIXED>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, L.total);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = a.qlist ? num_sms * per_sm : std::min(a.nq, num_sms * per_sm);
    e = cudaMemsetAsync(a.queue, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, NT, L.total, st>>>(ix, a, L, kcap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (!finalize) return cudaSuccess;
    if (mid && (e = cudaEventRecord(mid, st)) != cudaSuccess) return e;
    return launch_fin<M, MIXED>(ix, a, st);
}

template <int NT>
static cudaError_t launch_sp_nt(const DevIndex& ix, const ScanArgs& a, int num_sms, cudaStream_t st, cudaEvent_t mid,
                                bool fin) {
    const bool direct = a.flags & SCAN_TABLE_DIRECT;
    if (a.flags & SCAN_MIXED) {  // the precision form: expansion tables only
        if (direct) return cudaErrorNotSupported;
        switch (ix.m) {
            case 4: return launch_sp<4, false, NT, true>(ix, a, num_sms, st, mid, fin);
            case 8: return launch_sp<8, false, NT, true>(ix, a, num_sms, st, mid, fin);
            default: return launch_sp<16, false, NT, true>(ix, a, num_sms, st, mid, fin);
        }
    }
    switch (ix.m) {
        case 4:
            return direct ? launch_sp<4, true, NT>(ix, a, num_sms, st, mid, fin) : launch_sp<4, false, NT>(ix, a, num_sms, st, mid, fin);
        case 8:
            return direct ? launch_sp<8, true, NT>(ix, a, num_sms, st, mid, fin) : launch_sp<8, false, NT>(ix, a, num_sms, st, mid, fin);
        default:
            return direct ? launch_sp<16, true, NT>(ix, a, num_sms, st, mid, fin)
                          : launch_sp<16, false, NT>(ix, a, num_sms, st, mid, fin);
    }
}

cudaError_t launch_scan_persistent(const DevIndex& ix, const ScanArgs& a, int num_sms, int threads, cudaStream_t st,
                                   cudaEvent_t mid, bool finalize) {
    if (a.nq <= 0) return cudaSuccess;
    if (!scan_persistent_supported(ix, a)) return cudaErrorNotSupported;
    if ((a.flags & SCAN_KEYS_ONLY) && (!a.tau_out || finalize)) return cudaErrorInvalidValue;
    return threads == 1024 ? launch_sp_nt<1024>(ix, a, num_sms, st, mid, finalize)
                           : launch_sp_nt<512>(ix, a, num_sms, st, mid, finalize);
}

}  // namespace gbivf
