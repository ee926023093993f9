// Kernel launch interface of the GB300 IVF-PQ engine (internal; the public
// surface is the C ABI in include/gbivf.h).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbivf {

enum ScanFlags : int {
    SCAN_RERANK = 1,        // exact L2 re-rank of the kl ADC candidates
    SCAN_TABLE_DIRECT = 2,  // tables as sum (r-c)^2 (parallel2 core)
    SCAN_SRC_RESIDUAL = 4,  // residuals are given (nq*w x d) instead of queries
    SCAN_OUT_PACKED = 8,    // write min(L, k) results at out_start[q] (core_gpu)
    SCAN_MIXED = 16,        // precision form: FP16 approximate tables, exact re-score of alpha*k
    SCAN_REFINE = 32,       // re-rank the kl ADC candidates by their refined reconstruction
    SCAN_KEYS_ONLY = 64,    // persistent scan: hand off the best keys, their count and the k-th key only
};

// Device view of one index (all pointers in device memory).
struct DevIndex {
    int d = 0, C = 0, m = 0, ks = 0, ds = 0;
    int64_t rows = 0;             // code rows incl. alignment padding
    const float* coa = nullptr;        // C x d
    const float* coa_norm = nullptr;   // C   float norms (a-operand of the coarse product)
    const float* pq = nullptr;         // m x ks x ds
    const double* pq_norm = nullptr;   // m x ks double norms (b-operand of the table product)
    const float* pq_hi = nullptr;      // m x ks  RN32(pq_norm)
    const float* pq_lo = nullptr;      // m x ks  RN32(pq_norm - pq_hi)
    float pq_cmax = 0.0f;              // sum over sub-quantizers of the largest centroid norm (rounded up)
    const int64_t* list_beg = nullptr; // C   first row of each list
    const int32_t* list_len = nullptr; // C
    const uint8_t* codes = nullptr;    // rows x m
    const int32_t* ids = nullptr;      // rows (-1 in padding)
    const float* base = nullptr;       // nbase x d raw vectors (re-rank)
    const float* base_norm = nullptr;  // nbase float norms
    int64_t nbase = 0;
    // refinement codes of the residual error (x - y_l - c1(codes)): m2 x 256 x ds2 codebook,
    // rows x m2 codes in the row layout of `codes`
    int m2 = 0, ds2 = 0;
    const float* pq2 = nullptr;
    const uint8_t* codes2 = nullptr;
};

// The precision form's exact re-score (scan_persistent.cu, launch_finalize): per-query selects and
// gathers around a flat re-score kernel that works through queues of 32-candidate chunks.
struct RescoreWork {
    int32_t* list = nullptr;            // nq x cand_stride: hand-off slots to re-score, first set then second
    int* cnt = nullptr;                 // nq x 2: list length after the first set, after the second
    unsigned* marks = nullptr;          // nq x cand_stride / 32: slots of the first set
    unsigned long long* t0 = nullptr;   // nq: largest exact key of the first set
    unsigned long long* amax = nullptr; // nq: largest approximate key of the hand-off
    float* r2 = nullptr;                // nq: largest squared residual norm over the query's probes
    int4* queue = nullptr;              // 2 x qcap chunks (query, first, end, 0), one queue per set
    int* qcount = nullptr;              // [0], [1]: chunks queued per set
    int qcap = 0;
};

struct ScanArgs {
    int nq = 0, w = 0, k = 0, kl = 0, flags = 0;
    const float* queries = nullptr;    // nq x d
    const double* qnorm = nullptr;     // nq
    const int32_t* probes = nullptr;   // nq x w list ids (coaidx / rid_to_ivf)
    const float* residual = nullptr;   // (nq*w) x d when SCAN_SRC_RESIDUAL
    const int32_t* out_start = nullptr;// nq when SCAN_OUT_PACKED
    int32_t* out_ids = nullptr;
    float* out_dis = nullptr;
    int* queue = nullptr;              // work counter of the persistent kernel (zeroed per launch)
    // -0.0f, passed at run time: the exact tables form each product as fma(r, c, -0), which rounds
    // once like the reference's multiply; a -0 the compiler cannot see keeps it from treating the
    // FMA as a multiply and fusing it into the following add
    float neg_zero = -0.0f;
    // hand-off from the persistent scan to its finalize kernel: per query the
    // unsorted best keys and their base ids (cand_stride slots) and a count
    unsigned long long* cand_key = nullptr;
    int32_t* cand_id = nullptr;
    int32_t* cand_cnt = nullptr;
    int cand_stride = 0;
    // uneven batches: per-query probe count (<= w, the probes row stride) and
    // result count (<= k), results of query q at out_off[q]; NULL = uniform
    const int32_t* w_per_q = nullptr;
    const int32_t* k_per_q = nullptr;
    const int64_t* out_off = nullptr;
    // precision form (SCAN_MIXED): the approximate selection size min(sel_mult * k, sel_cap), and
    // the hand-off's list of each candidate (cand_id then holds its code row)
    int sel_mult = 1, sel_cap = 0;
    int sel_extra = 0;  // ... and at least k + sel_extra (mixed_sel)
    int32_t* cand_list = nullptr;
    // persistent scan over a subset of the batch: queries qlist[0 .. *nqlist) (NULL: 0 .. nq-1)
    const int32_t* qlist = nullptr;
    const int* nqlist = nullptr;
    // SCAN_KEYS_ONLY: per query the k-th best key when k were found, else KEY_MAX
    unsigned long long* tau_out = nullptr;
    // precision form: incremented by finalize for each query whose result it could not prove equal
    // to the exact form's (NULL: not counted)
    int* unproven = nullptr;
    // precision form: the re-score's workspace (required with SCAN_MIXED)
    RescoreWork rw;
};

// the precision form's approximate selection for a query returning kk results:
// min(max(sel_mult * kk, kk + sel_extra), sel_cap)
__host__ __device__ __forceinline__ int mixed_sel(const ScanArgs& a, int kk) {
    const int s = a.sel_mult * kk > kk + a.sel_extra ? a.sel_mult * kk : kk + a.sel_extra;
    return s < a.sel_cap ? s : a.sel_cap;
}

// per-query shape of a (possibly uneven) batch
// (values outside 1..w / 1..k are clamped, so a bad entry cannot overrun buffers)
__device__ __forceinline__ int query_w(const ScanArgs& a, int q) {
    return a.w_per_q ? min(max(a.w_per_q[q], 1), a.w) : a.w;
}
__device__ __forceinline__ int query_k(const ScanArgs& a, int q) {
    return a.k_per_q ? min(max(a.k_per_q[q], 1), a.k) : a.k;
}
__device__ __forceinline__ int64_t query_out(const ScanArgs& a, int q) {
    return a.out_off ? a.out_off[q] : (int64_t)q * a.k;
}

// query norms: double accumulation of float squares (nn.c:137-142)
cudaError_t launch_norm_d(const float* x, int64_t n, int d, double* out, cudaStream_t st);
// row norms: float, sequential (nn.c:129-135)
cudaError_t launch_norm_f(const float* x, int64_t n, int d, float* out, cudaStream_t st);
// coarse distances of nq queries to all C centroids: out nq x C
cudaError_t launch_coarse_dist(const DevIndex& ix, const float* q, const double* qnorm, int nq,
                               float* out, cudaStream_t st);
// per query, the w smallest (distance, centroid) of a nq x C distance block
cudaError_t launch_coarse_select(const float* dist, int nq, int C, int w, int32_t* coaidx,
                                 float* coadis, cudaStream_t st);
// fused residual + table + ADC scan + top-k (+ re-rank), one CTA per query
cudaError_t launch_scan(const DevIndex& ix, const ScanArgs& a, cudaStream_t st);

// persistent register-codebook scan (d = 128, ks = 256, m in {4, 8, 16},
// k or kl <= 1024) and its finalize kernel; `mid`, when given, is recorded between
// the two; returns cudaErrorNotSupported when not applicable
cudaError_t launch_scan_persistent(const DevIndex& ix, const ScanArgs& a, int num_sms, int threads,
                                   cudaStream_t st, cudaEvent_t mid = nullptr, bool finalize = true);
// the finalize kernel alone (order / re-score / re-rank the hand-off and write the results)
cudaError_t launch_finalize(const DevIndex& ix, const ScanArgs& a, cudaStream_t st);
bool scan_persistent_supported(const DevIndex& ix, const ScanArgs& a);
// candidate slots per query the persistent scan needs in ScanArgs::cand_*
int scan_persistent_stride(const ScanArgs& a);
// chunks per set of the precision form's re-score queue for nq queries and a hand-off stride
int rescore_queue_cap(int nq, int stride);

// List-centric scan (scan_lists.cu): the (query, list) pairs of a batch grouped by list, G queries
// per work item. Device workspace, sized by the host for nq queries, C lists and at most
// max_pairs (query, probe) pairs.
struct ListScanWork {
    int* w0 = nullptr;        // nq: the first pass's probe count per query
    int* pcnt = nullptr;      // C: pairs per list (zeroed at launch)
    int* pbeg = nullptr;      // C + 1: first pair of each list
    int* fill = nullptr;      // C: fill cursors
    int* gbeg = nullptr;      // C + 1: first group of each list
    int* bsum = nullptr;      // 2 x ceil(C / 4096): per block of lists, its pairs and groups (the prefix sums)
    int4* pairs = nullptr;    // max_pairs: (query, probe, position of the probe's first row, 0), by list
    int4* groups = nullptr;   // max_pairs x (1 + G): work-item descriptors (scan_lists.cu)
    int* counters = nullptr;  // [0] groups, [1] work counter, [2] overflowed queries
    unsigned long long* keysA = nullptr;  // nq x cand_stride: the first pass's best keys ...
    int* cntA = nullptr;                  // ... and their count
    unsigned long long* tau0 = nullptr;   // nq: the first pass's k-th key (KEY_MAX: fewer rows)
    unsigned long long* tau = nullptr;    // nq: the current bound, lowered during the scan
    unsigned int* hist = nullptr;         // nq x LC_HIST_BUCKETS: emitted keys by distance below tau0
    unsigned long long* ebuf = nullptr;   // nq x ecap: keys below tau from the list-centric pass ...
    int* ecnt = nullptr;                  // ... and their count (may exceed ecap: overflow)
    int ecap = 0;
    int32_t* ovf = nullptr;   // nq: the queries whose buffer overflowed
    int* err = nullptr;       // device error flag (a bounded wait ran out)
    int* queue_a = nullptr;   // work counters of the first pass and of the overflow pass
    int* queue_b = nullptr;
    int beta = 1;             // the first pass scans each query's nearest probes until beta * k_sel rows
};
constexpr int LC_HIST_BUCKETS = 256;
bool list_scan_supported(const DevIndex& ix, const ScanArgs& a);
int list_scan_ecap(const ScanArgs& a);
// The list-centric search pipeline up to the finalize hand-off (a.cand_*): planning, first pass,
// grouping, the list-centric scan, selection and the overflow pass. ev (optional, 5 events) marks
// its stages: first pass start/end, scan start/end, overflow pass start.
cudaError_t launch_list_scan(const DevIndex& ix, const ScanArgs& a, const ListScanWork& w, int num_sms,
                             cudaStream_t st, cudaEvent_t* ev);

// [min, max] of n int32 values on the device, returned to the host (synchronises the stream)
cudaError_t launch_id_range(const int32_t* ids, int64_t n, int* range, cudaStream_t st);
// rows of `width` bytes in list order (list l: rows off[l] .. off[l+1]) -> dst rows beg[l] ..
cudaError_t launch_scatter_rows(const uint8_t* src, const int64_t* off, const int64_t* beg, int C, int width,
                                uint8_t* dst, cudaStream_t st);

// mixed-precision coarse stage (d = 128): BF16 tiles, tcgen05 GEMM, exact re-check
cudaError_t launch_bf16_tiles(const float* x, int n, int rows_per_tile, uint8_t* out, cudaStream_t st);
cudaError_t launch_bf16_split_tiles(const float* x, int n, uint8_t* out, cudaStream_t st);
size_t coarse_mma_tile_bytes(int n, bool centroids);
// out: nq x C approximate distances; or, with amin, per (query, 128-centroid
// tile) the smallest (distance, centroid) key, nq x coarse_mma_ctiles(C)
cudaError_t launch_coarse_mma(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C, const double* qnorm,
                              const float* cnorm, float* out, int* err, cudaStream_t st,
                              unsigned long long* amin = nullptr);
int coarse_mma_ctiles(int C);
cudaError_t launch_coarse_recheck(const float* approx, int nq, int C, int w, const float* q, const double* qnorm,
                                  const float* coa, const float* cnorm, const float* clen, int32_t* coaidx,
                                  float* coadis, int* ncand, cudaStream_t st);
constexpr int MMA_QUERY_TILE = 128;

// Error bound of the BF16-split coarse distances (derivation in coarse_mma.cu):
// |approx - exact| <= mixed_eps(||q||^2, ||q||, ||c||^2, ||c||).
constexpr float MIXED_EPS_REL = 2.0f * 2.0f * (1.52587890625e-05f + 256.0f * 4.76837158203125e-07f);
__device__ __forceinline__ float mixed_eps(float qn, float qlen, float cn, float cl) {
    return MIXED_EPS_REL * qlen * cl + 9.5367431640625e-07f * (qn + cn);
}

// Filtered coarse stage for large C (coarse_filter.cu). Per query a bound
// thr[q] is taken from a sample of the centroids; the full pass appends every
// centroid that can beat it to the query's candidate slots and counts the
// centroids certainly within it; the exact keyed top-w is then taken over the
// candidates, or over all C when the count shows the bound was too low.
struct CoarseFilter {
    const float* thr = nullptr;  // nq: bound of each query
    int* cnt = nullptr;          // nq: centroids whose distance is certainly <= thr (NULL: = ncand)
    int* ncand = nullptr;        // nq: candidates appended (may exceed cap; only cap are stored)
    int32_t* cand = nullptr;     // nq x cap candidate centroids
    int cap = 0;
    const float* clen = nullptr;  // mixed form: centroid lengths (||c|| rounded up)
    // mixed form: the GEMM's pre-test survivors (centroid, accumulator bits),
    // per (query, centroid range, column half) up to sreg each, with their
    // counts (nq x 2*nsplit; a count above sreg means the region overflowed);
    // the exact candidate and count tests run in launch_coarse_cand_select
    int2* surv = nullptr;
    int* scnt = nullptr;
    int sreg = 0, nsplit = 0;
    // uneven batches: each query's probe count (<= w; NULL: w for all), so that its candidates and
    // selection cover its own top-wq only
    const int32_t* w_per_q = nullptr;
};
// the sample rank of each query of an uneven batch: min(r, ceil(scale * wq) + 8), wq = the query's
// probe count clamped to 1..w (w_per_q NULL: r for all)
struct SampleRank {
    const int32_t* w_per_q = nullptr;
    int w = 0;
    double scale = 0.0;
};
// sample size, rank and candidate capacity of the filtered stage; false when
// the plain select over the full distance block is used instead
bool coarse_filter_shape(int C, int w, int d, int* S, int* r, int* cap);
// the plain form's pass: exact distances (as launch_coarse_dist) filtered by f
cudaError_t launch_coarse_dist_filter(const DevIndex& ix, const float* q, const double* qnorm, int nq,
                                      const CoarseFilter& f, cudaStream_t st);
// the mixed form's pass: tcgen05 approximate distances filtered by f
cudaError_t launch_coarse_mma_filter(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                     const double* qnorm, const float* cnorm, const CoarseFilter& f, int* err,
                                     cudaStream_t st);
// persistent pipelined tcgen05 coarse GEMM (coarse_gemm.cu); query tiles for
// it hold coarse_gemm_qtile_bytes(nq) bytes (a multiple of two 128-row tiles);
// per-centroid columns colG = ||c||^2 (1 - 2^-20) / 2 (+inf past C) and
// colK = MIXED_EPS_REL ||c|| / 2 (0 past C) hold coarse_gemm_col_floats(C) floats
size_t coarse_gemm_qtile_bytes(int nq);
size_t coarse_gemm_col_floats(int C);
// approximate distances nq x C (row stride ld)
cudaError_t launch_coarse_gemm_store(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                     const double* qnorm, const float* cnorm, float* out, int64_t ld, int num_sms,
                                     int* err, cudaStream_t st, bool stall_copy = false);
// per query and 32 centroids, about the smallest upper bound approx + eps: nq x C/32 (C % 32 == 0)
cudaError_t launch_coarse_gemm_chunkmin(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                        const double* qnorm, const float* cnorm, const float* colG,
                                        const float* colK, float* out, int64_t ld, int num_sms, int* err,
                                        cudaStream_t st);
// centroid ranges per 256-query tile pair the persistent GEMM uses for (nq, C)
int coarse_gemm_nsplit(int nq, int C, int num_sms, int* split_tiles);
// nearest centroid by the approximate distance: part[q * 2 * nsplit + g] = the best key of each
// (centroid range, column half) g, nsplit = coarse_gemm_nsplit(nq, C, num_sms)
// (hi_only: the c_hi tiles alone, half the work, for index building)
cudaError_t launch_coarse_gemm_argmin(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C, const float* cnorm,
                                      unsigned long long* part, int num_sms, int* err, cudaStream_t st,
                                      bool hi_only = false);
// the mixed form's filtered pass (f.surv / f.scnt / f.sreg / f.nsplit as above);
// cn_max / clen_max: maxima of cnorm / f.clen
cudaError_t launch_coarse_gemm_filter(const uint8_t* qtiles, const uint8_t* ctiles, int nq, int C,
                                      const double* qnorm, const float* cnorm, const CoarseFilter& f,
                                      const float* colG, const float* colK, float cn_max, float clen_max,
                                      int num_sms, int* err, cudaStream_t st);
// thr[q] = a bound at about the r-th smallest of row q of a nq x L block (row
// stride ld): the r-th smallest of the minima of 512 interleaved groups (so
// at least r values lie at or below it); r <= 128 and r <= L
cudaError_t launch_coarse_sample_bound(const float* vals, int nq, int L, int64_t ld, int r, float* thr,
                                       cudaStream_t st, SampleRank sr = SampleRank());
// thr[q] = r-th smallest of a nq x S block of distances (clen != NULL: of the
// upper bounds approx + mixed_eps)
cudaError_t launch_coarse_sample_kth(const float* vals, int nq, int S, int r, const double* qnorm,
                                     const float* cnorm, const float* clen, float* thr, cudaStream_t st,
                                     SampleRank sr = SampleRank());
// exact keyed top-w per query from the candidates of f (stats[0] += candidates
// re-checked, stats[1] += queries that fell back to all C centroids)
cudaError_t launch_coarse_cand_select(const DevIndex& ix, const float* q, const double* qnorm, int nq, int w,
                                      const CoarseFilter& f, int32_t* coaidx, float* coadis, int* stats,
                                      cudaStream_t st);

// index building (build_gpu.cu); synchronous, allocate their own temporaries
// (hi_only, d = 128: centroids rounded to BF16 -- faster, not always the nearest; bulk index building)
cudaError_t assign_rows(const float* x, int64_t n, int64_t ld, int d, const float* cent, int k, int32_t* assign,
                        cudaStream_t st, bool hi_only = false);
cudaError_t kmeans_rows(const float* x, int64_t n, int64_t ld, int d, int k, int niter, uint64_t seed, float* cent,
                        cudaStream_t st);
cudaError_t gen_mixture(float* out, int64_t n, int d, const float* means, int ncomp, const double* cdf, float sigma,
                        uint64_t seed, uint64_t stream_id, int64_t row0, cudaStream_t st);
cudaError_t pq_train_rows(const float* r, int64_t n, int d, int m, int niter, uint64_t seed, float* pq,
                          cudaStream_t st);
cudaError_t pq_encode_rows(const float* x, int64_t n, int d, const int32_t* coarse, const float* coa, int m,
                           const float* pq, uint8_t* codes, cudaStream_t st);
// out = x - coa[coarse] - c1(codes) (coarse may be NULL), n x d
cudaError_t pq_error_rows(const float* x, int64_t n, int d, const int32_t* coarse, const float* coa, int m,
                          const float* pq, const uint8_t* codes, float* out, cudaStream_t st);

// largest k / kl / w the scan kernel supports
constexpr int MAX_K = 2048;
constexpr int MAX_W = 4096;

}  // namespace gbivf
