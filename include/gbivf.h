/*
 * gbivf -- GB300-native IVF-PQ search, C ABI.
 *
 * Drop-in for the IVF-PQ search path of rafaelms101/mestrado. Every entry
 * point takes plain pointers and sizes, returns a status (GBIVF_OK or an
 * error code; gbivf_last_error() gives the message of the calling thread's
 * last failure) and never exits the process. Host-pointer entry points copy
 * their inputs to the GPU, run, copy the results back and return when the
 * results are in the caller's buffers. The caller owns every buffer; an
 * index handle owns its device memory, so a process may hold many indexes.
 *
 * Conventions kept from the reference:
 *   - index content: coarse centroids (C x d), nsq sub-quantizers of ks
 *     centroids each (ks <= 256, so codes are bytes), one inverted list per
 *     coarse centroid holding base ids and PQ codes;
 *   - ids are 0-based row-major nq x k for ivfpq_search
 *     (sequential/ivf_pq/ivf_search.cpp:133), 1-based column-major k x nq for
 *     pq_search (sequential/pq-utils/pq_search.cpp:58-63), packed at
 *     qid_to_starting_outid for core_gpu (parallel2/ivf_pq/ivf_search.cpp:
 *     127-149);
 *   - distances are squared L2 in the reference's float arithmetic.
 * Where the reference cannot return k results it asserts (nn.c:468); here
 * the missing slots are filled with id -1 and distance +inf.
 */
#ifndef GBIVF_H
#define GBIVF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBIVF_OK 0
#define GBIVF_ERR_INVALID 1     /* bad argument */
#define GBIVF_ERR_CUDA 2        /* CUDA runtime error */
#define GBIVF_ERR_NOMEM 3       /* device or host allocation failed */
#define GBIVF_ERR_UNSUPPORTED 4 /* valid but outside what this build supports */

/* search flags */
#define GBIVF_RERANK 0x1u       /* exact L2 re-rank of the kl ADC candidates to k */
#define GBIVF_TABLE_DIRECT 0x2u /* tables as sum (r-c)^2 (parallel2) instead of the expansion */
#define GBIVF_MIXED_COARSE 0x4u /* coarse stage as a BF16 tensor-core GEMM + exact FP32 re-check (d = 128);
                                   the probed lists are identical to the plain path's */
#define GBIVF_COARSE_FULL 0x8u  /* large C (>= 16384, w <= 1024): keep the full C-wide distance block and
                                   select from it, instead of the default sample-bound candidate filter;
                                   the results are the same either way */
#define GBIVF_MIXED_SCAN 0x10u  /* precision form of the scan (d = 128, ks = 256, m in {4, 8, 16}): PQ tables
                                   built approximately (packed fused multiply-adds) and held in FP16,
                                   summed in FP32; of the max(GBIVF_MIXED_SCAN_ALPHA * k, k +
                                   GBIVF_MIXED_SCAN_EXTRA) best (at most 4096),
                                   those within the tables' error bound of the k-th exact distance are
                                   re-scored in the reference's FP32 arithmetic, so every returned distance
                                   is the plain form's and the ids match it unless a true neighbour fell
                                   outside the approximate selection (gbivf_last_unproven counts the
                                   queries where that could not be excluded) */
#define GBIVF_MIXED_SCAN_ALPHA 2
#define GBIVF_MIXED_SCAN_EXTRA 64 /* the approximate selection is at least k + GBIVF_MIXED_SCAN_EXTRA */
#define GBIVF_RERANK_REFINE 0x20u /* re-rank the kl ADC candidates by the distance to their refined
                                     reconstruction y + c1(codes) + c2(refinement codes) instead of the
                                     raw vectors (needs gbivf_index_set_refine; k <= kl <= 1024). FP32:
                                     sequential sums over the 8 blocks of 16 dimensions, then the 8
                                     partial sums in block order */
#define GBIVF_MIXED_SCAN_AUTO 0x40u /* the engine picks the scan form: the precision form (as
                                     GBIVF_MIXED_SCAN) where gbivf_index_autotune, called with this flag,
                                     measured it faster on this index, else the exact form; on an index
                                     not tuned so, the precision form when m = 16 (its table build is
                                     cheap against the 4096-entry exact table). Falls back to the exact
                                     form where the precision form does not apply. Not combined with
                                     GBIVF_MIXED_SCAN */
#define GBIVF_LIST_SCAN 0x80u   /* scan list by list: the batch's (query, probe) pairs grouped by list,
                                   one work item per list and group of 4 (exact form) or 8 (precision
                                   form) queries, their tables interleaved so that one 16-byte shared
                                   load serves the group; each query's top-k through a threshold from
                                   a scan of its nearest probes. Same results as the per-query scan.
                                   Not with GBIVF_TABLE_DIRECT or GBIVF_QUERY_SCAN */
#define GBIVF_QUERY_SCAN 0x200u /* scan query by query (one CTA per query at a time). Without either
                                   flag the engine picks: the autotuner's measured choice, else the
                                   list-centric scan for batches of at least 1024 queries on an index
                                   whose lists average at most 768 codes, where it applies */
#define GBIVF_PROFILE 0x100u    /* record CUDA events around the coarse and scan stages */
#define GBIVF_ERR_TIMEOUT 5     /* a bounded device-side wait ran out (the kernel stopped and reported it) */

typedef struct gbivf_index gbivf_index;

const char *gbivf_last_error(void);
int gbivf_version(void);

/* Upload an IVF-PQ index (flat layout). coa: coarsek x d; pq: nsq x ks x
 * (d/nsq), sub-quantizer s centroid c at pq[(s*ks + c)*(d/nsq)]; list l
 * holds rows list_off[l] .. list_off[l+1]-1 of ids (int32) and codes
 * (nsq bytes per row).
 * Replaces: preallocate_gpu_mem(pqtipo, ivf_t*, int)
 * (parallel2/ivf_pq/mycuda.h:8) and the ivfpq_t / ivf_t arguments of
 * ivfpq_search (sequential/ivf_pq/ivf_search.h:20). */
int gbivf_index_create(gbivf_index **out, int device, int d, int coarsek, const float *coa,
                       int nsq, int ks, const float *pq, const int64_t *list_off,
                       const int32_t *ids, const uint8_t *codes);

/* gbivf_index_create with the lists already in device memory (d_ids: n int32,
 * d_codes: n x nsq bytes, list order as list_off gives it; ks must be 256):
 * for indexes built on the GPU, where a host copy of billions of codes would
 * be the slowest step. coa, pq and list_off are host arrays. */
int gbivf_index_create_device(gbivf_index **out, int device, int d, int coarsek, const float *coa, int nsq, int ks,
                              const float *pq, const int64_t *list_off, const int32_t *d_ids,
                              const uint8_t *d_codes);

/* Upload an index given as the reference holds it: ivfpq_t fields plus one
 * ivf_t per list (ids, idstam, int32 codes n x nsq).
 * pq_centroids[s] is the ks x ds array of sub-quantizer s (pqtipo.centroids,
 * sequential/pq-utils/pq_new.h:26-33); list_ids[l] / list_codes[l] /
 * list_sizes[l] are ivf[l].ids / ivf[l].codes.mat / ivf[l].idstam
 * (sequential/ivf_pq/myIVF.h:23-27). Codes must be < ks <= 256.
 * Replaces: preallocate_gpu_mem (parallel2/ivf_pq/mycuda.cu:193-221). */
int gbivf_index_create_from_lists(gbivf_index **out, int device, int d, int coarsek,
                                  const float *coa, int nsq, int ks,
                                  const float *const *pq_centroids, const int32_t *list_sizes,
                                  const int32_t *const *list_ids,
                                  const int32_t *const *list_codes);

/* Refinement codes for GBIVF_RERANK_REFINE (no counterpart in the reference):
 * a second product quantizer of the residual error e = x - y_list - c1(codes),
 * m2 sub-quantizers of 256 centroids (pq2: m2 x 256 x 128/m2 floats, host),
 * and one m2-byte code per indexed vector in the order of the index's ids
 * (host codes2, or device d_codes2). d = 128. */
int gbivf_index_set_refine(gbivf_index *ix, int m2, int ks2, const float *pq2, const uint8_t *codes2);
int gbivf_index_set_refine_device(gbivf_index *ix, int m2, int ks2, const float *pq2, const uint8_t *d_codes2);

/* Raw base vectors (n x d, row id = base id) for GBIVF_RERANK: the
 * `mat vbase` argument of ivfpq_search (sequential/ivf_pq/ivf_search.cpp:9,
 * 115-121), uploaded once instead of per call. */
int gbivf_index_set_base(gbivf_index *ix, const float *base, int64_t n, int d);

/* Replaces: deallocate_gpu_mem() (parallel2/ivf_pq/mycuda.h:9). */
int gbivf_index_destroy(gbivf_index *ix);

/* d, coarsek, nsq, ks, number of stored vectors (any pointer may be NULL). */
int gbivf_index_dims(const gbivf_index *ix, int *d, int *coarsek, int *nsq, int *ks, int64_t *n);

/* ivfpq_search(ivfpq, ivf, vquery, vbase, k, kl, w, ids, dis)
 * (sequential/ivf_pq/ivf_search.cpp:9-153). queries: nq x d host floats.
 * With GBIVF_RERANK: the kl best ADC candidates are re-ranked by exact L2
 * against the base set with gbivf_index_set_base, keeping k (the reference
 * always re-ranks). Without it: the k best ADC candidates (kl ignored).
 * ids: nq x k (0-based base ids), dis: nq x k distances (the reference
 * leaves dis unwritten; here it receives the re-rank or ADC distances). */
int gbivf_ivfpq_search(gbivf_index *ix, const float *queries, int nq, int k, int kl, int w,
                       unsigned flags, int32_t *ids, float *dis);

/* Same, with device pointers, enqueued on `stream` (a cudaStream_t, NULL =
 * the default stream); returns after launching. */
int gbivf_ivfpq_search_device(gbivf_index *ix, const float *d_queries, int nq, int k, int kl,
                              int w, unsigned flags, int32_t *d_ids, float *d_dis, void *stream);

/* Uneven batch (many queries with their own nprobe and k in one launch
 * sequence, as the batched workload needs): query q probes w_per_q[q] lists
 * (1..coarsek) and returns k_per_q[q] results; results are packed, query q's
 * at the exclusive prefix sum of k_per_q (ids/dis hold sum(k_per_q)
 * entries), ascending, -1 / +inf padded. No re-rank. Host buffers.
 * No counterpart in the reference, whose calls share one k and w. */
int gbivf_search_batched(gbivf_index *ix, const float *queries, int nq, const int32_t *w_per_q,
                         const int32_t *k_per_q, unsigned flags, int32_t *ids, float *dis);

/* Same with device buffers: d_w / d_k per query (values are clamped to
 * 1..max_w / 1..max_k), d_out_off the output offset of each query; max_w and
 * max_k bound them. Enqueued on `stream`; returns after launching. */
int gbivf_search_batched_device(gbivf_index *ix, const float *d_queries, int nq, const int32_t *d_w,
                                const int32_t *d_k, const int64_t *d_out_off, int max_w, int max_k,
                                unsigned flags, int32_t *d_ids, float *d_dis, void *stream);

/* A search captured as a CUDA graph, replayed with one launch.
 * gbivf_graph_capture runs the described device-buffer search once on
 * `stream` (sizing the index's workspace), then captures the same launch
 * sequence; gbivf_graph_launch replays it on any stream with whatever the
 * buffers hold at that time. Arguments are those of
 * gbivf_ivfpq_search_device, plus optional d_w / d_k / d_out_off (all three,
 * k and w as maxima) for an uneven batch as gbivf_search_batched_device
 * takes them. Replays share the index's workspace: do not overlap them with
 * other searches on the same index. */
typedef struct gbivf_graph gbivf_graph;
int gbivf_graph_capture(gbivf_index *ix, const float *d_queries, int nq, int k, int kl, int w,
                        unsigned flags, int32_t *d_ids, float *d_dis, const int32_t *d_w,
                        const int32_t *d_k, const int64_t *d_out_off, void *stream, gbivf_graph **out);
int gbivf_graph_launch(gbivf_graph *g, void *stream);
int gbivf_graph_destroy(gbivf_graph *g);
/* Kernel launches one replay of the graph makes (its kernel nodes; memsets
 * and copies are not counted). No counterpart in the reference. */
int gbivf_graph_kernel_count(const gbivf_graph *g, int *kernels);

/* Autotuner: times the scan kernels that can serve this index and search
 * shape (persistent register-codebook kernel with 512 or 1024 threads, the
 * general kernel, or the list-centric pipeline) on a calibration batch of
 * device queries, keeps the fastest for later searches on this index (the
 * list-centric choice applies to batches of 1024 queries or more, as the
 * engine's own rule does) and reports it in *choice (512, 1024, 0 for the
 * general kernel, 1 for the list-centric pipeline); times_ms (4 entries, may
 * be NULL) receives each variant's scan time, -1 where it does not apply. When the environment
 * variable GBIVF_TUNE_CACHE names a file, choices are read from and appended
 * to it, keyed by index shape, list-size histogram, GPU and search shape. */
/* The scan form GBIVF_MIXED_SCAN_AUTO resolves to on this index: *tuned = 1 once gbivf_index_autotune
 * measured it (with that flag), *mixed = 1 for the precision form. No counterpart in the reference. */
int gbivf_index_scan_form(const gbivf_index *ix, int *tuned, int *mixed);
int gbivf_index_autotune(gbivf_index *ix, const float *d_queries, int nq, int k, int kl, int w,
                         unsigned flags, int *choice, float *times_ms);

/* Stage times (milliseconds, CUDA events on the launching stream) of the
 * last search made with GBIVF_PROFILE: coarse assignment (query norms,
 * distances, k-min) and the fused scan (tables, ADC, top-k, re-rank).
 * Waits for that search to finish. No counterpart in the reference, which
 * prints gettimeofday deltas (sequential/ivf_pq/ivf_search.cpp:105-111). */
int gbivf_last_stage_ms(gbivf_index *ix, float *coarse_ms, float *scan_ms);

/* The same with the scan split in two: the scan kernels (tables, ADC, top-k)
 * and the finalize kernels (ordering, the precision form's exact re-score,
 * RERANK or the refinement re-rank). scan_ms + finalize_ms is the scan time
 * of gbivf_last_stage_ms. */
int gbivf_last_stages_ms(gbivf_index *ix, float *coarse_ms, float *scan_ms, float *finalize_ms);

/* The parts of the last GBIVF_PROFILE search's scan stage when it ran list by
 * list (GBIVF_LIST_SCAN), in ms: [0] planning, [1] the first pass over each
 * query's nearest probes, [2] grouping the pairs by list, [3] the list-centric
 * scan kernel, [4] selection, [5] the pass over overflowed queries, [6]
 * finalize; and its counters: [0] (query, probe) pairs scanned list by list,
 * [1] work items, [2] queries that overflowed their buffer, [3] 1 if the scan
 * ran list by list. Either array may be NULL. Waits for the search. No
 * counterpart in the reference. */
int gbivf_last_scan_parts(gbivf_index *ix, float *parts_ms, int64_t *counters);

/* The number of queries of the last search with GBIVF_MIXED_SCAN whose result
 * the precision form could not prove identical to the exact form's (0 after a
 * search without it). The precision form re-scores, in the reference's FP32
 * arithmetic, every approximate candidate whose approximate distance lies
 * within the FP16 tables' error bound of the k-th (kl-th) exact distance; a
 * query is proven when all such candidates were among the GBIVF_MIXED_SCAN_ALPHA
 * * k approximate best it kept. Read once the search has completed (after the
 * host call returns, or after the caller synchronised a device search's
 * stream). No counterpart in the reference. */
int gbivf_last_unproven(gbivf_index *ix, int64_t *queries);

/* The coarse stage alone: knn_full(2, nq, C, d, w, coa, queries, ...)
 * (sequential/ivf_pq/ivf_search.cpp:37-38): the w nearest lists per query,
 * ascending. coaidx, coadis: nq x w host arrays. */
int gbivf_coarse_assign(gbivf_index *ix, const float *queries, int nq, int w, int32_t *coaidx,
                        float *coadis);

/* Size of the device scratch array behind gbivf_coarse_assign_noalloc. */
#define GBIVF_NOALLOC_SCRATCH_BYTES (16u << 20)

/* The coarse stage for callers that cannot allocate device memory (a host
 * that gives plugins a fixed device-memory budget and forbids allocation, or
 * a serving loop that must not take cudaMalloc's device-wide
 * synchronisation). Same results as gbivf_coarse_assign, on device buffers:
 * d_queries nq x d, d_coaidx / d_coadis nq x w, enqueued on `stream`
 * (a cudaStream_t, NULL = default stream); returns after launching. It
 * allocates nothing: its scratch is one file-scope device array of
 * GBIVF_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit, so nq * (8 + 4 * coarsek) plus alignment must fit in it (larger
 * calls return GBIVF_ERR_UNSUPPORTED; split the batch: 4,088 queries at
 * coarsek = 1024). The first call on a device, and the first after the
 * device's context was replaced (cudaDeviceReset), looks up the array's
 * address (cudaGetSymbolAddress), so make it before any stream capture.
 * Calls that overlap on the GPU share the array and race. No counterpart in
 * the reference. */
int gbivf_coarse_assign_noalloc(gbivf_index *ix, const float *d_queries, int nq, int w,
                                int32_t *d_coaidx, float *d_coadis, void *stream);

/* gbivf_coarse_assign with search flags (GBIVF_MIXED_COARSE selects the
 * tensor-core form, GBIVF_COARSE_FULL the full-block selection). `ncand`,
 * when not NULL, receives the number of centroids re-checked exactly after
 * the first pass (0 for the plain form over the full block). */
int gbivf_coarse_assign_flags(gbivf_index *ix, const float *queries, int nq, int w, unsigned flags,
                              int32_t *coaidx, float *coadis, int64_t *ncand);

/* The coarse stage on device buffers, enqueued on `stream` (returns after
 * launching; allocates workspace on first use): d_coaidx / d_coadis nq x w.
 * flags: GBIVF_MIXED_COARSE, GBIVF_COARSE_FULL. A device-side timeout of the
 * tensor-core form is reported by the next synchronous call on the index. */
int gbivf_coarse_assign_device(gbivf_index *ix, const float *d_queries, int nq, int w, unsigned flags,
                               int32_t *d_coaidx, float *d_coadis, void *stream);

/* Work counters of the last gbivf_coarse_assign_flags call: centroids whose
 * distance was computed exactly after the first pass (the candidates of the
 * mixed form or of the large-C filter) and queries for which the large-C
 * filter's sample bound proved too low, so that all C centroids were taken
 * exactly. Either may be NULL. No counterpart in the reference. */
int gbivf_last_coarse_stats(gbivf_index *ix, int64_t *rechecked, int64_t *fallback_queries);

/* core_gpu(PQ, residual, ivf, ivf_size, rid_to_ivf, qid_to_starting_outid,
 * idxs, dists, k, w) (parallel2/ivf_pq/mycuda.cu:119-188): residual is
 * nres x d (nres = nq*w), list rid_to_ivf[r] for residual r; tables are the
 * direct sum of squared differences (mycuda.cu:59-64). For query q the
 * min(k, sum of its lists' sizes) best (distance, base id) are written
 * ascending at qid_to_starting_outid[q]. */
int gbivf_core_gpu(gbivf_index *ix, const float *residual, int nres, const int32_t *rid_to_ivf,
                   const int32_t *qid_to_starting_outid, int32_t *idxs, float *dists, int k,
                   int w);

/* Flat PQ: upload n codes (n x nsq bytes) with their quantizer.
 * Replaces the codebook / pqtipo arguments of pq_search
 * (sequential/pq-utils/pq_search.h:21). */
int gbivf_pq_create(gbivf_index **out, int device, int d, int nsq, int ks, const float *pq,
                    const uint8_t *codes, int64_t n);

/* pq_search(pq, codebook, vquery, k, dis, ids)
 * (sequential/pq-utils/pq_search.cpp:10-68): exhaustive ADC, k best per
 * query; dis and ids are k x nq column-major, ids 1-based. k <= n. */
int gbivf_pq_search(gbivf_index *ix, const float *queries, int nq, int k, float *dis,
                    int32_t *ids);

/* ---- index building on the GPU (device buffers; return when done) ----
 * The reference trains and encodes on one CPU thread with yael's k-means and
 * exact 1-NN (sequential/ivf_pq/ivf_new.cpp:4-33, ivf_assign.cpp:3-52,
 * pq-utils/pq_new.cpp:6-59, pq-utils/pq_assign.cpp:12-53); these replace
 * those steps for large base sets. Assignment to d = 128 centroids runs on
 * the tensor cores; centroid sums accumulate in FP64. */

/* n x d byte-valued vectors of a Gaussian mixture: component c (uniform, or
 * drawn through d_cdf, the cumulative weights of ncomp components), value
 * clip(round(means[c] + sigma * N(0,1)), 0, 255). Counter-based: rows
 * row0 .. row0+n-1 of stream `stream_id` are the same whatever the chunking. */
int gbivf_generate_mixture(float *d_out, int64_t n, int d, const float *d_means, int ncomp,
                           const double *d_cdf, float sigma, uint64_t seed, uint64_t stream_id,
                           int64_t row0, void *stream);

/* Lloyd k-means, niter iterations (d = 128, or 8, 16, 32), k x d centroids. */
int gbivf_kmeans(const float *d_x, int64_t n, int d, int k, int niter, uint64_t seed,
                 float *d_centroids, void *stream);

/* Nearest of k centroids for each of n rows (d = 128, or 8, 16, 32). */
int gbivf_assign(const float *d_x, int64_t n, int d, const float *d_centroids, int k,
                 int32_t *d_assign, void *stream);

/* gbivf_assign with flags: GBIVF_ASSIGN_BF16 (d = 128) compares against the
 * centroids rounded to BF16 -- half the tensor-core work of the default
 * split form, and not always the nearest centroid: for bulk index building. */
#define GBIVF_ASSIGN_BF16 0x1u
int gbivf_assign_flags(const float *d_x, int64_t n, int d, const float *d_centroids, int k, int32_t *d_assign,
                       unsigned flags, void *stream);

/* Sub-quantizers: m k-means of 256 centroids on the sub-vectors of the
 * residuals d_r (n x d); d_pq receives m x 256 x (d/m). */
int gbivf_pq_train(const float *d_r, int64_t n, int d, int m, int niter, uint64_t seed, float *d_pq,
                   void *stream);

/* The residual error a refinement quantizer encodes: d_out = x - coa[coarse]
 * - c1(codes), n x d (d_coarse may be NULL). Device buffers; synchronous. */
int gbivf_pq_error(const float *d_x, int64_t n, int d, const int32_t *d_coarse, const float *d_coa, int m,
                   const float *d_pq, const uint8_t *d_codes, float *d_out, void *stream);

/* PQ codes (n x m bytes) of rows d_x, of their residuals to d_coa[d_coarse[i]]
 * when d_coarse is not NULL. */
int gbivf_pq_encode(const float *d_x, int64_t n, int d, const int32_t *d_coarse, const float *d_coa,
                    int m, const float *d_pq, uint8_t *d_codes, void *stream);

/* Self-test of the bounded device-side waits (no counterpart in the reference):
 * runs one CTA of the tensor-core coarse product with its first centroid-tile
 * copy withheld, so that the wait for it runs out (after about 2 s of the
 * global timer); the kernel must stop, report it (timed_out = 1) and leave
 * the context usable, which a second, normal run checks (clean_ok = 1).
 * stalled_ms: the stalled launch's duration. Nothing faults. */
int gbivf_selftest_wait_timeout(int device, int *timed_out, float *stalled_ms, int *clean_ok);

#ifdef __cplusplus
}
#endif

#endif /* GBIVF_H */
