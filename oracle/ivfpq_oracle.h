/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle of the IVF-PQ search path.
 *
 * This header declares a plain-C restatement of rafaelms101/mestrado's
 * sequential IVF-PQ search (sequential/ivf_pq/ivf_search.cpp:9-203 and the
 * yael kernels it calls). Only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark load it, as the checker; the product
 * path (mestrado_gb300) never links or calls it.
 *
 * Index layout used by the oracle (same as the GPU engine's host input):
 *   coa      C x d    float32, row-major coarse centroids
 *   pq       m x ks x ds float32, sub-quantizer centroids [s][c][l]
 *   list_off C+1      int64, list l holds entries [list_off[l], list_off[l+1])
 *   ids      n        int32 base ids, list-contiguous
 *   codes    n x m    uint8 PQ codes, list-contiguous
 */
#ifndef IVFPQ_ORACLE_H
#define IVFPQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Tie rule for the two heap-based selections (coarse k-min and re-rank).
 * ORC_TIES_HEAP restates yael's binary max-heap exactly (ties follow the
 * heap, as the reference does). ORC_TIES_KEYED orders every selection by
 * (distance, index), the deterministic rule the GPU engine uses. */
#define ORC_TIES_HEAP 0
#define ORC_TIES_KEYED 1

/* Table formula. EXPANSION = ||r||^2 + ||c||^2 - 2 r.c as
 * compute_cross_distances (sequential/yael_needs/nn.c:120-150) with a
 * reference-order sgemm; DIRECT = sum (r-c)^2 as parallel2's dist2
 * (parallel2/ivf_pq/ivf_search.cpp:49-57). */
#define ORC_TABLE_EXPANSION 0
#define ORC_TABLE_DIRECT 1

typedef struct {
    int d, coarsek, m, ks;
    const float *coa;
    const float *pq;
    const int64_t *list_off;
    const int32_t *ids;
    const uint8_t *codes;
} orc_index;

/* compute_cross_distances_nonpacked (nn.c:120-150): dist2[i + ldd*j] =
 * ||a_i||^2 (float) + ||b_j||^2 (double) - 2 a_i.b_j (reference-order sgemm). */
void orc_cross_distances(int d, int na, int nb, const float *a, int lda,
                         const float *b, int ldb, float *dist2, int ldd);

/* knn_full (nn.c:463-537), L2 only: for each of n1 rows of mat1, the k
 * nearest of the n2 rows of mat2, ascending. */
void orc_knn_full(int n1, int n2, int d, int k, const float *mat2,
                  const float *mat1, int *vw, float *vwdis, int ties);

/* Exact k smallest of val[0..n), ascending, ties by position
 * (fvec_k_min, sequential/yael_needs/sorting.c:180-194). */
void orc_k_min(const float *val, int n, int k, int *idx);

/* ivfpq_search (sequential/ivf_pq/ivf_search.cpp:9-153). For each query:
 * coarse k-min (w), residuals, m x ks tables, ADC scan of the w lists,
 * k-min kl, then (rerank != 0) exact L2 re-rank of the kl candidates
 * against base to k. ids is nq x k row-major, 0-based base ids, padded
 * with -1 when fewer than k candidates exist. dis receives the re-rank
 * distances (or the ADC distances without rerank), +inf where padded.
 * Optional stage outputs (any may be NULL):
 *   coaidx/coadis  nq x w    coarse k-min
 *   adc_ids/adc_dis nq x kl  ADC k-min before re-rank (base ids), -1 pad
 * nthreads > 1 runs queries in parallel (OpenMP). Returns 0 on success. */
int orc_ivfpq_search(const orc_index *ix, const float *queries, int nq,
                     const float *base, int k, int kl, int w, int rerank,
                     int ties, int table_mode, int32_t *ids, float *dis,
                     int32_t *coaidx, float *coadis, int32_t *adc_ids,
                     float *adc_dis, int nthreads);

/* pq_search (sequential/pq-utils/pq_search.cpp:10-68): flat ADC over n
 * codes. Outputs are column-major (k x nq: element [l*nq + i]) and ids are
 * 1-based, as the reference writes them. */
int orc_pq_search(int d, int m, int ks, const float *pq, const uint8_t *codes,
                  int64_t n, const float *queries, int nq, int k, float *dis,
                  int32_t *ids, int nthreads);

/* core_cpu (parallel2/ivf_pq/ivf_search.cpp:61-117) given residuals
 * (nres x d, nres = nq*w) and rid_to_ivf: direct-sum tables, ADC scan and
 * an exact top-k per query, written packed at qid_to_starting_outid,
 * ascending by (distance, position). */
/* uneven batch (per-query nprobe and k, packed outputs at out_off[q]), no re-rank */
int orc_ivfpq_search_batched(const orc_index *ix, const float *queries, int nq,
                             const int32_t *w_per_q, const int32_t *k_per_q,
                             const int64_t *out_off, int ties, int32_t *ids,
                             float *dis, int nthreads);

int orc_core_cpu(const orc_index *ix, const float *residual, int nres,
                 const int32_t *rid_to_ivf, const int32_t *qid_to_starting_outid,
                 int32_t *idxs, float *dists, int k, int w, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
