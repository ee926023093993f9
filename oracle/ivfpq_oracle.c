/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle for the IVF-PQ search path.
 *
 * A plain-C restatement of the search path of rafaelms101/mestrado,
 * written from the reference's behaviour (not its text). The tests, the
 * smoke check and the benchmark's CPU-baseline leg use it as the checker
 * and as the timed CPU implementation; the GPU engine never calls it.
 *
 * Arithmetic follows the reference order exactly so that results can be
 * compared bit for bit:
 *   - squared norms of the "a" operand: float, sequential
 *     (sequential/yael_needs/nn.c:129-135);
 *   - squared norms of the "b" operand: double accumulation of float
 *     products, added to the float norm in double and rounded to float
 *     (nn.c:137-145);
 *   - the -2 a.b term: a reference-order (netlib loop order) sgemm, i.e. a
 *     float dot product summed in ascending index with no fused multiply-add,
 *     then c = (-2 * dot) + c (nn.c:76-88);
 *   - the ADC sum: float, sequential over sub-quantizers starting from 0
 *     (sequential/ivf_pq/ivf_search.cpp:189-200).
 * Build with -ffp-contract=off so that no multiply-add is fused.
 */
#include "ivfpq_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* reference-order distance arithmetic                                  */
/* ------------------------------------------------------------------ */

/* float norm, sequential (nn.c:129-135) */
static float norm_f(const float *a, int d) {
    float s = 0.0f;
    for (int j = 0; j < d; j++) {
        float p = a[j] * a[j];
        s = s + p;
    }
    return s;
}

/* double accumulation of float products (nn.c:137-142) */
static double norm_d(const float *b, int d) {
    double s = 0.0;
    for (int j = 0; j < d; j++) {
        float p = b[j] * b[j];
        s = s + (double)p;
    }
    return s;
}

/* the sgemm inner product, netlib order: TEMP = TEMP + A(L,I)*B(L,J) */
static float dot_f(const float *a, const float *b, int d) {
    float t = 0.0f;
    for (int l = 0; l < d; l++) {
        float p = a[l] * b[l];
        t = t + p;
    }
    return t;
}

/* one expansion-form distance given the two norms (nn.c:143-145 + 85-86) */
static float expansion_dist(float norm_a, double norm_b, const float *a,
                            const float *b, int d) {
    float c = (float)(norm_b + (double)norm_a);
    float t = dot_f(a, b, d);
    float m2t = -2.0f * t;
    return m2t + c;
}

/* parallel2's dist2 (parallel2/ivf_pq/ivf_search.cpp:49-57) */
static float direct_dist(const float *a, const float *b, int d) {
    float s = 0.0f;
    for (int i = 0; i < d; i++) {
        float diff = a[i] - b[i];
        float p = diff * diff;
        s = s + p;
    }
    return s;
}

void orc_cross_distances(int d, int na, int nb, const float *a, int lda,
                         const float *b, int ldb, float *dist2, int ldd) {
    float *na2 = (float *)malloc(sizeof(float) * (na > 0 ? na : 1));
    for (int i = 0; i < na; i++) na2[i] = norm_f(a + (long)lda * i, d);
    for (int j = 0; j < nb; j++) {
        double nb2 = norm_d(b + (long)ldb * j, d);
        for (int i = 0; i < na; i++)
            dist2[(long)j * ldd + i] = (float)(nb2 + (double)na2[i]);
    }
    for (int j = 0; j < nb; j++)
        for (int i = 0; i < na; i++) {
            float t = dot_f(a + (long)lda * i, b + (long)ldb * j, d);
            float m2t = -2.0f * t;
            dist2[(long)j * ldd + i] = m2t + dist2[(long)j * ldd + i];
        }
    free(na2);
}

/* ------------------------------------------------------------------ */
/* selection                                                            */
/* ------------------------------------------------------------------ */

/* monotone map float -> uint32 (negative values below positive ones) */
static uint32_t fkey(float f) {
    f = f + 0.0f; /* -0 -> +0 */
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static int cmp_u64(const void *x, const void *y) {
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* Hoare-partition quickselect: afterwards a[0..k) holds the k smallest */
static void select_u64(uint64_t *a, long n, long k) {
    long lo = 0, hi = n - 1, want = k - 1;
    while (hi > lo) {
        uint64_t x = a[lo], y = a[(lo + hi) / 2], z = a[hi], piv;
        if (x < y) piv = (y < z) ? y : ((x < z) ? z : x);
        else piv = (x < z) ? x : ((y < z) ? z : y);
        long i = lo, j = hi;
        while (i <= j) {
            while (a[i] < piv) i++;
            while (a[j] > piv) j--;
            if (i <= j) {
                uint64_t t = a[i];
                a[i] = a[j];
                a[j] = t;
                i++;
                j--;
            }
        }
        if (want <= j) hi = j;
        else if (want >= i) lo = i;
        else break;
    }
}

/* k smallest keys of a[0..n) sorted ascending into a[0..k) */
static void topk_u64(uint64_t *a, long n, long k) {
    if (k <= 0) return;
    if (k < n) select_u64(a, n, k);
    qsort(a, (size_t)(k < n ? k : n), sizeof(uint64_t), cmp_u64);
}

void orc_k_min(const float *val, int n, int k, int *idx) {
    if (n <= 0 || k <= 0) return;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * n);
    for (int i = 0; i < n; i++) keys[i] = ((uint64_t)fkey(val[i]) << 32) | (uint32_t)i;
    topk_u64(keys, n, k);
    for (int i = 0; i < k && i < n; i++) idx[i] = (int)(uint32_t)keys[i];
    free(keys);
}

/* yael's binary max-heap, 1-based (sequential/yael_needs/binheap.c:102-170) */
typedef struct {
    int k, maxk;
    float *val;   /* val[1..maxk] */
    int *label;   /* label[1..maxk] */
} mheap;

static void mheap_push(mheap *h, int label, float v) {
    int i = ++h->k;
    while (i > 1) {
        int f = i >> 1;
        if (h->val[f] >= v) break;
        h->val[i] = h->val[f];
        h->label[i] = h->label[f];
        i = f;
    }
    h->val[i] = v;
    h->label[i] = label;
}

static void mheap_pop(mheap *h) {
    float v = h->val[h->k];
    int i = 1;
    for (;;) {
        int i1 = i << 1, i2 = i1 + 1;
        if (i1 > h->k) break;
        if (i2 == h->k + 1 || h->val[i1] > h->val[i2]) {
            if (v > h->val[i1]) break;
            h->val[i] = h->val[i1];
            h->label[i] = h->label[i1];
            i = i1;
        } else {
            if (v > h->val[i2]) break;
            h->val[i] = h->val[i2];
            h->label[i] = h->label[i2];
            i = i2;
        }
    }
    h->val[i] = h->val[h->k];
    h->label[i] = h->label[h->k];
    h->k--;
}

/* feed v[0..n) with labels 0..n-1 (fbinheap_addn_label_range) */
static void mheap_addn(mheap *h, int n, const float *v) {
    int i;
    for (i = 0; i < n && h->k < h->maxk; i++)
        if (!isnan(v[i])) mheap_push(h, i, v[i]);
    if (h->k == 0) return;
    float lim = h->val[1];
    for (; i < n; i++) {
        if (v[i] < lim) {
            mheap_pop(h);
            mheap_push(h, i, v[i]);
            lim = h->val[1];
        }
    }
}

/* fbinheap_sort: order by value, then heap slot (sorting.c:216-219) */
static void mheap_sort(const mheap *h, int *lab, float *val) {
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (h->k > 0 ? h->k : 1));
    for (int i = 0; i < h->k; i++)
        keys[i] = ((uint64_t)fkey(h->val[i + 1]) << 32) | (uint32_t)i;
    qsort(keys, (size_t)h->k, sizeof(uint64_t), cmp_u64);
    for (int i = 0; i < h->k; i++) {
        int slot = (int)(uint32_t)keys[i] + 1;
        lab[i] = h->label[slot];
        val[i] = h->val[slot];
    }
    free(keys);
}

/* k smallest of v[0..n) into (lab, val): reference heap rule or keyed rule.
 * Slots beyond the available count get label -1 and value +inf. */
static void select_k(const float *v, int n, int k, int ties, int *lab, float *val) {
    int got = 0;
    if (k == 1) {
        /* nn_single_full (nn.c:404-458): strict '<' from 1e30 */
        float best = 1e30f;
        int bi = -1;
        for (int i = 0; i < n; i++)
            if (v[i] < best) {
                best = v[i];
                bi = i;
            }
        lab[0] = bi;
        val[0] = bi < 0 ? INFINITY : best;
        return;
    }
    if (ties == ORC_TIES_HEAP) {
        mheap h;
        h.k = 0;
        h.maxk = k;
        h.val = (float *)malloc(sizeof(float) * (k + 1));
        h.label = (int *)malloc(sizeof(int) * (k + 1));
        mheap_addn(&h, n, v);
        mheap_sort(&h, lab, val);
        got = h.k;
        free(h.val);
        free(h.label);
    } else {
        uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (n > 0 ? n : 1));
        int nn = 0;
        for (int i = 0; i < n; i++)
            if (!isnan(v[i])) keys[nn++] = ((uint64_t)fkey(v[i]) << 32) | (uint32_t)i;
        got = k < nn ? k : nn;
        topk_u64(keys, nn, got);
        for (int i = 0; i < got; i++) {
            lab[i] = (int)(uint32_t)keys[i];
            val[i] = v[lab[i]];
        }
        free(keys);
    }
    for (int i = got; i < k; i++) {
        lab[i] = -1;
        val[i] = INFINITY;
    }
}

void orc_knn_full(int n1, int n2, int d, int k, const float *mat2,
                  const float *mat1, int *vw, float *vwdis, int ties) {
    float *na = (float *)malloc(sizeof(float) * (n2 > 0 ? n2 : 1));
    float *dist = (float *)malloc(sizeof(float) * (n2 > 0 ? n2 : 1));
    for (int i = 0; i < n2; i++) na[i] = norm_f(mat2 + (long)i * d, d);
    for (int q = 0; q < n1; q++) {
        const float *x = mat1 + (long)q * d;
        double nb = norm_d(x, d);
        for (int i = 0; i < n2; i++) dist[i] = expansion_dist(na[i], nb, mat2 + (long)i * d, x, d);
        select_k(dist, n2, k, ties, vw + (long)q * k, vwdis + (long)q * k);
    }
    free(na);
    free(dist);
}

/* ------------------------------------------------------------------ */
/* IVF-PQ search                                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    float *coa_norm; /* C, float (a-operand norms of the coarse product) */
    double *pq_norm; /* m*ks, double (b-operand norms of the table product) */
} orc_pre;

static int pre_init(const orc_index *ix, orc_pre *p) {
    int ds = ix->d / ix->m;
    p->coa_norm = (float *)malloc(sizeof(float) * ix->coarsek);
    p->pq_norm = (double *)malloc(sizeof(double) * ix->m * ix->ks);
    if (!p->coa_norm || !p->pq_norm) return -1;
    for (int c = 0; c < ix->coarsek; c++) p->coa_norm[c] = norm_f(ix->coa + (long)c * ix->d, ix->d);
    for (int e = 0; e < ix->m * ix->ks; e++) p->pq_norm[e] = norm_d(ix->pq + (long)e * ds, ds);
    return 0;
}

static void pre_free(orc_pre *p) {
    free(p->coa_norm);
    free(p->pq_norm);
}

/* m x ks table for one residual (ivf_search.cpp:82-87, or parallel2's
 * direct form). r is the d-dimensional residual. */
static void build_table(const orc_index *ix, const orc_pre *pre, const float *r,
                        int table_mode, float *tab) {
    int ds = ix->d / ix->m;
    for (int s = 0; s < ix->m; s++) {
        const float *rs = r + s * ds;
        float rn = norm_f(rs, ds);
        for (int c = 0; c < ix->ks; c++) {
            const float *cen = ix->pq + ((long)s * ix->ks + c) * ds;
            tab[s * ix->ks + c] = (table_mode == ORC_TABLE_DIRECT)
                                      ? direct_dist(rs, cen, ds)
                                      : expansion_dist(rn, pre->pq_norm[s * ix->ks + c], rs, cen, ds);
        }
    }
}

/* sumidxtab2 (ivf_search.cpp:182-203) over one list */
static void adc_scan(const orc_index *ix, const float *tab, long beg, long n, float *out) {
    int m = ix->m, ks = ix->ks;
    for (long i = 0; i < n; i++) {
        const uint8_t *code = ix->codes + (beg + i) * m;
        float acc = 0.0f;
        for (int s = 0; s < m; s++) acc = acc + tab[s * ks + code[s]];
        out[i] = acc;
    }
}

static int check_index(const orc_index *ix) {
    if (!ix || ix->d <= 0 || ix->m <= 0 || ix->d % ix->m || ix->ks <= 0 || ix->ks > 256 ||
        ix->coarsek <= 0)
        return -1;
    return 0;
}

int orc_ivfpq_search(const orc_index *ix, const float *queries, int nq,
                     const float *base, int k, int kl, int w, int rerank,
                     int ties, int table_mode, int32_t *ids, float *dis,
                     int32_t *coaidx, float *coadis, int32_t *adc_ids,
                     float *adc_dis, int nthreads) {
    if (check_index(ix) || nq < 0 || k <= 0 || w <= 0 || w > ix->coarsek) return -1;
    if (rerank && (kl <= 0 || !base)) return -1;
    int kk = rerank ? kl : k; /* width of the ADC k-min */
    orc_pre pre;
    if (pre_init(ix, &pre)) return -2;
    const int d = ix->d, C = ix->coarsek;
    int err = 0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 2) num_threads(nthreads)
#endif
    for (int q = 0; q < nq; q++) {
        const float *x = queries + (long)q * d;
        float *cd = (float *)malloc(sizeof(float) * C);
        int *qco = (int *)malloc(sizeof(int) * w);
        float *qcd = (float *)malloc(sizeof(float) * w);
        float *r = (float *)malloc(sizeof(float) * d);
        float *tab = (float *)malloc(sizeof(float) * ix->m * ix->ks);
        if (!cd || !qco || !qcd || !r || !tab) {
            err = -2;
            free(cd); free(qco); free(qcd); free(r); free(tab);
            continue;
        }
        /* coarse: knn_full(2, nq, C, d, w, coa, queries) (ivf_search.cpp:37-38) */
        double xn = norm_d(x, d);
        for (int c = 0; c < C; c++)
            cd[c] = expansion_dist(pre.coa_norm[c], xn, ix->coa + (long)c * d, x, d);
        select_k(cd, C, w, ties, qco, qcd);
        if (coaidx)
            for (int j = 0; j < w; j++) coaidx[(long)q * w + j] = qco[j];
        if (coadis)
            for (int j = 0; j < w; j++) coadis[(long)q * w + j] = qcd[j];

        /* candidates of the w probed lists, in probe order (:72-96) */
        long L = 0;
        for (int j = 0; j < w; j++)
            if (qco[j] >= 0) L += ix->list_off[qco[j] + 1] - ix->list_off[qco[j]];
        float *qdis = (float *)malloc(sizeof(float) * (L > 0 ? L : 1));
        int32_t *qid = (int32_t *)malloc(sizeof(int32_t) * (L > 0 ? L : 1));
        long pos = 0;
        for (int j = 0; j < w; j++) {
            int l = qco[j];
            if (l < 0) continue;
            const float *cen = ix->coa + (long)l * d;
            for (int i = 0; i < d; i++) r[i] = x[i] - cen[i]; /* bsxfunMINUS */
            build_table(ix, &pre, r, table_mode, tab);
            long beg = ix->list_off[l], n = ix->list_off[l + 1] - beg;
            adc_scan(ix, tab, beg, n, qdis + pos);
            memcpy(qid + pos, ix->ids + beg, sizeof(int32_t) * n);
            pos += n;
        }
        /* k_min of kk (:100-107): exact, ties by position */
        int ktmp = (int)(L < kk ? L : kk);
        int *sel = (int *)malloc(sizeof(int) * (ktmp > 0 ? ktmp : 1));
        orc_k_min(qdis, (int)L, ktmp, sel);
        if (adc_ids || adc_dis)
            for (int c = 0; c < kk; c++) {
                if (adc_ids) adc_ids[(long)q * kk + c] = c < ktmp ? qid[sel[c]] : -1;
                if (adc_dis) adc_dis[(long)q * kk + c] = c < ktmp ? qdis[sel[c]] : INFINITY;
            }
        if (rerank) {
            /* RERANK (:113-134): exact L2 of the ktmp candidates, k nearest */
            float *near = (float *)malloc(sizeof(float) * d * (ktmp > 0 ? ktmp : 1));
            int *lab = (int *)malloc(sizeof(int) * k);
            float *val = (float *)malloc(sizeof(float) * k);
            for (int b = 0; b < ktmp; b++)
                memcpy(near + (long)b * d, base + (long)qid[sel[b]] * d, sizeof(float) * d);
            int kr = k < ktmp ? k : ktmp;
            if (kr > 0) orc_knn_full(1, ktmp, d, kr, near, x, lab, val, ties);
            for (int c = 0; c < k; c++) {
                ids[(long)q * k + c] = c < kr ? qid[sel[lab[c]]] : -1;
                if (dis) dis[(long)q * k + c] = c < kr ? val[c] : INFINITY;
            }
            free(near);
            free(lab);
            free(val);
        } else {
            for (int c = 0; c < k; c++) {
                ids[(long)q * k + c] = c < ktmp ? qid[sel[c]] : -1;
                if (dis) dis[(long)q * k + c] = c < ktmp ? qdis[sel[c]] : INFINITY;
            }
        }
        free(sel);
        free(qdis);
        free(qid);
        free(cd);
        free(qco);
        free(qcd);
        free(r);
        free(tab);
    }
    pre_free(&pre);
    return err;
}

/* The uneven batch of the engine's gbivf_search_batched, restated per query
 * with the same steps as orc_ivfpq_search (no re-rank): query q probes its
 * w_per_q[q] nearest lists and keeps its k_per_q[q] best ADC candidates,
 * written at out_off[q] (ids -1 / distances +inf past L_q). */
int orc_ivfpq_search_batched(const orc_index *ix, const float *queries, int nq,
                             const int32_t *w_per_q, const int32_t *k_per_q,
                             const int64_t *out_off, int ties, int32_t *ids,
                             float *dis, int nthreads) {
    if (check_index(ix) || nq < 0) return -1;
    for (int q = 0; q < nq; q++)
        if (w_per_q[q] <= 0 || w_per_q[q] > ix->coarsek || k_per_q[q] <= 0) return -1;
    orc_pre pre;
    if (pre_init(ix, &pre)) return -2;
    const int d = ix->d, C = ix->coarsek;
    int err = 0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int q = 0; q < nq; q++) {
        const int w = w_per_q[q], k = k_per_q[q];
        const float *x = queries + (long)q * d;
        float *cd = (float *)malloc(sizeof(float) * C);
        int *qco = (int *)malloc(sizeof(int) * w);
        float *qcd = (float *)malloc(sizeof(float) * w);
        float *r = (float *)malloc(sizeof(float) * d);
        float *tab = (float *)malloc(sizeof(float) * ix->m * ix->ks);
        if (!cd || !qco || !qcd || !r || !tab) {
            err = -2;
            free(cd); free(qco); free(qcd); free(r); free(tab);
            continue;
        }
        double xn = norm_d(x, d);
        for (int c = 0; c < C; c++)
            cd[c] = expansion_dist(pre.coa_norm[c], xn, ix->coa + (long)c * d, x, d);
        select_k(cd, C, w, ties, qco, qcd);
        long L = 0;
        for (int j = 0; j < w; j++)
            if (qco[j] >= 0) L += ix->list_off[qco[j] + 1] - ix->list_off[qco[j]];
        float *qdis = (float *)malloc(sizeof(float) * (L > 0 ? L : 1));
        int32_t *qid = (int32_t *)malloc(sizeof(int32_t) * (L > 0 ? L : 1));
        long pos = 0;
        for (int j = 0; j < w; j++) {
            int l = qco[j];
            if (l < 0) continue;
            const float *cen = ix->coa + (long)l * d;
            for (int i = 0; i < d; i++) r[i] = x[i] - cen[i];
            build_table(ix, &pre, r, ORC_TABLE_EXPANSION, tab);
            long beg = ix->list_off[l], n = ix->list_off[l + 1] - beg;
            adc_scan(ix, tab, beg, n, qdis + pos);
            memcpy(qid + pos, ix->ids + beg, sizeof(int32_t) * n);
            pos += n;
        }
        int kt = (int)(L < k ? L : k);
        int *sel = (int *)malloc(sizeof(int) * (kt > 0 ? kt : 1));
        orc_k_min(qdis, (int)L, kt, sel);
        const long o = (long)out_off[q];
        for (int c = 0; c < k; c++) {
            ids[o + c] = c < kt ? qid[sel[c]] : -1;
            dis[o + c] = c < kt ? qdis[sel[c]] : INFINITY;
        }
        free(sel);
        free(qdis);
        free(qid);
        free(cd);
        free(qco);
        free(qcd);
        free(r);
        free(tab);
    }
    pre_free(&pre);
    return err;
}

int orc_pq_search(int d, int m, int ks, const float *pq, const uint8_t *codes,
                  int64_t n, const float *queries, int nq, int k, float *dis,
                  int32_t *ids, int nthreads) {
    if (d <= 0 || m <= 0 || d % m || ks <= 0 || ks > 256 || k <= 0 || k > n) return -1;
    orc_index ix;
    memset(&ix, 0, sizeof(ix));
    ix.d = d;
    ix.m = m;
    ix.ks = ks;
    ix.coarsek = 1;
    ix.pq = pq;
    ix.codes = codes;
    orc_pre pre;
    pre.coa_norm = NULL;
    pre.pq_norm = (double *)malloc(sizeof(double) * m * ks);
    int ds = d / m;
    for (int e = 0; e < m * ks; e++) pre.pq_norm[e] = norm_d(pq + (long)e * ds, ds);
    int err = 0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int q = 0; q < nq; q++) {
        float *tab = (float *)malloc(sizeof(float) * m * ks);
        float *all = (float *)malloc(sizeof(float) * n);
        int *sel = (int *)malloc(sizeof(int) * k);
        if (!tab || !all || !sel) {
            err = -2;
            free(tab); free(all); free(sel);
            continue;
        }
        /* tables from the query's own sub-vectors (pq_search.cpp:50-54) */
        build_table(&ix, &pre, queries + (long)q * d, ORC_TABLE_EXPANSION, tab);
        adc_scan(&ix, tab, 0, n, all); /* sumidxtab (:70-86) */
        orc_k_min(all, (int)n, k, sel);
        for (int l = 0; l < k; l++) { /* column-major, 1-based (:58-63) */
            dis[(long)nq * l + q] = all[sel[l]];
            ids[(long)nq * l + q] = sel[l] + 1;
        }
        free(tab);
        free(all);
        free(sel);
    }
    free(pre.pq_norm);
    return err;
}

int orc_core_cpu(const orc_index *ix, const float *residual, int nres,
                 const int32_t *rid_to_ivf, const int32_t *qid_to_starting_outid,
                 int32_t *idxs, float *dists, int k, int w, int nthreads) {
    if (check_index(ix) || w <= 0 || k <= 0 || nres % w) return -1;
    const int d = ix->d;
    int nq = nres / w, err = 0;
    orc_pre pre;
    pre.coa_norm = NULL;
    pre.pq_norm = NULL;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 2) num_threads(nthreads)
#endif
    for (int q = 0; q < nq; q++) {
        long L = 0;
        for (int j = 0; j < w; j++) {
            int l = rid_to_ivf[q * w + j];
            L += ix->list_off[l + 1] - ix->list_off[l];
        }
        float *tab = (float *)malloc(sizeof(float) * ix->m * ix->ks);
        float *qdis = (float *)malloc(sizeof(float) * (L > 0 ? L : 1));
        int32_t *qid = (int32_t *)malloc(sizeof(int32_t) * (L > 0 ? L : 1));
        int *sel = (int *)malloc(sizeof(int) * k);
        if (!tab || !qdis || !qid || !sel) {
            err = -2;
            free(tab); free(qdis); free(qid); free(sel);
            continue;
        }
        long pos = 0;
        for (int j = 0; j < w; j++) {
            int rid = q * w + j, l = rid_to_ivf[rid];
            build_table(ix, &pre, residual + (long)rid * d, ORC_TABLE_DIRECT, tab);
            long beg = ix->list_off[l], n = ix->list_off[l + 1] - beg;
            adc_scan(ix, tab, beg, n, qdis + pos);
            memcpy(qid + pos, ix->ids + beg, sizeof(int32_t) * n);
            pos += n;
        }
        int kt = (int)(L < k ? L : k);
        orc_k_min(qdis, (int)L, kt, sel);
        long out = qid_to_starting_outid[q];
        for (int c = 0; c < kt; c++) {
            dists[out + c] = qdis[sel[c]];
            idxs[out + c] = qid[sel[c]];
        }
        free(tab);
        free(qdis);
        free(qid);
        free(sel);
    }
    return err;
}
