/*
 * TEST INFRASTRUCTURE ONLY -- C entry points into the reference's own
 * sequential IVF-PQ code, compiled from the reference sources into
 * oracle/_ref/libref_seq.so by oracle/build.py. Used to pin the oracle and
 * to write the golden fixtures; never part of the product.
 *
 * Every function converts flat arrays into the reference's structs
 * (ivfpq_t, ivf_t, pqtipo, mat, matI from sequential/ivf_pq/myIVF.h and
 * sequential/pq-utils/pq_new.h) and calls the reference functions in the
 * order sequential/ivf_pq/ivf_search.cpp:9-153 calls them.
 */
#include <stdlib.h>
#include <string.h>

#include "ivf_pq/ivf_assign.h"
#include "ivf_pq/ivf_new.h"
#include "ivf_pq/ivf_search.h"

static mat mk_mat(const float *src, int n, int d) {
    mat m;
    m.n = n;
    m.d = d;
    m.mat = (float *)malloc(sizeof(float) * (size_t)n * d);
    memcpy(m.mat, src, sizeof(float) * (size_t)n * d);
    return m;
}

/* ivfpq_t + ivf_t[] from flat arrays; codes are int32 n x nsq */
static void mk_index(int d, int coarsek, int nsq, const float *coa, const float *pq,
                     const int *list_sizes, const int *ids, const int *codes,
                     ivfpq_t *ix, ivf_t **ivf_out) {
    int ds = d / nsq, ks = 256;
    ix->coarsek = ix->coa_centroidsn = coarsek;
    ix->coa_centroidsd = d;
    ix->coa_centroids = (float *)malloc(sizeof(float) * coarsek * d);
    memcpy(ix->coa_centroids, coa, sizeof(float) * coarsek * d);
    ix->pq.nsq = nsq;
    ix->pq.ks = ks;
    ix->pq.ds = ds;
    ix->pq.centroidsn = ks * ds;
    ix->pq.centroidsd = nsq;
    ix->pq.centroids = (float **)malloc(sizeof(float *) * nsq);
    for (int s = 0; s < nsq; s++) {
        ix->pq.centroids[s] = (float *)malloc(sizeof(float) * ks * ds);
        memcpy(ix->pq.centroids[s], pq + (size_t)s * ks * ds, sizeof(float) * ks * ds);
    }
    ivf_t *ivf = (ivf_t *)malloc(sizeof(ivf_t) * coarsek);
    long off = 0;
    for (int l = 0; l < coarsek; l++) {
        int n = list_sizes[l];
        ivf[l].idstam = n;
        ivf[l].ids = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
        memcpy(ivf[l].ids, ids + off, sizeof(int) * n);
        ivf[l].codes.n = n;
        ivf[l].codes.d = nsq;
        ivf[l].codes.mat = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1) * nsq);
        memcpy(ivf[l].codes.mat, codes + off * nsq, sizeof(int) * (size_t)n * nsq);
        off += n;
    }
    *ivf_out = ivf;
}

static void free_index(ivfpq_t *ix, ivf_t *ivf) {
    for (int l = 0; l < ix->coarsek; l++) {
        free(ivf[l].ids);
        free(ivf[l].codes.mat);
    }
    free(ivf);
    for (int s = 0; s < ix->pq.nsq; s++) free(ix->pq.centroids[s]);
    free(ix->pq.centroids);
    free(ix->coa_centroids);
}

extern "C" {

/* ivfpq_new + ivfpq_assign (sequential/ivf_test.cpp:52-59). Call once per
 * process: ivfpq_assign keeps its list array in a static (ivf_assign.cpp:19). */
int ref_build_index(const float *train, int ntrain, const float *base, int nbase, int d,
                    int coarsek, int nsq, float *coa_out, float *pq_out, int *list_sizes_out,
                    int *ids_out, int *codes_out) {
    mat vtrain = mk_mat(train, ntrain, d);
    ivfpq_t ix = ivfpq_new(coarsek, nsq, vtrain);
    mat vbase = mk_mat(base, nbase, d);
    ivf_t *ivf = ivfpq_assign(ix, vbase);
    memcpy(coa_out, ix.coa_centroids, sizeof(float) * coarsek * d);
    int ks = ix.pq.ks, ds = ix.pq.ds;
    for (int s = 0; s < nsq; s++)
        memcpy(pq_out + (size_t)s * ks * ds, ix.pq.centroids[s], sizeof(float) * ks * ds);
    long off = 0;
    for (int l = 0; l < coarsek; l++) {
        list_sizes_out[l] = ivf[l].idstam;
        memcpy(ids_out + off, ivf[l].ids, sizeof(int) * ivf[l].idstam);
        memcpy(codes_out + off * nsq, ivf[l].codes.mat, sizeof(int) * (size_t)ivf[l].idstam * nsq);
        off += ivf[l].idstam;
    }
    free(vtrain.mat);
    free(vbase.mat);
    return ks;
}

/* the reference ivfpq_search itself; ids is nq x k */
int ref_ivfpq_search(int d, int coarsek, int nsq, const float *coa, const float *pq,
                     const int *list_sizes, const int *ids, const int *codes,
                     const float *queries, int nq, const float *base, int nbase, int k, int kl,
                     int w, int *ids_out) {
    ivfpq_t ix;
    ivf_t *ivf;
    mk_index(d, coarsek, nsq, coa, pq, list_sizes, ids, codes, &ix, &ivf);
    mat vq = mk_mat(queries, nq, d);
    mat vb = mk_mat(base, nbase, d);
    float *dis = (float *)malloc(sizeof(float) * (size_t)nq * k);
    ivfpq_search(ix, ivf, vq, vb, k, kl, w, ids_out, dis);
    free(dis);
    free(vq.mat);
    free(vb.mat);
    free_index(&ix, ivf);
    return 0;
}

/* ivfpq_search up to the ADC k-min (ivf_search.cpp:37-107), using the
 * reference's knn_full, bsxfunMINUS, compute_cross_distances, sumidxtab2
 * and k_min. Outputs: coarse (nq x w) and the kl best ADC candidates
 * (base ids, distances; -1 / 0 padded when fewer exist). */
int ref_adc_stage(int d, int coarsek, int nsq, const float *coa, const float *pq,
                  const int *list_sizes, const int *ids, const int *codes, const float *queries,
                  int nq, int kl, int w, int *coaidx, float *coadis, int *adc_ids,
                  float *adc_dis) {
    ivfpq_t ix;
    ivf_t *ivf;
    mk_index(d, coarsek, nsq, coa, pq, list_sizes, ids, codes, &ix, &ivf);
    mat vq = mk_mat(queries, nq, d);
    int ks = ix.pq.ks, ds = ix.pq.ds;
    knn_full(2, nq, coarsek, d, w, ix.coa_centroids, vq.mat, NULL, coaidx, coadis);
    mat distab;
    distab.mat = (float *)malloc(sizeof(float) * ks * nsq);
    distab.n = nsq;
    distab.d = ks;
    float *tmp = (float *)malloc(sizeof(float) * ks);
    for (int q = 0; q < nq; q++) {
        int *qco = coaidx + (size_t)q * w;
        mat v = bsxfunMINUS(vq, ix.coa_centroids, d, q, qco, w);
        long L = 0;
        for (int j = 0; j < w; j++) L += ivf[qco[j]].codes.n;
        mat qdis;
        qdis.n = (int)L;
        qdis.d = 1;
        qdis.mat = (float *)malloc(sizeof(float) * (L > 0 ? L : 1));
        int *qidx = (int *)malloc(sizeof(int) * (L > 0 ? L : 1));
        long pos = 0;
        for (int j = 0; j < w; j++) {
            for (int s = 0; s < nsq; s++) {
                compute_cross_distances(ds, 1, ks, v.mat + j * v.d + s * ds, ix.pq.centroids[s], tmp);
                memcpy(distab.mat + s * ks, tmp, sizeof(float) * ks);
            }
            ivf_t *e = &ivf[qco[j]];
            float *part = sumidxtab2(distab, e->codes, 0);
            memcpy(qdis.mat + pos, part, sizeof(float) * e->codes.n);
            memcpy(qidx + pos, e->ids, sizeof(int) * e->idstam);
            pos += e->codes.n;
            free(part);
        }
        int ktmp = (int)(L < kl ? L : kl);
        float *dis1 = (float *)malloc(sizeof(float) * (ktmp > 0 ? ktmp : 1));
        int *ids1 = (int *)malloc(sizeof(int) * (ktmp > 0 ? ktmp : 1));
        /* k_min's branch needs n > 1 (pq_search.cpp:94-97) */
        if (ktmp > 0 && L > 1) k_min(qdis, ktmp, dis1, ids1);
        else if (ktmp == 1) {
            dis1[0] = qdis.mat[0];
            ids1[0] = 1;
        }
        for (int c = 0; c < kl; c++) {
            adc_ids[(size_t)q * kl + c] = c < ktmp ? qidx[ids1[c] - 1] : -1;
            adc_dis[(size_t)q * kl + c] = c < ktmp ? dis1[c] : 0.0f;
        }
        free(dis1);
        free(ids1);
        free(qdis.mat);
        free(qidx);
        free(v.mat);
    }
    free(tmp);
    free(distab.mat);
    free(vq.mat);
    free_index(&ix, ivf);
    return 0;
}

/* the reference pq_search (sequential/pq-utils/pq_search.cpp:10-68) */
int ref_pq_search(int d, int nsq, const float *pq, const int *codes, int n, const float *queries,
                  int nq, int k, float *dis, int *ids) {
    pqtipo p;
    int ks = 256, ds = d / nsq;
    p.nsq = nsq;
    p.ks = ks;
    p.ds = ds;
    p.centroidsn = ks * ds;
    p.centroidsd = nsq;
    p.centroids = (float **)malloc(sizeof(float *) * nsq);
    for (int s = 0; s < nsq; s++) p.centroids[s] = (float *)(pq + (size_t)s * ks * ds);
    matI cb;
    cb.n = n;
    cb.d = nsq;
    cb.mat = (int *)codes;
    mat vq = mk_mat(queries, nq, d);
    pq_search(p, cb, vq, k, dis, ids);
    free(vq.mat);
    free(p.centroids);
    return 0;
}

/* pq_new + pq_assign as sequential/pq_test.cpp:45-56 runs them (PQ on
 * raw vectors). pq_out is nsq x 256 x ds, codes_out nbase x nsq. */
int ref_build_pq(const float *train, int ntrain, const float *base, int nbase, int d, int nsq,
                 float *pq_out, int *codes_out) {
    mat vtrain = mk_mat(train, ntrain, d);
    pqtipo p = pq_new(nsq, vtrain, nsq);
    mat vbase = mk_mat(base, nbase, d);
    matI cb = pq_assign(p, vbase);
    for (int s = 0; s < nsq; s++)
        memcpy(pq_out + (size_t)s * p.ks * p.ds, p.centroids[s], sizeof(float) * p.ks * p.ds);
    memcpy(codes_out, cb.mat, sizeof(int) * (size_t)nbase * nsq);
    free(vtrain.mat);
    free(vbase.mat);
    return p.ks;
}

/* one expansion-form distance, the way knn_full's re-rank computes it:
 * a = base vector (float norm), b = query (double norm). */
float ref_l2(int d, const float *a, const float *b) {
    float out;
    compute_cross_distances(d, 1, 1, a, b, &out);
    return out;
}

} /* extern "C" */
