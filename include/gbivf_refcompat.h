/*
 * gbivf reference-compatible C++ entry points, sequential variant.
 *
 * libgbivf_refcompat_seq.so exports the reference's own C++ functions with
 * their exact signatures (same mangled names), implemented on the gbivf C
 * ABI, so that a program built against rafaelms101/mestrado's sequential
 * headers links against this library instead of ivf_pq/ivf_search.o and
 * pq-utils/pq_search.o:
 *
 *   ivfpq_search  sequential/ivf_pq/ivf_search.h:20 (_Z12ivfpq_search5ivfpqP3ivf3matS2_iiiPiPf)
 *   pq_search     sequential/pq-utils/pq_search.h:21 (_Z9pq_search6pqtipo4matI3matiPfPi)
 *
 * The structs below restate the layouts of the reference's types
 * (sequential/pq-utils/pq_test_load_vectors.h:16-26,
 * sequential/pq-utils/pq_new.h:26-33, sequential/ivf_pq/myIVF.h:15-27) with
 * the same tag names, which is what the mangled names encode. Include either
 * the reference's headers or this one, not both.
 *
 * Behaviour kept from the reference: ids are written as it writes them (row
 * major 0-based for ivfpq_search, column-major 1-based for pq_search); on an
 * error the process prints the message and exits with EXIT_FAILURE, as the
 * reference's GPU path does (parallel2/ivf_pq/mycuda.cu:11-14). Differences:
 * `dis` of ivfpq_search is written (the reference leaves it unset); ties in
 * distance may be ordered differently.
 */
#ifndef GBIVF_REFCOMPAT_H
#define GBIVF_REFCOMPAT_H

typedef struct {
    float *mat;
    int n, d;
} mat;

typedef struct {
    int *mat;
    int n, d;
} matI;

typedef struct pqtipo {
    int nsq;
    int ks;
    int ds;
    float **centroids; /* nsq arrays of ks x ds */
    int centroidsn;
    int centroidsd;
} pqtipo;

typedef struct ivfpq {
    pqtipo pq;
    int coarsek;
    float *coa_centroids;
    int coa_centroidsn;
    int coa_centroidsd;
} ivfpq_t;

typedef struct ivf {
    int *ids;
    int idstam;
    matI codes; /* idstam x nsq int32 codes */
} ivf_t;

/* ivfpq_search: w probes, ADC k-min of kl, exact re-rank of those kl against
 * vbase to k; ids nq x k. The index (ivfpq + ivf) and vbase stay on the GPU
 * between calls while their contents are unchanged: every call fingerprints
 * their bytes (one pass over them) and uploads again on any change, because
 * the reference's ivfpq_assign returns the same static ivf array each time
 * (sequential/ivf_pq/ivf_assign.cpp:19). */
void ivfpq_search(ivfpq_t ivfpq, ivf_t *ivf, mat vquery, mat vbase, int k, int kl, int w, int *ids,
                  float *dis);

/* pq_search: exhaustive ADC over the codebook; dis and ids k x nq
 * column-major, ids 1-based. The codes and centroids stay on the GPU between
 * calls while their contents (fingerprinted on every call) are unchanged. */
void pq_search(pqtipo pq, matI codebook, mat vquery, int k, float *dis, int *ids);

#endif
