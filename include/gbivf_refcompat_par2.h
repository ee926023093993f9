/*
 * gbivf reference-compatible C++ entry points, parallel2 GPU slot.
 *
 * libgbivf_refcompat_par2.so exports, with the reference's exact signatures
 * (parallel2/ivf_pq/mycuda.h:7-9), the three functions of its CUDA search
 * core, implemented on the gbivf C ABI, so that parallel2's search rank links
 * against this library instead of mycuda.o and selects it unchanged through
 * do_on's function pointer (parallel2/ivf_pq/ivf_search.cpp:120-159):
 *
 *   core_gpu            _Z8core_gpu6pqtipo3matP3ivfiPiS3_4matIS0_ii
 *   preallocate_gpu_mem _Z19preallocate_gpu_mem6pqtipoP3ivfi
 *   deallocate_gpu_mem  _Z18deallocate_gpu_memv
 *
 * parallel2's pqtipo differs from the sequential one: its centroids are one
 * flat nsq x ks x ds array (parallel2/pq-utils/pq_new.h:26-33). The other
 * structs restate parallel2/pq-utils/pq_test_load_vectors.h:19-27 and
 * parallel2/ivf_pq/myIVF.h:21-33 with the same tag names.
 *
 * As in the reference, one index per process is held by the library between
 * preallocate_gpu_mem and deallocate_gpu_mem; errors print and exit with
 * EXIT_FAILURE (mycuda.cu:11-14). core_gpu writes, per query, the
 * min(k, candidates) best (distance, id) ascending at qid_to_starting_outid.
 */
#ifndef GBIVF_REFCOMPAT_PAR2_H
#define GBIVF_REFCOMPAT_PAR2_H

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
    float *centroids; /* nsq x ks x ds */
    int centroidsn;
    int centroidsd;
} pqtipo;

typedef struct ivf {
    int *ids;
    int idstam;
    matI codes;
} ivf_t;

void core_gpu(pqtipo PQ, mat residual, ivf_t *ivf, int ivf_size, int *rid_to_ivf,
              int *qid_to_starting_outid, matI idxs, mat dists, int k, int w);
void preallocate_gpu_mem(pqtipo PQ, ivf_t *ivf, int ivf_size);
void deallocate_gpu_mem();

#endif
