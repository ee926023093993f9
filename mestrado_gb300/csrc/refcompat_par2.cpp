// parallel2's CUDA search core on the gbivf C ABI (declared in
// include/gbivf_refcompat_par2.h).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/gbivf.h"
#include "../../include/gbivf_refcompat_par2.h"

namespace {

gbivf_index* g_ix = nullptr;  // the process's one index (mycuda.cu:21-22)

void die(const char* what) {
    fprintf(stderr, "gbivf: %s: %s\n", what, gbivf_last_error());
    exit(EXIT_FAILURE);
}

}  // namespace

void preallocate_gpu_mem(pqtipo PQ, ivf_t* ivf, int ivf_size) {
    if (g_ix) gbivf_index_destroy(g_ix);
    g_ix = nullptr;
    const int d = PQ.nsq * PQ.ds;
    std::vector<float> zero((size_t)ivf_size * d, 0.0f);  // core_gpu takes residuals, never centroids
    std::vector<const float*> pqs(PQ.nsq);
    for (int s = 0; s < PQ.nsq; s++) pqs[s] = PQ.centroids + (size_t)s * PQ.ks * PQ.ds;
    std::vector<const int32_t*> lid(ivf_size), lcode(ivf_size);
    std::vector<int32_t> lsize(ivf_size);
    for (int l = 0; l < ivf_size; l++) {
        lid[l] = ivf[l].ids;
        lcode[l] = ivf[l].codes.mat;
        lsize[l] = ivf[l].idstam;
    }
    if (gbivf_index_create_from_lists(&g_ix, 0, d, ivf_size, zero.data(), PQ.nsq, PQ.ks, pqs.data(), lsize.data(),
                                      lid.data(), lcode.data()))
        die("preallocate_gpu_mem");
}

void deallocate_gpu_mem() {
    if (g_ix) gbivf_index_destroy(g_ix);
    g_ix = nullptr;
}

void core_gpu(pqtipo PQ, mat residual, ivf_t* ivf, int ivf_size, int* rid_to_ivf, int* qid_to_starting_outid,
              matI idxs, mat dists, int k, int w) {
    (void)PQ;
    (void)ivf;
    (void)ivf_size;
    if (!g_ix) {
        fprintf(stderr, "gbivf: core_gpu before preallocate_gpu_mem\n");
        exit(EXIT_FAILURE);
    }
    if (gbivf_core_gpu(g_ix, residual.mat, residual.n, rid_to_ivf, qid_to_starting_outid, idxs.mat, dists.mat, k, w))
        die("core_gpu");
}
