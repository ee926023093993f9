// The reference's sequential search entry points on the gbivf C ABI
// (declared in include/gbivf_refcompat.h).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/gbivf.h"
#include "../../include/gbivf_refcompat.h"

namespace {

void die(const char* what) {
    fprintf(stderr, "gbivf: %s: %s\n", what, gbivf_last_error());
    exit(EXIT_FAILURE);
}

// one IVF index and one flat codebook per process, as the reference assumes
gbivf_index* g_ivf_ix = nullptr;
const ivf_t* g_ivf_key = nullptr;
const float* g_base_key = nullptr;
int g_base_n = -1;

gbivf_index* g_pq_ix = nullptr;
const int* g_pq_key = nullptr;
int g_pq_n = -1;

}  // namespace

void ivfpq_search(ivfpq_t ivfpq, ivf_t* ivf, mat vquery, mat vbase, int k, int kl, int w, int* ids, float* dis) {
    if (g_ivf_key != ivf || !g_ivf_ix) {
        if (g_ivf_ix) gbivf_index_destroy(g_ivf_ix);
        g_ivf_ix = nullptr;
        const int C = ivfpq.coarsek;
        std::vector<const int32_t*> lid(C), lcode(C);
        std::vector<int32_t> lsize(C);
        for (int l = 0; l < C; l++) {
            lid[l] = ivf[l].ids;
            lcode[l] = ivf[l].codes.mat;
            lsize[l] = ivf[l].idstam;
        }
        if (gbivf_index_create_from_lists(&g_ivf_ix, 0, ivfpq.coa_centroidsd, C, ivfpq.coa_centroids, ivfpq.pq.nsq,
                                          ivfpq.pq.ks, (const float* const*)ivfpq.pq.centroids, lsize.data(),
                                          lid.data(), lcode.data()))
            die("ivfpq_search: index upload");
        g_ivf_key = ivf;
        g_base_key = nullptr;
        g_base_n = -1;
    }
    if (g_base_key != vbase.mat || g_base_n != vbase.n) {
        if (gbivf_index_set_base(g_ivf_ix, vbase.mat, vbase.n, vbase.d)) die("ivfpq_search: base upload");
        g_base_key = vbase.mat;
        g_base_n = vbase.n;
    }
    std::vector<float> own;
    if (!dis) {
        own.resize((size_t)vquery.n * k);
        dis = own.data();
    }
    if (gbivf_ivfpq_search(g_ivf_ix, vquery.mat, vquery.n, k, kl, w, GBIVF_RERANK, ids, dis))
        die("ivfpq_search");
}

void pq_search(pqtipo pq, matI codebook, mat vquery, int k, float* dis, int* ids) {
    if (g_pq_key != codebook.mat || g_pq_n != codebook.n || !g_pq_ix) {
        if (g_pq_ix) gbivf_index_destroy(g_pq_ix);
        g_pq_ix = nullptr;
        const int ds = pq.ds;
        std::vector<float> flat((size_t)pq.nsq * pq.ks * ds);
        for (int s = 0; s < pq.nsq; s++)
            for (int e = 0; e < pq.ks * ds; e++) flat[(size_t)s * pq.ks * ds + e] = pq.centroids[s][e];
        std::vector<uint8_t> codes((size_t)codebook.n * pq.nsq);
        for (size_t i = 0; i < codes.size(); i++) {
            const int c = codebook.mat[i];
            if (c < 0 || c >= pq.ks || c > 255) {
                fprintf(stderr, "gbivf: pq_search: code %d outside 0..%d\n", c, pq.ks - 1);
                exit(EXIT_FAILURE);
            }
            codes[i] = (uint8_t)c;
        }
        if (gbivf_pq_create(&g_pq_ix, 0, pq.nsq * ds, pq.nsq, pq.ks, flat.data(), codes.data(), codebook.n))
            die("pq_search: codebook upload");
        g_pq_key = codebook.mat;
        g_pq_n = codebook.n;
    }
    if (gbivf_pq_search(g_pq_ix, vquery.mat, vquery.n, k, dis, ids)) die("pq_search");
}
