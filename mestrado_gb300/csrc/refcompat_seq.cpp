// The reference's sequential search entry points on the gbivf C ABI
// (declared in include/gbivf_refcompat.h).
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/gbivf.h"
#include "../../include/gbivf_refcompat.h"

namespace {

void die(const char* what) {
    fprintf(stderr, "gbivf: %s: %s\n", what, gbivf_last_error());
    exit(EXIT_FAILURE);
}

// 64-bit content fingerprint of a byte range, folded into h: 8-byte words
// through four independent multiply-rotate lanes, the tail bytes last, the
// length mixed in. Not cryptographic; it tells one index or base from another.
struct Fingerprint {
    uint64_t lane[4] = {0x243f6a8885a308d3ull, 0x13198a2e03707344ull, 0xa4093822299f31d0ull,
                        0x082efa98ec4e6c89ull};
    uint64_t len = 0;
    static uint64_t mix(uint64_t h, uint64_t v) {
        h ^= v * 0x9e3779b97f4a7c15ull;
        h = (h << 29) | (h >> 35);
        return h * 0xbf58476d1ce4e5b9ull;
    }
    void add(const void* p, size_t bytes) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        size_t i = 0;
        for (; i + 32 <= bytes; i += 32) {
            uint64_t w[4];
            memcpy(w, b + i, 32);
            for (int j = 0; j < 4; j++) lane[j] = mix(lane[j], w[j]);
        }
        uint64_t t = 0;
        for (int j = 0; i < bytes; i++, j++) {
            t |= (uint64_t)b[i] << (8 * (j & 7));
            if ((j & 7) == 7 || i + 1 == bytes) {
                lane[0] = mix(lane[0], t);
                t = 0;
            }
        }
        len += bytes;
    }
    void add_int(int64_t v) { add(&v, sizeof v); }
    uint64_t value() const {
        uint64_t h = len;
        for (int j = 0; j < 4; j++) h = mix(h, lane[j]);
        return h ^ (h >> 31);
    }
};

// The uploaded index and base are identified by their CONTENT, re-read on every call: the
// reference's ivfpq_assign hands back the same static ivf_t array each time
// (sequential/ivf_pq/ivf_assign.cpp:19) and rewrites vectors in place, so a pointer says nothing
// about what it points to. One pass over the index's bytes (and the base's) per call is the price.
uint64_t index_fingerprint(const ivfpq_t& ivfpq, const ivf_t* ivf) {
    Fingerprint f;
    const int C = ivfpq.coarsek, d = ivfpq.coa_centroidsd, nsq = ivfpq.pq.nsq, ks = ivfpq.pq.ks, ds = ivfpq.pq.ds;
    f.add_int(C);
    f.add_int(d);
    f.add_int(nsq);
    f.add_int(ks);
    f.add_int(ds);
    f.add(ivfpq.coa_centroids, sizeof(float) * (size_t)C * d);
    for (int s = 0; s < nsq; s++) f.add(ivfpq.pq.centroids[s], sizeof(float) * (size_t)ks * ds);
    for (int l = 0; l < C; l++) {
        const int n = ivf[l].idstam;
        f.add_int(n);
        if (n > 0) {
            f.add(ivf[l].ids, sizeof(int) * (size_t)n);
            f.add(ivf[l].codes.mat, sizeof(int) * (size_t)n * nsq);
        }
    }
    return f.value();
}

uint64_t mat_fingerprint(const mat& m) {
    Fingerprint f;
    f.add_int(m.n);
    f.add_int(m.d);
    if (m.n > 0 && m.d > 0) f.add(m.mat, sizeof(float) * (size_t)m.n * m.d);
    return f.value();
}

uint64_t flat_fingerprint(const pqtipo& pq, const matI& codebook) {
    Fingerprint f;
    f.add_int(pq.nsq);
    f.add_int(pq.ks);
    f.add_int(pq.ds);
    for (int s = 0; s < pq.nsq; s++) f.add(pq.centroids[s], sizeof(float) * (size_t)pq.ks * pq.ds);
    f.add_int(codebook.n);
    f.add_int(codebook.d);
    f.add(codebook.mat, sizeof(int) * (size_t)codebook.n * pq.nsq);
    return f.value();
}

// one IVF index and one flat codebook per process, as the reference assumes
gbivf_index* g_ivf_ix = nullptr;
uint64_t g_ivf_fp = 0;
bool g_base_set = false;
uint64_t g_base_fp = 0;

gbivf_index* g_pq_ix = nullptr;
uint64_t g_pq_fp = 0;

}  // namespace

void ivfpq_search(ivfpq_t ivfpq, ivf_t* ivf, mat vquery, mat vbase, int k, int kl, int w, int* ids, float* dis) {
    const uint64_t ifp = index_fingerprint(ivfpq, ivf);
    if (!g_ivf_ix || ifp != g_ivf_fp) {
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
        g_ivf_fp = ifp;
        g_base_set = false;
    }
    const uint64_t bfp = mat_fingerprint(vbase);
    if (!g_base_set || bfp != g_base_fp) {
        if (gbivf_index_set_base(g_ivf_ix, vbase.mat, vbase.n, vbase.d)) die("ivfpq_search: base upload");
        g_base_fp = bfp;
        g_base_set = true;
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
    const uint64_t pfp = flat_fingerprint(pq, codebook);
    if (!g_pq_ix || pfp != g_pq_fp) {
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
        g_pq_fp = pfp;
    }
    if (gbivf_pq_search(g_pq_ix, vquery.mat, vquery.n, k, dis, ids)) die("pq_search");
}
