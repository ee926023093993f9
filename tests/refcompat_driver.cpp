// A caller of the reference's sequential ivfpq_search, linked against
// libgbivf_refcompat_seq.so instead of the reference's ivf_search.o.
//
// It drives the shim the way the reference's own driver does
// (sequential/ivf_test.cpp: build the index, keep the raw base for the
// re-rank, call ivfpq_search once per query batch), and it reproduces the
// trap of the reference's index builder: ivfpq_assign returns the same static
// ivf_t array on every call (sequential/ivf_pq/ivf_assign.cpp:19), so a second
// index arrives at the same address with new contents. Here one ivf_t array,
// one coarse-centroid buffer, one set of PQ centroid buffers and one base
// buffer are allocated once and refilled in place for each index.
//
//   refcompat_driver DIR k kl w
//
// DIR holds index_<t>.bin, queries.bin and base_<t>.bin for t in {A, B}
// (written by tests/test_refcompat_driver.py); the driver searches A, then B,
// then A again, and writes ids_<i>.bin / dis_<i>.bin for calls i = 0, 1, 2.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbivf_refcompat.h"

namespace {

std::vector<char> slurp(const std::string& path) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path.c_str());
        exit(2);
    }
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> b((size_t)n);
    if (n > 0 && fread(b.data(), 1, (size_t)n, f) != (size_t)n) exit(2);
    fclose(f);
    return b;
}

void spill(const std::string& path, const void* p, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f || fwrite(p, 1, bytes, f) != bytes) exit(3);
    fclose(f);
}

struct Reader {
    const char* p;
    template <class T>
    const T* take(size_t count) {
        const T* r = reinterpret_cast<const T*>(p);
        p += sizeof(T) * count;
        return r;
    }
};

// the caller's buffers, allocated on the first index and refilled in place afterwards
ivfpq_t g_ivfpq;
ivf_t* g_ivf = nullptr;
std::vector<float*> g_pq;
float* g_base = nullptr;

// index file: int32 C, d, nsq, ks; float coa[C*d]; float pq[nsq*ks*(d/nsq)]; int32 sizes[C];
// int32 ids[n]; int32 codes[n*nsq]
void load_index(const std::string& path) {
    std::vector<char> b = slurp(path);
    Reader r{b.data()};
    const int* hdr = r.take<int>(4);
    const int C = hdr[0], d = hdr[1], nsq = hdr[2], ks = hdr[3], ds = d / nsq;
    const float* coa = r.take<float>((size_t)C * d);
    const float* pq = r.take<float>((size_t)nsq * ks * ds);
    const int* sizes = r.take<int>(C);
    size_t n = 0;
    for (int l = 0; l < C; l++) n += sizes[l];
    const int* ids = r.take<int>(n);
    const int* codes = r.take<int>(n * nsq);
    if (!g_ivf) {
        g_ivf = static_cast<ivf_t*>(calloc(C, sizeof(ivf_t)));
        g_ivfpq.coa_centroids = static_cast<float*>(malloc(sizeof(float) * C * d));
        g_pq.resize(nsq);
        for (int s = 0; s < nsq; s++) g_pq[s] = static_cast<float*>(malloc(sizeof(float) * ks * ds));
        g_ivfpq.pq.centroids = g_pq.data();
    }
    g_ivfpq.coarsek = C;
    g_ivfpq.coa_centroidsn = C;
    g_ivfpq.coa_centroidsd = d;
    memcpy(g_ivfpq.coa_centroids, coa, sizeof(float) * C * d);
    g_ivfpq.pq.nsq = nsq;
    g_ivfpq.pq.ks = ks;
    g_ivfpq.pq.ds = ds;
    g_ivfpq.pq.centroidsn = ks * ds;
    g_ivfpq.pq.centroidsd = nsq;
    for (int s = 0; s < nsq; s++) memcpy(g_pq[s], pq + (size_t)s * ks * ds, sizeof(float) * ks * ds);
    size_t o = 0;
    for (int l = 0; l < C; l++) {
        ivf_t& v = g_ivf[l];
        const int m = sizes[l];
        // the list buffers grow when needed and are otherwise rewritten where they are
        if (m > v.idstam || !v.ids) {
            free(v.ids);
            free(v.codes.mat);
            v.ids = static_cast<int*>(malloc(sizeof(int) * (m > 0 ? m : 1)));
            v.codes.mat = static_cast<int*>(malloc(sizeof(int) * (size_t)(m > 0 ? m : 1) * nsq));
        }
        v.idstam = m;
        v.codes.n = m;
        v.codes.d = nsq;
        if (m > 0) {
            memcpy(v.ids, ids + o, sizeof(int) * m);
            memcpy(v.codes.mat, codes + o * nsq, sizeof(int) * (size_t)m * nsq);
        }
        o += m;
    }
}

// base / query file: int32 n, d; float x[n*d]
mat load_mat(const std::string& path, float* reuse) {
    std::vector<char> b = slurp(path);
    Reader r{b.data()};
    const int* hdr = r.take<int>(2);
    mat m;
    m.n = hdr[0];
    m.d = hdr[1];
    m.mat = reuse ? reuse : static_cast<float*>(malloc(sizeof(float) * (size_t)m.n * m.d));
    memcpy(m.mat, r.take<float>((size_t)m.n * m.d), sizeof(float) * (size_t)m.n * m.d);
    return m;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: %s DIR k kl w\n", argv[0]);
        return 1;
    }
    const std::string dir = argv[1];
    const int k = atoi(argv[2]), kl = atoi(argv[3]), w = atoi(argv[4]);
    mat vquery = load_mat(dir + "/queries.bin", nullptr);
    const char* order[3] = {"A", "B", "A"};
    std::vector<int> ids((size_t)vquery.n * k);
    std::vector<float> dis((size_t)vquery.n * k);
    for (int i = 0; i < 3; i++) {
        load_index(dir + "/index_" + order[i] + ".bin");
        mat vbase = load_mat(dir + "/base_" + order[i] + ".bin", g_base);
        g_base = vbase.mat;  // one base buffer, refilled in place
        ivfpq_search(g_ivfpq, g_ivf, vquery, vbase, k, kl, w, ids.data(), dis.data());
        spill(dir + "/ids_" + std::to_string(i) + ".bin", ids.data(), sizeof(int) * ids.size());
        spill(dir + "/dis_" + std::to_string(i) + ".bin", dis.data(), sizeof(float) * dis.size());
    }
    printf("refcompat_driver: 3 searches of %d queries\n", vquery.n);
    return 0;
}
