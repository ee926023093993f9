// C ABI of the GB300 IVF-PQ engine (declared in include/gbivf.h).
//
// Host side: validates arguments, lays the index out in HBM (list starts
// aligned to 16 bytes so that code rows load as 4/8/16-byte vectors),
// computes the index-constant norms once, keeps a per-index workspace that
// grows on demand, and enqueues the kernels of kernels.cu.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <limits>
#include <vector>

#include <cuda.h>

#include "../../include/gbivf.h"
#include "exact_round.cuh"
#include "kernels.cuh"

using namespace gbivf;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    g_err = b;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? GBIVF_ERR_NOMEM : GBIVF_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// growable device buffer
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes + bytes / 4;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

// reference-order norms on the host (nn.c:129-145)
float norm_f_host(const float* a, int d) {
    float s = 0.0f;
    for (int j = 0; j < d; j++) {
        float p = a[j] * a[j];
        s = s + p;
    }
    return s;
}

double norm_d_host(const float* a, int d) {
    double s = 0.0;
    for (int j = 0; j < d; j++) {
        float p = a[j] * a[j];
        s = s + (double)p;
    }
    return s;
}

}  // namespace

struct gbivf_index {
    int device = 0;
    DevIndex dx;
    std::vector<int32_t> h_len;  // list sizes (host copy)
    std::vector<int64_t> h_off, h_beg;  // list offsets in the caller's (unpadded) order, padded first rows
    DBuf pq2, codes2;            // refinement codebook and codes (gbivf_index_set_refine)
    int32_t min_id = 0, max_id = -1;  // range of stored base ids (re-rank bounds)
    int num_sms = 0;
    bool mixed_pending = false;       // a coarse stage with device flags ran since the last flag check
    int64_t last_ncand = 0;           // centroids re-checked exactly by the last checked coarse stage
    int64_t last_fallbacks = 0;       // queries of it that took all C centroids exactly
    float clen_max = 0.0f, cn_max = 0.0f;  // maxima of the centroid lengths / squared norms (mixed form)
    bool use_persistent = true;       // register-codebook scan where the shape allows
    bool auto_tuned = false;          // GBIVF_MIXED_SCAN_AUTO: measured by the autotuner ...
    bool auto_mixed = false;          // ... and the precision form was the faster
    int scan_threads = 512;           // block size of the persistent scan (512 or 1024)
    std::vector<void*> owned;    // index allocations
    DBuf base, base_norm;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    // workspace
    DBuf w_q, w_qn, w_coaidx, w_coadis, w_cdist, w_ids, w_dis, w_res, w_start, w_queue, w_ckey, w_cid, w_ccnt;
    // mixed-precision coarse stage: centroid BF16 tiles, centroid lengths, query tiles, flags
    DBuf coa_tiles, coa_len, coa_colG, coa_colK, w_qtiles, w_flags;
    // filtered coarse stage (large C): per-query bounds, counters, candidate slots, GEMM survivors
    DBuf w_thr, w_fcnt, w_cand, w_surv, w_scnt;
    // hand-off lists of the precision form and the refinement re-rank; the precision form's count of
    // queries whose result its finalize could not prove equal to the exact form's
    DBuf w_clist, w_unproven;
    DBuf w_rs;                        // the precision form's re-score workspace (RescoreWork)
    bool last_mixed = false;          // the last search used the precision form of the scan
    // list-centric scan (scan_lists.cu): one workspace block, its layout, stage events
    DBuf lc_ws;
    ListScanWork lcw;
    cudaEvent_t lc_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool last_list_scan = false;      // the last profiled search scanned list by list
    // without GBIVF_LIST_SCAN / GBIVF_QUERY_SCAN: 0 = the engine's rule (list by list for batches of at least
    // LIST_MIN_QUERIES on an index whose lists average at most LIST_MAX_MEAN_LEN codes), 1 = list by list for
    // large batches, 2 = query by query; list_pref: the autotuner's measured choice (-1: none)
    int list_mode = 0;
    int list_pref = -1;
    double mean_len = 0.0;
    int lc_ecap = 0;                  // per-query emission capacity of the list-centric scan (0: the default)
    int sel_mult = GBIVF_MIXED_SCAN_ALPHA;  // the precision form's approximate selection per result
    // stage events (GBIVF_PROFILE): start, coarse done, search done, scan kernel done
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_valid = false;
};

namespace {

// allocate `count` elements owned by the index and copy them from the host (h may be NULL: allocate only)
template <class T>
cudaError_t upload(gbivf_index* ix, const T* h, size_t count, T** out) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    ix->owned.push_back(p);
    if (count && h) e = cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice);
    *out = static_cast<T*>(p);
    return e;
}

void free_index(gbivf_index* ix) {
    for (void* p : ix->owned) cudaFree(p);
    ix->owned.clear();
    for (DBuf* b : {&ix->base, &ix->base_norm, &ix->w_q, &ix->w_qn, &ix->w_coaidx, &ix->w_coadis,
                    &ix->w_cdist, &ix->w_ids, &ix->w_dis, &ix->w_res, &ix->w_start, &ix->w_queue,
                    &ix->w_ckey, &ix->w_cid, &ix->w_ccnt, &ix->coa_tiles, &ix->coa_len, &ix->coa_colG, &ix->coa_colK, &ix->w_qtiles, &ix->w_flags,
                    &ix->w_thr, &ix->w_fcnt, &ix->w_cand, &ix->w_surv, &ix->w_scnt, &ix->w_clist,
                    &ix->w_unproven, &ix->w_rs, &ix->pq2, &ix->codes2, &ix->lc_ws})
        b->release();
    if (ix->stream) cudaStreamDestroy(ix->stream);
    ix->stream = nullptr;
    for (auto& e : ix->ev)
        if (e) cudaEventDestroy(e), e = nullptr;
    for (auto& e : ix->lc_ev)
        if (e) cudaEventDestroy(e), e = nullptr;
}

int create_impl(gbivf_index** out, int device, int d, int coarsek, const float* coa, int nsq, int ks,
                const float* pq, const int64_t* list_off, const int32_t* ids, const uint8_t* codes,
                bool dev_lists = false) {
    if (!out) return fail(GBIVF_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (d <= 0 || nsq <= 0 || d % nsq) return fail(GBIVF_ERR_INVALID, "d=%d must be a positive multiple of nsq=%d", d, nsq);
    if (ks <= 0 || ks > 256) return fail(GBIVF_ERR_UNSUPPORTED, "ks=%d: codes are bytes, so ks must be in 1..256", ks);
    if (coarsek <= 0) return fail(GBIVF_ERR_INVALID, "coarsek=%d", coarsek);
    if (nsq * ks > 64 * 256) return fail(GBIVF_ERR_UNSUPPORTED, "nsq*ks=%d exceeds the shared-memory table limit", nsq * ks);
    if (!coa || !pq || !list_off) return fail(GBIVF_ERR_INVALID, "NULL index array");
    if (list_off[0] != 0) return fail(GBIVF_ERR_INVALID, "list_off[0] must be 0");
    for (int l = 0; l < coarsek; l++)
        if (list_off[l + 1] < list_off[l]) return fail(GBIVF_ERR_INVALID, "list_off decreases at list %d", l);
    const int64_t n = list_off[coarsek];
    if (n > 0 && (!ids || !codes)) return fail(GBIVF_ERR_INVALID, "NULL ids/codes");
    if (dev_lists && ks != 256)
        return fail(GBIVF_ERR_UNSUPPORTED, "device-resident lists need ks = 256 (every byte is a valid code)");
    if (!dev_lists)
        for (int64_t i = 0; i < n * nsq; i++)
            if (codes[i] >= ks)
                return fail(GBIVF_ERR_INVALID, "code %d >= ks=%d at byte %lld", codes[i], ks, (long long)i);
    for (int l = 0; l < coarsek; l++)
        if (list_off[l + 1] - list_off[l] > 0x7fffffffLL) return fail(GBIVF_ERR_UNSUPPORTED, "list %d too long", l);
    if (n > 0xffffffffLL) return fail(GBIVF_ERR_UNSUPPORTED, "more than 2^32 vectors");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GBIVF_ERR_CUDA, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(GBIVF_ERR_INVALID, "device %d of %d", device, ndev);
    DeviceGuard g(device);
    if (!g.ok) return fail(GBIVF_ERR_CUDA, "cudaSetDevice(%d) failed", device);

    auto* ix = new gbivf_index();
    ix->device = device;
    if (!dev_lists) {
        for (int64_t i = 0; i < n; i++) {
            if (i == 0 || ids[i] < ix->min_id) ix->min_id = ids[i];
            if (i == 0 || ids[i] > ix->max_id) ix->max_id = ids[i];
        }
    } else if (n > 0) {
        int range[2];
        cudaError_t e = launch_id_range(ids, n, range, 0);
        if (e != cudaSuccess) {
            delete ix;
            return cuda_fail(e, "id range");
        }
        ix->min_id = range[0];
        ix->max_id = range[1];
    }
    const int ds = d / nsq;
    // list starts aligned so that a list's first code row sits on 16 bytes
    int g16 = std::gcd(nsq, 16);
    const int64_t align_rows = 16 / g16;
    std::vector<int64_t> beg(coarsek);
    ix->h_len.resize(coarsek);
    ix->h_off.assign(list_off, list_off + coarsek + 1);
    int64_t rows = 0;
    for (int l = 0; l < coarsek; l++) {
        rows = (rows + align_rows - 1) / align_rows * align_rows;
        beg[l] = rows;
        ix->h_len[l] = (int32_t)(list_off[l + 1] - list_off[l]);
        rows += ix->h_len[l];
    }
    rows = (rows + align_rows - 1) / align_rows * align_rows;
    ix->h_beg = beg;
    std::vector<uint8_t> pcodes;
    std::vector<int32_t> pids;
    if (!dev_lists) {
        pcodes.assign((size_t)std::max<int64_t>(rows, 1) * nsq, 0);
        pids.assign((size_t)std::max<int64_t>(rows, 1), -1);
        for (int l = 0; l < coarsek; l++) {
            int64_t len = ix->h_len[l];
            if (!len) continue;
            memcpy(&pcodes[(size_t)beg[l] * nsq], codes + list_off[l] * nsq, (size_t)len * nsq);
            memcpy(&pids[(size_t)beg[l]], ids + list_off[l], (size_t)len * sizeof(int32_t));
        }
    }
    std::vector<float> cn(coarsek);
    for (int c = 0; c < coarsek; c++) cn[c] = norm_f_host(coa + (int64_t)c * d, d);
    std::vector<double> pn((size_t)nsq * ks);
    std::vector<float> phi((size_t)nsq * ks), plo((size_t)nsq * ks);
    for (int e = 0; e < nsq * ks; e++) {
        pn[e] = norm_d_host(pq + (int64_t)e * ds, ds);
        split_norm(pn[e], &phi[e], &plo[e]);
    }
    // the precision form's error bound uses sum_s max_c ||c_s||^2 (rounded up)
    double cmax = 0.0;
    for (int sq = 0; sq < nsq; sq++) {
        double mx = 0.0;
        for (int c = 0; c < ks; c++) mx = std::max(mx, pn[(size_t)sq * ks + c]);
        cmax += mx;
    }
    if (cudaDeviceGetAttribute(&ix->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) ix->num_sms = 1;
    if (const char* v = getenv("GBIVF_SCAN_THREADS")) ix->scan_threads = atoi(v) == 1024 ? 1024 : 512;
    // a smaller emission buffer than the default sends more queries through the overflow pass
    if (const char* v = getenv("GBIVF_LIST_SCAN_CAP")) ix->lc_ecap = std::max(0, atoi(v));
    // rows of the first pass per selected candidate (its threshold tightens as it grows)
    if (const char* v = getenv("GBIVF_LIST_SCAN_BETA")) ix->lcw.beta = std::max(1, atoi(v));
    // the precision form's approximate selection, GBIVF_MIXED_SCAN_ALPHA * k by default
    if (const char* v = getenv("GBIVF_MIXED_SCAN_SEL")) ix->sel_mult = std::min(16, std::max(1, atoi(v)));
    if (const char* v = getenv("GBIVF_SCAN_KERNEL")) {
        ix->use_persistent = strcmp(v, "general") != 0;
        ix->list_mode = strcmp(v, "lists") == 0 ? 1 : 2;
    }
    ix->mean_len = coarsek ? (double)n / coarsek : 0.0;

    DevIndex& dx = ix->dx;
    dx.d = d;
    dx.C = coarsek;
    dx.m = nsq;
    dx.ks = ks;
    dx.ds = ds;
    dx.rows = rows;
    cudaError_t e = cudaSuccess;
    float *p_coa, *p_cn, *p_pq, *p_phi, *p_plo;
    double* p_pn;
    int64_t* p_beg;
    int32_t *p_len, *p_ids;
    uint8_t* p_codes;
    if ((e = upload(ix, coa, (size_t)coarsek * d, &p_coa)) != cudaSuccess ||
        (e = upload(ix, cn.data(), cn.size(), &p_cn)) != cudaSuccess ||
        (e = upload(ix, pq, (size_t)nsq * ks * ds, &p_pq)) != cudaSuccess ||
        (e = upload(ix, pn.data(), pn.size(), &p_pn)) != cudaSuccess ||
        (e = upload(ix, phi.data(), phi.size(), &p_phi)) != cudaSuccess ||
        (e = upload(ix, plo.data(), plo.size(), &p_plo)) != cudaSuccess ||
        (e = upload(ix, beg.data(), beg.size(), &p_beg)) != cudaSuccess ||
        (e = upload(ix, ix->h_len.data(), ix->h_len.size(), &p_len)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        free_index(ix);
        delete ix;
        return cuda_fail(e, "index upload");
    }
    if (!dev_lists) {
        e = upload(ix, pcodes.data(), pcodes.size(), &p_codes);
        if (e == cudaSuccess) e = upload(ix, pids.data(), pids.size(), &p_ids);
    } else {
        // device-resident lists: padded buffers, then one scatter per array (no host copy)
        const size_t nr = (size_t)std::max<int64_t>(rows, 1);
        int64_t *d_off = nullptr, *d_beg = nullptr;
        e = upload(ix, (const uint8_t*)nullptr, nr * nsq, &p_codes);
        if (e == cudaSuccess) e = upload(ix, (const int32_t*)nullptr, nr, &p_ids);
        if (e == cudaSuccess) e = upload(ix, list_off, (size_t)coarsek + 1, &d_off);
        if (e == cudaSuccess) e = upload(ix, beg.data(), beg.size(), &d_beg);
        if (e == cudaSuccess) e = cudaMemset(p_codes, 0, nr * nsq);
        if (e == cudaSuccess) e = cudaMemset(p_ids, 0xff, nr * sizeof(int32_t));
        if (e == cudaSuccess) e = launch_scatter_rows(codes, d_off, d_beg, coarsek, nsq, p_codes, 0);
        if (e == cudaSuccess)
            e = launch_scatter_rows(reinterpret_cast<const uint8_t*>(ids), d_off, d_beg, coarsek, 4,
                                    reinterpret_cast<uint8_t*>(p_ids), 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        free_index(ix);
        delete ix;
        return cuda_fail(e, "index upload");
    }
    dx.coa = p_coa;
    dx.coa_norm = p_cn;
    dx.pq = p_pq;
    dx.pq_norm = p_pn;
    dx.pq_hi = p_phi;
    dx.pq_lo = p_plo;
    dx.pq_cmax = (float)(cmax * (1.0 + 0x1p-20));
    dx.list_beg = p_beg;
    dx.list_len = p_len;
    dx.codes = p_codes;
    dx.ids = p_ids;
    *out = ix;
    return GBIVF_OK;
}

// queries per coarse-distance block: at most 64 Mi floats of scratch and
// 65535 row tiles of 64 queries (the kernel's grid.y)
int coarse_batch(int nq, int C) {
    int64_t bq = std::min<int64_t>(nq, (64ll << 20) / C);
    bq = std::min<int64_t>(bq, 65535ll * 64);
    return (int)std::max<int64_t>(1, bq);
}

// Workspace of the list-centric scan for this search shape, carved from one device block.
int prepare_list_scan(gbivf_index* ix, const ScanArgs& a) {
    const int64_t nq = a.nq, C = ix->dx.C, P = nq * a.w;
    ListScanWork& w = ix->lcw;
    w.ecap = ix->lc_ecap > 0 ? std::min(ix->lc_ecap, list_scan_ecap(a)) : list_scan_ecap(a);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t r = off;
        off += (bytes + 255) / 256 * 256;
        return r;
    };
    const size_t o_w0 = take(4 * nq), o_pcnt = take(4 * C), o_pbeg = take(4 * (C + 1)), o_fill = take(4 * C),
                 o_gbeg = take(4 * (C + 1)), o_bsum = take(8 * ((C + 4095) / 4096)), o_pairs = take(16 * P), o_groups = take(16 * 9 * P), o_cnt = take(4 * 8),
                 o_keys = take(8 * nq * a.cand_stride), o_cntA = take(4 * nq), o_tau = take(8 * nq),
                 o_tau0 = take(8 * nq), o_hist = take(4 * nq * (int64_t)LC_HIST_BUCKETS),
                 o_ebuf = take(8 * nq * (int64_t)w.ecap), o_ecnt = take(4 * nq), o_ovf = take(4 * nq);
    CK(ix->lc_ws.ensure(off));
    unsigned char* b = ix->lc_ws.as<unsigned char>();
    w.w0 = reinterpret_cast<int*>(b + o_w0);
    w.pcnt = reinterpret_cast<int*>(b + o_pcnt);
    w.pbeg = reinterpret_cast<int*>(b + o_pbeg);
    w.fill = reinterpret_cast<int*>(b + o_fill);
    w.gbeg = reinterpret_cast<int*>(b + o_gbeg);
    w.bsum = reinterpret_cast<int*>(b + o_bsum);
    w.pairs = reinterpret_cast<int4*>(b + o_pairs);
    w.groups = reinterpret_cast<int4*>(b + o_groups);
    w.counters = reinterpret_cast<int*>(b + o_cnt);  // [0..2] groups, work counter, overflows; [3], [4] queues
    w.queue_a = w.counters + 3;
    w.queue_b = w.counters + 4;
    w.keysA = reinterpret_cast<unsigned long long*>(b + o_keys);
    w.cntA = reinterpret_cast<int*>(b + o_cntA);
    w.tau = reinterpret_cast<unsigned long long*>(b + o_tau);
    w.tau0 = reinterpret_cast<unsigned long long*>(b + o_tau0);
    w.hist = reinterpret_cast<unsigned int*>(b + o_hist);
    w.ebuf = reinterpret_cast<unsigned long long*>(b + o_ebuf);
    w.ecnt = reinterpret_cast<int*>(b + o_ecnt);
    w.ovf = reinterpret_cast<int32_t*>(b + o_ovf);
    CK(ix->w_flags.ensure(4 * sizeof(int)));
    w.err = ix->w_flags.as<int>();
    return GBIVF_OK;
}

// whether this search scans list by list (GBIVF_LIST_SCAN, or the engine's choice for large batches)
// The engine's default scan order. Measured on one GB300: list by list wins where lists are short
// against the per-query scan's per-probe cost (100M / 262,144 lists, ~380 codes: 26.6 vs 39.3 ms;
// 10M / 65,536 lists, ~150 codes: 3.8 vs 4.4 ms) and loses on long lists that the per-query kernel
// already amortises (1M / 1,024 lists, ~980 codes: 3.7 vs 2.9 ms).
constexpr int LIST_MIN_QUERIES = 1024;
constexpr double LIST_MAX_MEAN_LEN = 768.0;

bool use_list_scan(const gbivf_index* ix, const ScanArgs& a, unsigned gflags) {
    if (gflags & GBIVF_QUERY_SCAN) return false;
    bool want = gflags & GBIVF_LIST_SCAN;
    if (!want && a.nq >= LIST_MIN_QUERIES) {
        if (ix->list_mode == 1) want = true;
        else if (ix->list_mode == 0)
            want = ix->list_pref >= 0 ? ix->list_pref == 1 : ix->mean_len <= LIST_MAX_MEAN_LEN;
    }
    return want && list_scan_supported(ix->dx, a);
}

// the list-centric pipeline, the persistent register-codebook kernel where it applies, else the
// general one
int run_scan(gbivf_index* ix, ScanArgs& a, cudaStream_t st, cudaEvent_t mid = nullptr, unsigned gflags = 0) {
    CK(ix->w_queue.ensure(sizeof(int)));
    a.queue = ix->w_queue.as<int>();
    const bool mixed = a.flags & SCAN_MIXED;
    ix->last_mixed = mixed;
    if (mixed) {
        a.sel_mult = ix->sel_mult;
        a.sel_extra = GBIVF_MIXED_SCAN_EXTRA;
        a.sel_cap = 4096;
        if (!scan_persistent_supported(ix->dx, a))
            return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_MIXED_SCAN needs d = 128, ks = 256, m in {4, 8, 16} and "
                                               "k (or kl) <= 1024");
    }
    const bool refine = a.flags & SCAN_REFINE;
    if (refine && !scan_persistent_supported(ix->dx, a))
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_RERANK_REFINE needs d = 128, ks = 256, m in {4, 8, 16}");
    const bool lists = use_list_scan(ix, a, gflags);
    if (!lists && (gflags & GBIVF_LIST_SCAN))
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_LIST_SCAN needs d = 128, ks = 256, m in {4, 8, 16}, k (or kl) "
                                           "<= 1024 and the expansion tables");
    ix->last_list_scan = lists;
    if (lists || mixed || refine || (ix->use_persistent && scan_persistent_supported(ix->dx, a))) {
        const int stride = scan_persistent_stride(a);
        CK(ix->w_ckey.ensure(sizeof(unsigned long long) * (size_t)a.nq * stride));
        CK(ix->w_cid.ensure(sizeof(int32_t) * (size_t)a.nq * stride));
        CK(ix->w_ccnt.ensure(sizeof(int32_t) * (size_t)a.nq));
        a.cand_key = ix->w_ckey.as<unsigned long long>();
        a.cand_id = ix->w_cid.as<int32_t>();
        a.cand_cnt = ix->w_ccnt.as<int32_t>();
        a.cand_stride = stride;
        if (mixed || refine) {
            CK(ix->w_clist.ensure(sizeof(int32_t) * (size_t)a.nq * stride));
            a.cand_list = ix->w_clist.as<int32_t>();
        }
        if (mixed) {
            CK(ix->w_unproven.ensure(sizeof(int)));
            CK(cudaMemsetAsync(ix->w_unproven.p, 0, sizeof(int), st));
            a.unproven = ix->w_unproven.as<int>();
            // the re-score's workspace, one block: list, marks, counts, bounds, the two chunk queues
            const size_t nq = (size_t)a.nq, sd = (size_t)stride;
            const int qcap = rescore_queue_cap(a.nq, stride);
            auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
            const size_t o_list = 0, o_marks = o_list + up(4 * nq * sd), o_cnt = o_marks + up(nq * sd / 8),
                         o_t0 = o_cnt + up(8 * nq), o_amax = o_t0 + up(8 * nq), o_r2 = o_amax + up(8 * nq),
                         o_queue = o_r2 + up(4 * nq), o_qcount = o_queue + up(2 * 16 * (size_t)qcap),
                         total = o_qcount + 256;
            CK(ix->w_rs.ensure(total));
            unsigned char* b = static_cast<unsigned char*>(ix->w_rs.p);
            a.rw.list = reinterpret_cast<int32_t*>(b + o_list);
            a.rw.marks = reinterpret_cast<unsigned*>(b + o_marks);
            a.rw.cnt = reinterpret_cast<int*>(b + o_cnt);
            a.rw.t0 = reinterpret_cast<unsigned long long*>(b + o_t0);
            a.rw.amax = reinterpret_cast<unsigned long long*>(b + o_amax);
            a.rw.r2 = reinterpret_cast<float*>(b + o_r2);
            a.rw.queue = reinterpret_cast<int4*>(b + o_queue);
            a.rw.qcount = reinterpret_cast<int*>(b + o_qcount);
            a.rw.qcap = qcap;
        }
        if (lists) {
            if (!(a.flags & (SCAN_MIXED | SCAN_REFINE))) {  // the select kernel writes lists only for those
                a.cand_list = nullptr;
            } else if (!a.cand_list) {
                return fail(GBIVF_ERR_INVALID, "hand-off lists missing");
            }
            int rc = prepare_list_scan(ix, a);
            if (rc) return rc;
            const bool prof = mid != nullptr;
            if (prof)
                for (auto& e : ix->lc_ev)
                    if (!e) CK(cudaEventCreate(&e));
            CK(launch_list_scan(ix->dx, a, ix->lcw, ix->num_sms, st, prof ? ix->lc_ev : nullptr));
            ix->mixed_pending = true;  // the scan's bounded waits report through the device flags
            if (mid) CK(cudaEventRecord(mid, st));
            CK(launch_finalize(ix->dx, a, st));
        } else {
            CK(launch_scan_persistent(ix->dx, a, ix->num_sms, ix->scan_threads, st, mid));
        }
    } else {
        CK(launch_scan(ix->dx, a, st));
        if (mid) CK(cudaEventRecord(mid, st));  // one kernel: no separate finalize
    }
    return GBIVF_OK;
}

int check_search(gbivf_index* ix, int nq, int k, int kl, int w, unsigned flags) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (nq < 0) return fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    if (k <= 0 || k > MAX_K) return fail(k <= 0 ? GBIVF_ERR_INVALID : GBIVF_ERR_UNSUPPORTED, "k=%d (1..%d)", k, MAX_K);
    if (w <= 0 || w > ix->dx.C) return fail(GBIVF_ERR_INVALID, "w=%d must be in 1..coarsek=%d", w, ix->dx.C);
    if (w > MAX_W) return fail(GBIVF_ERR_UNSUPPORTED, "w=%d > %d", w, MAX_W);
    if (flags & ~(GBIVF_RERANK | GBIVF_TABLE_DIRECT | GBIVF_PROFILE | GBIVF_MIXED_COARSE | GBIVF_COARSE_FULL |
                  GBIVF_MIXED_SCAN | GBIVF_RERANK_REFINE | GBIVF_MIXED_SCAN_AUTO | GBIVF_LIST_SCAN | GBIVF_QUERY_SCAN))
        return fail(GBIVF_ERR_INVALID, "unknown flags 0x%x", flags);
    if ((flags & GBIVF_LIST_SCAN) && (flags & GBIVF_QUERY_SCAN))
        return fail(GBIVF_ERR_INVALID, "GBIVF_LIST_SCAN and GBIVF_QUERY_SCAN exclude each other");
    if ((flags & GBIVF_LIST_SCAN) && (flags & GBIVF_TABLE_DIRECT))
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_LIST_SCAN uses the expansion tables (not GBIVF_TABLE_DIRECT)");
    if ((flags & GBIVF_MIXED_SCAN) && (flags & GBIVF_MIXED_SCAN_AUTO))
        return fail(GBIVF_ERR_INVALID, "GBIVF_MIXED_SCAN_AUTO chooses the scan form: not with GBIVF_MIXED_SCAN");
    if ((flags & GBIVF_MIXED_SCAN) && (flags & GBIVF_TABLE_DIRECT))
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_MIXED_SCAN uses the expansion tables (not GBIVF_TABLE_DIRECT)");
    if (flags & GBIVF_RERANK_REFINE) {
        if (flags & (GBIVF_RERANK | GBIVF_TABLE_DIRECT))
            return fail(GBIVF_ERR_INVALID, "GBIVF_RERANK_REFINE excludes GBIVF_RERANK and GBIVF_TABLE_DIRECT");
        if (!ix->dx.codes2) return fail(GBIVF_ERR_INVALID, "GBIVF_RERANK_REFINE needs gbivf_index_set_refine first");
        if (kl <= 0 || kl > 1024 || kl < k)
            return fail(GBIVF_ERR_UNSUPPORTED, "kl=%d: the refinement re-rank takes k <= kl <= 1024", kl);
    }
    if ((flags & GBIVF_MIXED_COARSE) && ix->dx.d != 128)
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_MIXED_COARSE needs d = 128 (d = %d)", ix->dx.d);
    if (flags & GBIVF_RERANK) {
        if (kl <= 0 || kl > MAX_K) return fail(kl <= 0 ? GBIVF_ERR_INVALID : GBIVF_ERR_UNSUPPORTED, "kl=%d (1..%d)", kl, MAX_K);
        if (!ix->base.p) return fail(GBIVF_ERR_INVALID, "GBIVF_RERANK needs gbivf_index_set_base first");
        if (ix->max_id >= 0 && (ix->min_id < 0 || (int64_t)ix->max_id >= ix->dx.nbase))
            return fail(GBIVF_ERR_INVALID, "stored ids %d..%d fall outside the %lld base rows", ix->min_id, ix->max_id,
                        (long long)ix->dx.nbase);
    }
    return GBIVF_OK;
}

// BF16 centroid tiles and centroid lengths of the mixed form, built once
int prepare_mixed(gbivf_index* ix, cudaStream_t st) {
    if (ix->coa_tiles.p) return GBIVF_OK;
    const DevIndex& dx = ix->dx;
    CK(ix->coa_tiles.ensure(coarse_mma_tile_bytes(dx.C, true)));
    CK(launch_bf16_split_tiles(dx.coa, dx.C, ix->coa_tiles.as<uint8_t>(), st));
    std::vector<float> len(dx.C);
    std::vector<float> cn(dx.C);
    CK(cudaMemcpyAsync(cn.data(), dx.coa_norm, sizeof(float) * dx.C, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // per-centroid columns of the persistent GEMM's pre-test and sample (coarse_gemm.cu)
    const size_t ng = coarse_gemm_col_floats(dx.C);
    std::vector<float> colG(ng, std::numeric_limits<float>::infinity()), colK(ng, 0.0f);
    ix->clen_max = 0.0f;
    ix->cn_max = 0.0f;
    for (int c = 0; c < dx.C; c++) {
        len[c] = std::sqrt(cn[c]) * 1.0000002f;
        colG[c] = cn[c] * (1.0f - 9.5367431640625e-07f) * 0.5f;
        colK[c] = MIXED_EPS_REL * len[c] * 0.5f;
        ix->clen_max = std::max(ix->clen_max, len[c]);
        ix->cn_max = std::max(ix->cn_max, cn[c]);
    }
    CK(ix->coa_len.ensure(sizeof(float) * dx.C));
    CK(cudaMemcpyAsync(ix->coa_len.p, len.data(), sizeof(float) * dx.C, cudaMemcpyHostToDevice, st));
    CK(ix->coa_colG.ensure(sizeof(float) * ng));
    CK(cudaMemcpyAsync(ix->coa_colG.p, colG.data(), sizeof(float) * ng, cudaMemcpyHostToDevice, st));
    CK(ix->coa_colK.ensure(sizeof(float) * ng));
    CK(cudaMemcpyAsync(ix->coa_colK.p, colK.data(), sizeof(float) * ng, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return GBIVF_OK;
}

// BF16 query tiles for the persistent GEMM: whole 256-row pairs, the unused
// half of a last odd pair zeroed
int make_query_tiles(gbivf_index* ix, const float* qb, int nb, cudaStream_t st) {
    uint8_t* qt = ix->w_qtiles.as<uint8_t>();
    CK(launch_bf16_tiles(qb, nb, MMA_QUERY_TILE, qt, st));
    const size_t written = coarse_mma_tile_bytes(nb, false), total = coarse_gemm_qtile_bytes(nb);
    if (total > written) CK(cudaMemsetAsync(qt + written, 0, total - written, st));
    return GBIVF_OK;
}

// Filtered coarse stage (coarse_filter.cu) for large C, plain or mixed form.
int coarse_stage_filtered(gbivf_index* ix, const float* d_q, const double* qn, int nq, int w, bool mixed, int S,
                          int r, int cap, int32_t* coaidx, float* coadis, int* fl, cudaStream_t st,
                          const int32_t* d_w) {
    const DevIndex& dx = ix->dx;
    // queries per block: the sample block (bq x S floats) within 256 Mi floats
    int64_t bq = std::min<int64_t>(nq, std::max<int64_t>(MMA_QUERY_TILE, (256ll << 20) / S));
    bq = std::min<int64_t>(bq, 65535ll * 64);
    if (bq >= MMA_QUERY_TILE) bq = bq / MMA_QUERY_TILE * MMA_QUERY_TILE;
    CK(ix->w_cdist.ensure(sizeof(float) * (size_t)bq * S));
    CK(ix->w_thr.ensure(sizeof(float) * (size_t)bq));
    CK(ix->w_fcnt.ensure(2 * sizeof(int) * (size_t)bq));
    CK(ix->w_cand.ensure(sizeof(int32_t) * (size_t)bq * cap));
    if (mixed) CK(ix->w_qtiles.ensure(coarse_gemm_qtile_bytes((int)bq)));
    // mixed form: survivor regions of the GEMM, sized for about 4x the expected survivors
    // (3w + 64 candidates spread evenly over the centroid ranges) and for the largest block
    auto surv_shape = [&](int nb, int* nsplit, int* sreg) {
        int st_tiles = 1;
        *nsplit = coarse_gemm_nsplit(nb, dx.C, ix->num_sms, &st_tiles);
        const double expect = (3.0 * w + 64.0) * (st_tiles * 128.0 / dx.C) / 2.0;
        *sreg = std::min(4096, std::max(32, ((int)std::ceil(4.0 * expect) + 15) / 16 * 16));
    };
    if (mixed) {
        size_t need_s = 0, need_c = 0;
        for (int64_t nb : {bq, (int64_t)(nq % bq)}) {
            if (nb <= 0) continue;
            int ns, sr;
            surv_shape((int)nb, &ns, &sr);
            need_s = std::max(need_s, sizeof(int2) * (size_t)nb * 2 * ns * sr);
            need_c = std::max(need_c, sizeof(int) * (size_t)nb * 2 * ns);
        }
        CK(ix->w_surv.ensure(need_s));
        CK(ix->w_scnt.ensure(need_c));
    }
    float* cd = ix->w_cdist.as<float>();
    float* thr = ix->w_thr.as<float>();
    int* cnt = ix->w_fcnt.as<int>();
    CoarseFilter f;
    f.thr = thr;
    f.cnt = mixed ? cnt : nullptr;
    f.ncand = cnt + bq;
    f.cand = ix->w_cand.as<int32_t>();
    f.cap = cap;
    f.clen = mixed ? ix->coa_len.as<float>() : nullptr;
    DevIndex sx = dx;  // the sample: the first S centroids
    sx.C = S;
    for (int64_t q0 = 0; q0 < nq; q0 += bq) {
        const int nb = (int)std::min<int64_t>(bq, nq - q0);
        const float* qb = d_q + q0 * dx.d;
        CK(cudaMemsetAsync(cnt, 0, 2 * sizeof(int) * (size_t)bq, st));
        // an uneven batch: each query's bound, candidates and selection for its own probe count
        SampleRank sr;
        sr.w_per_q = d_w ? d_w + q0 : nullptr;
        sr.w = w;
        sr.scale = 2.0 * S / (double)dx.C;
        f.w_per_q = sr.w_per_q;
        if (mixed) {
            uint8_t* qt = ix->w_qtiles.as<uint8_t>();
            int rc = make_query_tiles(ix, qb, nb, st);
            if (rc) return rc;
            const float* colG = ix->coa_colG.as<float>();
            const float* colK = ix->coa_colK.as<float>();
            if (r <= 128 && r <= S / 32) {
                // sample: minima of 32-centroid chunks straight from the GEMM, bound from those
                CK(launch_coarse_gemm_chunkmin(qt, ix->coa_tiles.as<uint8_t>(), nb, S, qn + q0, dx.coa_norm, colG,
                                               colK, cd, S / 32, ix->num_sms, fl, st));
                CK(launch_coarse_sample_bound(cd, nb, S / 32, S / 32, r, thr, st, sr));
            } else {
                CK(launch_coarse_gemm_store(qt, ix->coa_tiles.as<uint8_t>(), nb, S, qn + q0, dx.coa_norm, cd, S,
                                            ix->num_sms, fl, st));
                CK(launch_coarse_sample_kth(cd, nb, S, r, qn + q0, dx.coa_norm, ix->coa_len.as<float>(), thr, st, sr));
            }
            surv_shape(nb, &f.nsplit, &f.sreg);
            f.surv = ix->w_surv.as<int2>();
            f.scnt = ix->w_scnt.as<int>();
            CK(launch_coarse_gemm_filter(qt, ix->coa_tiles.as<uint8_t>(), nb, dx.C, qn + q0, dx.coa_norm, f, colG,
                                         colK, ix->cn_max, ix->clen_max, ix->num_sms, fl, st));
        } else {
            CK(launch_coarse_dist(sx, qb, qn + q0, nb, cd, st));
            if (r <= 128)
                CK(launch_coarse_sample_bound(cd, nb, S, S, r, thr, st, sr));
            else
                CK(launch_coarse_sample_kth(cd, nb, S, r, qn + q0, nullptr, nullptr, thr, st, sr));
            CK(launch_coarse_dist_filter(dx, qb, qn + q0, nb, f, st));
        }
        CK(launch_coarse_cand_select(dx, qb, qn + q0, nb, w, f, coaidx + q0 * w, coadis + q0 * w, fl + 1, st));
    }
    return GBIVF_OK;
}

// Coarse stage: coaidx/coadis (nq x w) for device queries d_q with norms qn; with d_w (an uneven
// batch) the large-C filtered stage selects only each query's first d_w[q] entries (the rest of the
// row is -1), the prefix of its top-w.
// The flags word w_flags holds [0] the device error flag, [1] the number of
// centroids re-checked exactly, [2] the queries that took all C centroids.
int coarse_stage(gbivf_index* ix, const float* d_q, const double* qn, int nq, int w, unsigned flags, int32_t* coaidx,
                 float* coadis, cudaStream_t st, const int32_t* d_w = nullptr) {
    const DevIndex& dx = ix->dx;
    if (dx.C == 1) {
        CK(cudaMemsetAsync(coaidx, 0, sizeof(int32_t) * nq, st));
        return GBIVF_OK;
    }
    const bool mixed = flags & GBIVF_MIXED_COARSE;
    int S = 0, r = 0, cap = 0;
    if (coarse_filter_shape(dx.C, w, dx.d, &S, &r, &cap) && !(flags & GBIVF_COARSE_FULL)) {
        if (mixed) {
            int rc = prepare_mixed(ix, st);
            if (rc) return rc;
        }
        CK(ix->w_flags.ensure(4 * sizeof(int)));
        CK(cudaMemsetAsync(ix->w_flags.p, 0, 4 * sizeof(int), st));
        int rc = coarse_stage_filtered(ix, d_q, qn, nq, w, mixed, S, r, cap, coaidx, coadis, ix->w_flags.as<int>(),
                                       st, d_w);
        if (rc) return rc;
        ix->mixed_pending = true;
        return GBIVF_OK;
    }
    if (!mixed) {
        int bq = coarse_batch(nq, dx.C);
        CK(ix->w_cdist.ensure(sizeof(float) * (size_t)bq * dx.C));
        float* cd = ix->w_cdist.as<float>();
        for (int q0 = 0; q0 < nq; q0 += bq) {
            int nb = std::min(bq, nq - q0);
            CK(launch_coarse_dist(dx, d_q + (int64_t)q0 * dx.d, qn + q0, nb, cd, st));
            CK(launch_coarse_select(cd, nb, dx.C, w, coaidx + (int64_t)q0 * w, coadis + (int64_t)q0 * w, st));
        }
        return GBIVF_OK;
    }
    {
        int rc = prepare_mixed(ix, st);
        if (rc) return rc;
    }
    int bq = coarse_batch(nq, dx.C);
    if (bq >= MMA_QUERY_TILE) bq = bq / MMA_QUERY_TILE * MMA_QUERY_TILE;
    CK(ix->w_cdist.ensure(sizeof(float) * (size_t)bq * dx.C));
    CK(ix->w_qtiles.ensure(coarse_gemm_qtile_bytes(bq)));
    CK(ix->w_flags.ensure(4 * sizeof(int)));
    CK(cudaMemsetAsync(ix->w_flags.p, 0, 4 * sizeof(int), st));
    int* fl = ix->w_flags.as<int>();
    for (int q0 = 0; q0 < nq; q0 += bq) {
        int nb = std::min(bq, nq - q0);
        const float* qb = d_q + (int64_t)q0 * dx.d;
        int rc = make_query_tiles(ix, qb, nb, st);
        if (rc) return rc;
        CK(launch_coarse_gemm_store(ix->w_qtiles.as<uint8_t>(), ix->coa_tiles.as<uint8_t>(), nb, dx.C, qn + q0,
                                    dx.coa_norm, ix->w_cdist.as<float>(), dx.C, ix->num_sms, fl, st));
        CK(launch_coarse_recheck(ix->w_cdist.as<float>(), nb, dx.C, w, qb, qn + q0, dx.coa, dx.coa_norm,
                                 ix->coa_len.as<float>(), coaidx + (int64_t)q0 * w, coadis + (int64_t)q0 * w, fl + 1,
                                 st));
    }
    ix->mixed_pending = true;
    return GBIVF_OK;
}

// after a synchronised search: report a device-side timeout of the mixed coarse stage
int check_device_flags(gbivf_index* ix) {
    if (!ix->mixed_pending) return GBIVF_OK;
    ix->mixed_pending = false;
    int h[3] = {0, 0, 0};
    CK(cudaMemcpy(h, ix->w_flags.p, sizeof(h), cudaMemcpyDeviceToHost));
    ix->last_ncand = h[1];
    ix->last_fallbacks = h[2];
    if (h[0]) return fail(GBIVF_ERR_TIMEOUT, "a bounded device-side wait ran out (tensor-core coarse stage or "
                                             "list-centric scan)");
    return GBIVF_OK;
}

// queries already on the device; everything enqueued on st
// (uneven batches: d_w / d_k / d_off per query, w and k their maxima; NULL = uniform)
// whether the precision-form scan serves this index and search shape (scan_persistent_supported)
bool mixed_scan_applies(const DevIndex& dx, int k, int kl, unsigned flags) {
    const int kk = (flags & (GBIVF_RERANK | GBIVF_RERANK_REFINE)) ? kl : k;
    return dx.d == 128 && dx.ks == 256 && (dx.m == 4 || dx.m == 8 || dx.m == 16) && std::max(kk, k) <= 1024 &&
           !(flags & GBIVF_TABLE_DIRECT);
}

// GBIVF_MIXED_SCAN_AUTO -> GBIVF_MIXED_SCAN or nothing
unsigned resolve_scan_form(const gbivf_index* ix, unsigned flags, int k, int kl) {
    if (!(flags & GBIVF_MIXED_SCAN_AUTO)) return flags;
    flags &= ~GBIVF_MIXED_SCAN_AUTO;
    const bool want = ix->auto_tuned ? ix->auto_mixed : ix->dx.m == 16;
    return want && mixed_scan_applies(ix->dx, k, kl, flags) ? flags | GBIVF_MIXED_SCAN : flags;
}

int search_device_impl(gbivf_index* ix, const float* d_q, int nq, int k, int kl, int w, unsigned flags,
                       int32_t* d_ids, float* d_dis, cudaStream_t st, const int32_t* d_w = nullptr,
                       const int32_t* d_k = nullptr, const int64_t* d_off = nullptr) {
    if (nq == 0) return GBIVF_OK;
    flags = resolve_scan_form(ix, flags, k, kl);
    const DevIndex& dx = ix->dx;
    CK(ix->w_qn.ensure(sizeof(double) * nq));
    CK(ix->w_coaidx.ensure(sizeof(int32_t) * (size_t)nq * w));
    CK(ix->w_coadis.ensure(sizeof(float) * (size_t)nq * w));
    double* qn = ix->w_qn.as<double>();
    int32_t* coaidx = ix->w_coaidx.as<int32_t>();
    float* coadis = ix->w_coadis.as<float>();
    const bool prof = flags & GBIVF_PROFILE;
    if (prof) {
        for (auto& e : ix->ev)
            if (!e) CK(cudaEventCreate(&e));
        CK(cudaEventRecord(ix->ev[0], st));
    }
    ix->ev_valid = false;
    // device flags ([0] a bounded wait ran out, [1], [2] coarse-stage counters), cleared per search
    CK(ix->w_flags.ensure(4 * sizeof(int)));
    CK(cudaMemsetAsync(ix->w_flags.p, 0, 4 * sizeof(int), st));
    CK(launch_norm_d(d_q, nq, dx.d, qn, st));
    {
        int rc = coarse_stage(ix, d_q, qn, nq, w, flags, coaidx, coadis, st, d_w);
        if (rc) return rc;
    }
    ScanArgs a;
    a.nq = nq;
    a.w = w;
    a.k = k;
    a.kl = kl;
    a.flags = (flags & GBIVF_RERANK ? SCAN_RERANK : 0) | (flags & GBIVF_TABLE_DIRECT ? SCAN_TABLE_DIRECT : 0) |
              (flags & GBIVF_MIXED_SCAN ? SCAN_MIXED : 0) | (flags & GBIVF_RERANK_REFINE ? SCAN_REFINE : 0);
    a.queries = d_q;
    a.qnorm = qn;
    a.probes = coaidx;
    a.out_ids = d_ids;
    a.out_dis = d_dis;
    a.w_per_q = d_w;
    a.k_per_q = d_k;
    a.out_off = d_off;
    if (prof) CK(cudaEventRecord(ix->ev[1], st));
    {
        int rs = run_scan(ix, a, st, prof ? ix->ev[3] : nullptr, flags);
        if (rs) return rs;
    }
    if (prof) {
        CK(cudaEventRecord(ix->ev[2], st));
        ix->ev_valid = true;
    }
    return GBIVF_OK;
}

}  // namespace

extern "C" {

const char* gbivf_last_error(void) { return g_err.c_str(); }

int gbivf_version(void) { return 1; }

int gbivf_index_create(gbivf_index** out, int device, int d, int coarsek, const float* coa, int nsq, int ks,
                       const float* pq, const int64_t* list_off, const int32_t* ids, const uint8_t* codes) {
    return create_impl(out, device, d, coarsek, coa, nsq, ks, pq, list_off, ids, codes);
}

int gbivf_index_create_device(gbivf_index** out, int device, int d, int coarsek, const float* coa, int nsq, int ks,
                              const float* pq, const int64_t* list_off, const int32_t* d_ids, const uint8_t* d_codes) {
    if (list_off && list_off[coarsek] > 0 && (!d_ids || !d_codes)) return fail(GBIVF_ERR_INVALID, "NULL device lists");
    return create_impl(out, device, d, coarsek, coa, nsq, ks, pq, list_off, d_ids, d_codes, true);
}

int gbivf_index_create_from_lists(gbivf_index** out, int device, int d, int coarsek, const float* coa, int nsq,
                                  int ks, const float* const* pq_centroids, const int32_t* list_sizes,
                                  const int32_t* const* list_ids, const int32_t* const* list_codes) {
    if (!pq_centroids || !list_sizes || !list_ids || !list_codes) return fail(GBIVF_ERR_INVALID, "NULL argument");
    if (d <= 0 || nsq <= 0 || d % nsq || coarsek <= 0) return fail(GBIVF_ERR_INVALID, "bad dimensions");
    if (ks <= 0 || ks > 256) return fail(GBIVF_ERR_UNSUPPORTED, "ks=%d > 256 cannot be held as byte codes", ks);
    const int ds = d / nsq;
    std::vector<float> pq((size_t)nsq * ks * ds);
    for (int s = 0; s < nsq; s++) {
        if (!pq_centroids[s]) return fail(GBIVF_ERR_INVALID, "pq_centroids[%d] is NULL", s);
        memcpy(&pq[(size_t)s * ks * ds], pq_centroids[s], sizeof(float) * ks * ds);
    }
    std::vector<int64_t> off(coarsek + 1, 0);
    for (int l = 0; l < coarsek; l++) {
        if (list_sizes[l] < 0) return fail(GBIVF_ERR_INVALID, "list %d size %d", l, list_sizes[l]);
        off[l + 1] = off[l] + list_sizes[l];
    }
    std::vector<int32_t> ids((size_t)off[coarsek]);
    std::vector<uint8_t> codes((size_t)off[coarsek] * nsq);
    for (int l = 0; l < coarsek; l++) {
        int n = list_sizes[l];
        if (!n) continue;
        if (!list_ids[l] || !list_codes[l]) return fail(GBIVF_ERR_INVALID, "list %d arrays are NULL", l);
        memcpy(&ids[(size_t)off[l]], list_ids[l], sizeof(int32_t) * n);
        for (int64_t i = 0; i < (int64_t)n * nsq; i++) {
            int32_t c = list_codes[l][i];
            if (c < 0 || c >= ks) return fail(GBIVF_ERR_INVALID, "list %d code %d outside 0..%d", l, c, ks - 1);
            codes[(size_t)off[l] * nsq + i] = (uint8_t)c;
        }
    }
    return create_impl(out, device, d, coarsek, coa, nsq, ks, pq.data(), off.data(), ids.data(), codes.data());
}

int gbivf_index_set_base(gbivf_index* ix, const float* base, int64_t n, int d) {
    if (!ix || !base || n <= 0) return fail(GBIVF_ERR_INVALID, "bad base arguments");
    if (d != ix->dx.d) return fail(GBIVF_ERR_INVALID, "base d=%d, index d=%d", d, ix->dx.d);
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    CK(ix->base.ensure(sizeof(float) * (size_t)n * d));
    CK(ix->base_norm.ensure(sizeof(float) * (size_t)n));
    CK(cudaMemcpyAsync(ix->base.p, base, sizeof(float) * (size_t)n * d, cudaMemcpyHostToDevice, ix->stream));
    CK(launch_norm_f(ix->base.as<float>(), n, d, ix->base_norm.as<float>(), ix->stream));
    CK(cudaStreamSynchronize(ix->stream));
    ix->dx.base = ix->base.as<float>();
    ix->dx.base_norm = ix->base_norm.as<float>();
    ix->dx.nbase = n;
    return GBIVF_OK;
}

// refinement codes: codebook m2 x 256 x (d/m2) floats (host), codes n x m2 bytes in the caller's
// list order (host or device), placed in the padded row layout of the PQ codes
static int set_refine_impl(gbivf_index* ix, int m2, int ks2, const float* pq2, const uint8_t* codes2, bool on_device) {
    if (!ix || !pq2 || (!codes2 && ix->h_off.back() > 0)) return fail(GBIVF_ERR_INVALID, "bad refinement arguments");
    const DevIndex& dx = ix->dx;
    if (dx.d != 128) return fail(GBIVF_ERR_UNSUPPORTED, "refinement codes need d = 128 (d = %d)", dx.d);
    if (ks2 != 256) return fail(GBIVF_ERR_UNSUPPORTED, "refinement codebooks have 256 centroids (ks2 = %d)", ks2);
    if (m2 <= 0 || 128 % m2 || (128 / m2) % 4) return fail(GBIVF_ERR_UNSUPPORTED, "m2 = %d (a divisor of 32)", m2);
    if ((dx.ds % 4) != 0) return fail(GBIVF_ERR_UNSUPPORTED, "refinement re-rank needs d/m a multiple of 4");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    const int64_t n = ix->h_off.back(), rows = dx.rows;
    CK(ix->pq2.ensure(sizeof(float) * 256 * 128));
    CK(cudaMemcpyAsync(ix->pq2.p, pq2, sizeof(float) * 256 * 128, cudaMemcpyHostToDevice, ix->stream));
    CK(ix->codes2.ensure((size_t)std::max<int64_t>(rows, 1) * m2));
    CK(cudaMemsetAsync(ix->codes2.p, 0, (size_t)std::max<int64_t>(rows, 1) * m2, ix->stream));
    if (n > 0) {
        if (on_device) {
            DBuf off, beg;
            CK(off.ensure(sizeof(int64_t) * ix->h_off.size()));
            CK(beg.ensure(sizeof(int64_t) * ix->h_beg.size()));
            CK(cudaMemcpyAsync(off.p, ix->h_off.data(), sizeof(int64_t) * ix->h_off.size(), cudaMemcpyHostToDevice,
                               ix->stream));
            CK(cudaMemcpyAsync(beg.p, ix->h_beg.data(), sizeof(int64_t) * ix->h_beg.size(), cudaMemcpyHostToDevice,
                               ix->stream));
            CK(launch_scatter_rows(codes2, off.as<int64_t>(), beg.as<int64_t>(), dx.C, m2, ix->codes2.as<uint8_t>(),
                                   ix->stream));
            CK(cudaStreamSynchronize(ix->stream));
            off.release();
            beg.release();
        } else {
            std::vector<uint8_t> pc((size_t)rows * m2, 0);
            for (int l = 0; l < dx.C; l++) {
                const int64_t len = ix->h_off[l + 1] - ix->h_off[l];
                if (len) memcpy(&pc[(size_t)ix->h_beg[l] * m2], codes2 + ix->h_off[l] * m2, (size_t)len * m2);
            }
            CK(cudaMemcpyAsync(ix->codes2.p, pc.data(), pc.size(), cudaMemcpyHostToDevice, ix->stream));
            CK(cudaStreamSynchronize(ix->stream));
        }
    } else {
        CK(cudaStreamSynchronize(ix->stream));
    }
    ix->dx.m2 = m2;
    ix->dx.ds2 = 128 / m2;
    ix->dx.pq2 = ix->pq2.as<float>();
    ix->dx.codes2 = ix->codes2.as<uint8_t>();
    return GBIVF_OK;
}

int gbivf_index_set_refine(gbivf_index* ix, int m2, int ks2, const float* pq2, const uint8_t* codes2) {
    return set_refine_impl(ix, m2, ks2, pq2, codes2, false);
}

int gbivf_index_set_refine_device(gbivf_index* ix, int m2, int ks2, const float* pq2, const uint8_t* d_codes2) {
    return set_refine_impl(ix, m2, ks2, pq2, d_codes2, true);
}

int gbivf_index_destroy(gbivf_index* ix) {
    if (!ix) return GBIVF_OK;
    {
        DeviceGuard g(ix->device);
        if (ix->stream) cudaStreamSynchronize(ix->stream);
        free_index(ix);
    }
    delete ix;
    return GBIVF_OK;
}

int gbivf_index_dims(const gbivf_index* ix, int* d, int* coarsek, int* nsq, int* ks, int64_t* n) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (d) *d = ix->dx.d;
    if (coarsek) *coarsek = ix->dx.C;
    if (nsq) *nsq = ix->dx.m;
    if (ks) *ks = ix->dx.ks;
    if (n) {
        int64_t s = 0;
        for (int32_t v : ix->h_len) s += v;
        *n = s;
    }
    return GBIVF_OK;
}

int gbivf_ivfpq_search_device(gbivf_index* ix, const float* d_queries, int nq, int k, int kl, int w,
                              unsigned flags, int32_t* d_ids, float* d_dis, void* stream) {
    int rc = check_search(ix, nq, k, kl, w, flags);
    if (rc) return rc;
    if (nq > 0 && (!d_queries || !d_ids || !d_dis)) return fail(GBIVF_ERR_INVALID, "NULL device buffer");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    return search_device_impl(ix, d_queries, nq, k, kl, w, flags, d_ids, d_dis, (cudaStream_t)stream);
}

int gbivf_ivfpq_search(gbivf_index* ix, const float* queries, int nq, int k, int kl, int w, unsigned flags,
                       int32_t* ids, float* dis) {
    int rc = check_search(ix, nq, k, kl, w, flags);
    if (rc) return rc;
    if (nq == 0) return GBIVF_OK;
    if (!queries || !ids || !dis) return fail(GBIVF_ERR_INVALID, "NULL host buffer");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    const size_t qb = sizeof(float) * (size_t)nq * ix->dx.d, ob = (size_t)nq * k;
    CK(ix->w_q.ensure(qb));
    CK(ix->w_ids.ensure(sizeof(int32_t) * ob));
    CK(ix->w_dis.ensure(sizeof(float) * ob));
    CK(cudaMemcpyAsync(ix->w_q.p, queries, qb, cudaMemcpyHostToDevice, ix->stream));
    rc = search_device_impl(ix, ix->w_q.as<float>(), nq, k, kl, w, flags, ix->w_ids.as<int32_t>(),
                            ix->w_dis.as<float>(), ix->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ids, ix->w_ids.p, sizeof(int32_t) * ob, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaMemcpyAsync(dis, ix->w_dis.p, sizeof(float) * ob, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaStreamSynchronize(ix->stream));
    return check_device_flags(ix);
}

int gbivf_last_stage_ms(gbivf_index* ix, float* coarse_ms, float* scan_ms) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (!ix->ev_valid) return fail(GBIVF_ERR_INVALID, "no search with GBIVF_PROFILE since the last one without");
    DeviceGuard g(ix->device);
    CK(cudaEventSynchronize(ix->ev[2]));
    float a = 0, b = 0;
    CK(cudaEventElapsedTime(&a, ix->ev[0], ix->ev[1]));
    CK(cudaEventElapsedTime(&b, ix->ev[1], ix->ev[2]));
    if (coarse_ms) *coarse_ms = a;
    if (scan_ms) *scan_ms = b;
    return GBIVF_OK;
}

int gbivf_last_stages_ms(gbivf_index* ix, float* coarse_ms, float* scan_ms, float* finalize_ms) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (!ix->ev_valid) return fail(GBIVF_ERR_INVALID, "no search with GBIVF_PROFILE since the last one without");
    DeviceGuard g(ix->device);
    CK(cudaEventSynchronize(ix->ev[2]));
    float a = 0, b = 0, c = 0;
    CK(cudaEventElapsedTime(&a, ix->ev[0], ix->ev[1]));
    CK(cudaEventElapsedTime(&b, ix->ev[1], ix->ev[3]));
    CK(cudaEventElapsedTime(&c, ix->ev[3], ix->ev[2]));
    if (coarse_ms) *coarse_ms = a;
    if (scan_ms) *scan_ms = b;
    if (finalize_ms) *finalize_ms = c;
    return GBIVF_OK;
}

int gbivf_last_scan_parts(gbivf_index* ix, float* parts_ms, int64_t* counters) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (!ix->ev_valid) return fail(GBIVF_ERR_INVALID, "no search with GBIVF_PROFILE since the last one without");
    DeviceGuard g(ix->device);
    CK(cudaEventSynchronize(ix->ev[2]));
    const bool lists = ix->last_list_scan;
    if (parts_ms) {
        for (int i = 0; i < 7; i++) parts_ms[i] = 0.0f;
        if (lists) {
            cudaEvent_t seq[8] = {ix->ev[1], ix->lc_ev[0], ix->lc_ev[1], ix->lc_ev[2],
                                  ix->lc_ev[3], ix->lc_ev[4], ix->ev[3], ix->ev[2]};
            for (int i = 0; i < 7; i++) CK(cudaEventElapsedTime(&parts_ms[i], seq[i], seq[i + 1]));
        } else {
            CK(cudaEventElapsedTime(&parts_ms[3], ix->ev[1], ix->ev[3]));
            CK(cudaEventElapsedTime(&parts_ms[6], ix->ev[3], ix->ev[2]));
        }
    }
    if (counters) {
        for (int i = 0; i < 4; i++) counters[i] = 0;
        if (lists) {
            int h[3] = {0, 0, 0}, npairs = 0;
            CK(cudaMemcpy(h, ix->lcw.counters, sizeof(h), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(&npairs, ix->lcw.pbeg + ix->dx.C, sizeof(int), cudaMemcpyDeviceToHost));
            counters[0] = npairs;
            counters[1] = h[0];
            counters[2] = h[2];
            counters[3] = 1;
        }
    }
    return GBIVF_OK;
}

int gbivf_last_unproven(gbivf_index* ix, int64_t* queries) {
    if (!ix || !queries) return fail(GBIVF_ERR_INVALID, "index or output is NULL");
    DeviceGuard g(ix->device);
    *queries = 0;
    if (!ix->last_mixed || !ix->w_unproven.p) return GBIVF_OK;
    int h = 0;
    CK(cudaStreamSynchronize(ix->stream));
    CK(cudaMemcpy(&h, ix->w_unproven.p, sizeof(int), cudaMemcpyDeviceToHost));
    *queries = h;
    return GBIVF_OK;
}

}  // extern "C"

struct gbivf_graph {
    gbivf_index* ix = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// the scan kernel choices the autotuner compares
struct ScanVariant {
    bool persistent;
    int threads;
    bool lists;  // the list-centric pipeline
};
constexpr ScanVariant kVariants[4] = {{true, 512, false}, {true, 1024, false}, {false, 0, false}, {true, 512, true}};
constexpr int kVariantCode[4] = {512, 1024, 0, 1};  // *choice and the tuning cache's value

std::string tune_key(gbivf_index* ix, int k, int w, unsigned flags) {
    // index shape, a coarse histogram of list sizes, the GPU, and the search shape
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, ix->device) != cudaSuccess) p.name[0] = 0;
    int64_t n = 0, mx = 0;
    for (int32_t v : ix->h_len) {
        n += v;
        mx = std::max<int64_t>(mx, v);
    }
    int hist[8] = {0};
    const double mean = ix->h_len.empty() ? 1.0 : std::max(1.0, (double)n / ix->h_len.size());
    for (int32_t v : ix->h_len) {
        int b = 0;
        double r = v / mean;
        while (b < 7 && r > 0.25 * (1 << b)) b++;
        hist[b]++;
    }
    char buf[512];
    snprintf(buf, sizeof buf, "d%d_C%d_m%d_n%lld_max%lld_h%d.%d.%d.%d.%d.%d.%d.%d_k%d_w%d_f%x_%s", ix->dx.d, ix->dx.C,
             ix->dx.m, (long long)n, (long long)mx, hist[0], hist[1], hist[2], hist[3], hist[4], hist[5], hist[6],
             hist[7], k, w, flags & ~GBIVF_PROFILE, p.name);
    for (char* c = buf; *c; c++)
        if (*c == ' ' || *c == '\n') *c = '_';
    return buf;
}

}  // namespace

extern "C" {

int gbivf_graph_capture(gbivf_index* ix, const float* d_queries, int nq, int k, int kl, int w, unsigned flags,
                        int32_t* d_ids, float* d_dis, const int32_t* d_w, const int32_t* d_k, const int64_t* d_out_off,
                        void* stream, gbivf_graph** out) {
    if (!out) return fail(GBIVF_ERR_INVALID, "out is NULL");
    *out = nullptr;
    const bool uneven = d_w || d_k || d_out_off;
    if (uneven && !(d_w && d_k && d_out_off)) return fail(GBIVF_ERR_INVALID, "d_w, d_k and d_out_off go together");
    if (uneven && (flags & GBIVF_RERANK)) return fail(GBIVF_ERR_UNSUPPORTED, "uneven batches do not re-rank");
    flags &= ~GBIVF_PROFILE;
    int rc = check_search(ix, nq, k, uneven ? k : kl, w, flags);
    if (rc) return rc;
    if (nq <= 0 || !d_queries || !d_ids || !d_dis) return fail(GBIVF_ERR_INVALID, "empty or NULL search");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    cudaStream_t st = (cudaStream_t)stream;
    // one run sizes the workspace and prepares every lazily built buffer
    rc = search_device_impl(ix, d_queries, nq, k, uneven ? k : kl, w, flags, d_ids, d_dis, st, d_w, d_k, d_out_off);
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    ix->mixed_pending = false;
    auto* gr = new gbivf_graph();
    gr->ix = ix;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        delete gr;
        return cuda_fail(e, "cudaStreamBeginCapture");
    }
    rc = search_device_impl(ix, d_queries, nq, k, uneven ? k : kl, w, flags, d_ids, d_dis, st, d_w, d_k, d_out_off);
    e = cudaStreamEndCapture(st, &gr->graph);
    ix->mixed_pending = false;
    if (rc || e != cudaSuccess) {
        if (gr->graph) cudaGraphDestroy(gr->graph);
        delete gr;
        return rc ? rc : cuda_fail(e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&gr->exec, gr->graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(gr->graph);
        delete gr;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    *out = gr;
    return GBIVF_OK;
}

int gbivf_graph_launch(gbivf_graph* gr, void* stream) {
    if (!gr || !gr->exec) return fail(GBIVF_ERR_INVALID, "graph is NULL");
    DeviceGuard g(gr->ix->device);
    CK(cudaGraphLaunch(gr->exec, (cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_graph_kernel_count(const gbivf_graph* gr, int* kernels) {
    if (!gr || !gr->graph || !kernels) return fail(GBIVF_ERR_INVALID, "NULL argument");
    DeviceGuard g(gr->ix->device);
    size_t n = 0;
    CK(cudaGraphGetNodes(gr->graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) CK(cudaGraphGetNodes(gr->graph, nodes.data(), &n));
    int k = 0;
    for (size_t i = 0; i < n; i++) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nodes[i], &t));
        k += t == cudaGraphNodeTypeKernel;
    }
    *kernels = k;
    return GBIVF_OK;
}

int gbivf_graph_destroy(gbivf_graph* gr) {
    if (!gr) return GBIVF_OK;
    DeviceGuard g(gr->ix->device);
    if (gr->exec) cudaGraphExecDestroy(gr->exec);
    if (gr->graph) cudaGraphDestroy(gr->graph);
    delete gr;
    return GBIVF_OK;
}

int gbivf_index_autotune(gbivf_index* ix, const float* d_queries, int nq, int k, int kl, int w, unsigned flags,
                         int* choice, float* times_ms) {
    int rc = check_search(ix, nq, k, kl, w, flags);
    if (rc) return rc;
    if (nq <= 0 || !d_queries) return fail(GBIVF_ERR_INVALID, "empty calibration batch");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    // GBIVF_MIXED_SCAN_AUTO: the kernel variant is tuned on the exact form, then the two scan forms
    // are timed with it and the faster one is kept for the flag
    const bool auto_form = flags & GBIVF_MIXED_SCAN_AUTO;
    const std::string key = tune_key(ix, k, w, flags);
    const std::string form_key = key + "_scanform";
    flags &= ~GBIVF_MIXED_SCAN_AUTO;
    const char* cache = getenv("GBIVF_TUNE_CACHE");
    int cached_th = -1, cached_form = -1;
    if (cache) {  // "key threads" lines (threads 0 = the general kernel) and "key_scanform 0|1" lines
        if (FILE* f = fopen(cache, "r")) {
            char kbuf[600];
            int v = -1;
            while (fscanf(f, "%599s %d", kbuf, &v) == 2) {
                if (key == kbuf) cached_th = v;
                if (form_key == kbuf) cached_form = v;
            }
            fclose(f);
        }
    }
    if (cached_th >= 0) {
        ix->use_persistent = cached_th != 0;
        ix->scan_threads = cached_th == 1024 ? 1024 : 512;
        ix->list_pref = cached_th == 1 ? 1 : 0;
        if (choice) *choice = cached_th;
        if (times_ms) times_ms[0] = times_ms[1] = times_ms[2] = times_ms[3] = -1.0f;
        if (!auto_form) return GBIVF_OK;
        if (cached_form >= 0) {
            ix->auto_tuned = true;
            ix->auto_mixed = cached_form != 0;
            return GBIVF_OK;
        }
    }
    const size_t ob = (size_t)nq * k;
    CK(ix->w_ids.ensure(sizeof(int32_t) * ob));
    CK(ix->w_dis.ensure(sizeof(float) * ob));
    CK(ix->w_queue.ensure(sizeof(int)));
    // scan + finalize time of one search, the mean of repetitions 2 and 3
    auto time_scan = [&](unsigned fl, float* out) -> int {
        float sum = 0.0f;
        for (int rep = 0; rep < 3; rep++) {
            int r = search_device_impl(ix, d_queries, nq, k, kl, w, fl | GBIVF_PROFILE, ix->w_ids.as<int32_t>(),
                                       ix->w_dis.as<float>(), ix->stream);
            if (r) return r;
            CK(cudaStreamSynchronize(ix->stream));
            float sm = 0;
            CK(cudaEventElapsedTime(&sm, ix->ev[1], ix->ev[2]));
            if (rep > 0) sum += sm;
        }
        *out = sum / 2.0f;
        return GBIVF_OK;
    };
    if (cached_th < 0) {
        const bool save_p = ix->use_persistent;
        const int save_t = ix->scan_threads;
        float best = 1e30f;
        int best_i = -1;
        for (int i = 0; i < 4; i++) {
            ix->use_persistent = kVariants[i].persistent;
            ix->scan_threads = kVariants[i].persistent ? kVariants[i].threads : save_t;
            float t = -1.0f;
            ScanArgs probe;
            probe.nq = nq;
            probe.w = w;
            probe.k = k;
            probe.kl = kl;
            probe.flags = flags & GBIVF_RERANK ? SCAN_RERANK : 0;
            probe.queue = ix->w_queue.as<int>();
            const bool applies = kVariants[i].lists ? list_scan_supported(ix->dx, probe)
                                                    : !kVariants[i].persistent || scan_persistent_supported(ix->dx, probe);
            if (applies) {
                rc = time_scan((flags & ~(GBIVF_LIST_SCAN | GBIVF_QUERY_SCAN)) |
                                   (kVariants[i].lists ? GBIVF_LIST_SCAN : GBIVF_QUERY_SCAN),
                               &t);
                if (rc) break;
                if (t < best) {
                    best = t;
                    best_i = i;
                }
            }
            if (times_ms) times_ms[i] = t;
        }
        ix->mixed_pending = false;
        if (rc || best_i < 0) {
            ix->use_persistent = save_p;
            ix->scan_threads = save_t;
            return rc ? rc : fail(GBIVF_ERR_INVALID, "no scan kernel applies");
        }
        ix->use_persistent = kVariants[best_i].persistent;
        ix->scan_threads = kVariants[best_i].persistent ? kVariants[best_i].threads : save_t;
        ix->list_pref = kVariants[best_i].lists ? 1 : 0;
        const int th = kVariantCode[best_i];
        if (choice) *choice = th;
        if (cache)
            if (FILE* f = fopen(cache, "a")) {
                fprintf(f, "%s %d\n", key.c_str(), th);
                fclose(f);
            }
    }
    if (auto_form) {
        bool mixed = false;
        if (mixed_scan_applies(ix->dx, k, kl, flags)) {
            float t_exact = 0.0f, t_mixed = 0.0f;
            if ((rc = time_scan(flags, &t_exact)) || (rc = time_scan(flags | GBIVF_MIXED_SCAN, &t_mixed))) {
                ix->mixed_pending = false;
                return rc;
            }
            mixed = t_mixed < t_exact;
        }
        ix->mixed_pending = false;
        ix->auto_tuned = true;
        ix->auto_mixed = mixed;
        if (cache)
            if (FILE* f = fopen(cache, "a")) {
                fprintf(f, "%s %d\n", form_key.c_str(), mixed ? 1 : 0);
                fclose(f);
            }
    }
    return GBIVF_OK;
}

int gbivf_index_scan_form(const gbivf_index* ix, int* tuned, int* mixed) {
    if (!ix || !tuned || !mixed) return fail(GBIVF_ERR_INVALID, "NULL argument");
    *tuned = ix->auto_tuned ? 1 : 0;
    *mixed = (ix->auto_tuned ? ix->auto_mixed : ix->dx.m == 16) ? 1 : 0;
    return GBIVF_OK;
}

int gbivf_search_batched_device(gbivf_index* ix, const float* d_queries, int nq, const int32_t* d_w,
                                const int32_t* d_k, const int64_t* d_out_off, int max_w, int max_k, unsigned flags,
                                int32_t* d_ids, float* d_dis, void* stream) {
    if (flags & (GBIVF_RERANK | GBIVF_RERANK_REFINE)) return fail(GBIVF_ERR_UNSUPPORTED, "uneven batches do not re-rank");
    int rc = check_search(ix, nq, max_k, max_k, max_w, flags);
    if (rc) return rc;
    if (nq > 0 && (!d_queries || !d_w || !d_k || !d_out_off || !d_ids || !d_dis))
        return fail(GBIVF_ERR_INVALID, "NULL device buffer");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    return search_device_impl(ix, d_queries, nq, max_k, max_k, max_w, flags, d_ids, d_dis, (cudaStream_t)stream, d_w,
                              d_k, d_out_off);
}

int gbivf_search_batched(gbivf_index* ix, const float* queries, int nq, const int32_t* w_per_q,
                         const int32_t* k_per_q, unsigned flags, int32_t* ids, float* dis) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (nq < 0) return fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    if (nq == 0) return GBIVF_OK;
    if (!queries || !w_per_q || !k_per_q || !ids || !dis) return fail(GBIVF_ERR_INVALID, "NULL host buffer");
    if (flags & (GBIVF_RERANK | GBIVF_RERANK_REFINE)) return fail(GBIVF_ERR_UNSUPPORTED, "uneven batches do not re-rank");
    int max_w = 0, max_k = 0;
    std::vector<int64_t> off(nq);
    int64_t total = 0;
    for (int q = 0; q < nq; q++) {
        if (w_per_q[q] < 1 || w_per_q[q] > ix->dx.C)
            return fail(GBIVF_ERR_INVALID, "w_per_q[%d]=%d outside 1..%d", q, w_per_q[q], ix->dx.C);
        if (k_per_q[q] < 1) return fail(GBIVF_ERR_INVALID, "k_per_q[%d]=%d", q, k_per_q[q]);
        max_w = std::max(max_w, w_per_q[q]);
        max_k = std::max(max_k, k_per_q[q]);
        off[q] = total;
        total += k_per_q[q];
    }
    int rc = check_search(ix, nq, max_k, max_k, max_w, flags);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    const size_t qb = sizeof(float) * (size_t)nq * ix->dx.d;
    CK(ix->w_q.ensure(qb));
    CK(ix->w_ids.ensure(sizeof(int32_t) * (size_t)total));
    CK(ix->w_dis.ensure(sizeof(float) * (size_t)total));
    CK(ix->w_res.ensure(sizeof(int32_t) * (2 * (size_t)nq + 2) + sizeof(int64_t) * (size_t)nq));
    int32_t* dw = ix->w_res.as<int32_t>();
    int32_t* dk = dw + nq;
    int64_t* doff = reinterpret_cast<int64_t*>(dk + nq + (nq & 1));
    CK(cudaMemcpyAsync(ix->w_q.p, queries, qb, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(dw, w_per_q, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(dk, k_per_q, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * nq, cudaMemcpyHostToDevice, ix->stream));
    rc = search_device_impl(ix, ix->w_q.as<float>(), nq, max_k, max_k, max_w, flags, ix->w_ids.as<int32_t>(),
                            ix->w_dis.as<float>(), ix->stream, dw, dk, doff);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ids, ix->w_ids.p, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaMemcpyAsync(dis, ix->w_dis.p, sizeof(float) * (size_t)total, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaStreamSynchronize(ix->stream));
    return check_device_flags(ix);
}

int gbivf_coarse_assign_flags(gbivf_index* ix, const float* queries, int nq, int w, unsigned flags, int32_t* coaidx,
                              float* coadis, int64_t* ncand) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (w <= 0 || w > ix->dx.C || w > MAX_W) return fail(GBIVF_ERR_INVALID, "w=%d", w);
    if (flags & ~(GBIVF_MIXED_COARSE | GBIVF_COARSE_FULL | GBIVF_PROFILE))
        return fail(GBIVF_ERR_INVALID, "unknown flags 0x%x", flags);
    if ((flags & GBIVF_MIXED_COARSE) && ix->dx.d != 128)
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_MIXED_COARSE needs d = 128 (d = %d)", ix->dx.d);
    if (ncand) *ncand = 0;
    if (nq <= 0) return nq == 0 ? GBIVF_OK : fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    if (!queries || !coaidx || !coadis) return fail(GBIVF_ERR_INVALID, "NULL host buffer");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    const DevIndex& dx = ix->dx;
    const size_t qb = sizeof(float) * (size_t)nq * dx.d;
    CK(ix->w_q.ensure(qb));
    CK(ix->w_qn.ensure(sizeof(double) * nq));
    CK(ix->w_coaidx.ensure(sizeof(int32_t) * (size_t)nq * w));
    CK(ix->w_coadis.ensure(sizeof(float) * (size_t)nq * w));
    CK(cudaMemcpyAsync(ix->w_q.p, queries, qb, cudaMemcpyHostToDevice, ix->stream));
    CK(launch_norm_d(ix->w_q.as<float>(), nq, dx.d, ix->w_qn.as<double>(), ix->stream));
    int rc = coarse_stage(ix, ix->w_q.as<float>(), ix->w_qn.as<double>(), nq, w, flags, ix->w_coaidx.as<int32_t>(),
                          ix->w_coadis.as<float>(), ix->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(coaidx, ix->w_coaidx.p, sizeof(int32_t) * (size_t)nq * w, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaMemcpyAsync(coadis, ix->w_coadis.p, sizeof(float) * (size_t)nq * w, cudaMemcpyDeviceToHost, ix->stream));
    CK(cudaStreamSynchronize(ix->stream));
    ix->last_ncand = 0;
    ix->last_fallbacks = 0;
    rc = check_device_flags(ix);
    if (ncand) *ncand = ix->last_ncand;
    return rc;
}

int gbivf_coarse_assign_device(gbivf_index* ix, const float* d_queries, int nq, int w, unsigned flags,
                               int32_t* d_coaidx, float* d_coadis, void* stream) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (w <= 0 || w > ix->dx.C || w > MAX_W) return fail(GBIVF_ERR_INVALID, "w=%d", w);
    if (flags & ~(GBIVF_MIXED_COARSE | GBIVF_COARSE_FULL)) return fail(GBIVF_ERR_INVALID, "unknown flags 0x%x", flags);
    if ((flags & GBIVF_MIXED_COARSE) && ix->dx.d != 128)
        return fail(GBIVF_ERR_UNSUPPORTED, "GBIVF_MIXED_COARSE needs d = 128 (d = %d)", ix->dx.d);
    if (nq < 0) return fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    if (nq == 0) return GBIVF_OK;
    if (!d_queries || !d_coaidx || !d_coadis) return fail(GBIVF_ERR_INVALID, "NULL device buffer");
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    cudaStream_t st = (cudaStream_t)stream;
    CK(ix->w_qn.ensure(sizeof(double) * nq));
    CK(launch_norm_d(d_queries, nq, ix->dx.d, ix->w_qn.as<double>(), st));
    return coarse_stage(ix, d_queries, ix->w_qn.as<double>(), nq, w, flags, d_coaidx, d_coadis, st);
}

int gbivf_last_coarse_stats(gbivf_index* ix, int64_t* rechecked, int64_t* fallback_queries) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (rechecked) *rechecked = ix->last_ncand;
    if (fallback_queries) *fallback_queries = ix->last_fallbacks;
    return GBIVF_OK;
}

int gbivf_coarse_assign(gbivf_index* ix, const float* queries, int nq, int w, int32_t* coaidx, float* coadis) {
    return gbivf_coarse_assign_flags(ix, queries, nq, w, 0u, coaidx, coadis, nullptr);
}

int gbivf_core_gpu(gbivf_index* ix, const float* residual, int nres, const int32_t* rid_to_ivf,
                   const int32_t* qid_to_starting_outid, int32_t* idxs, float* dists, int k, int w) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (w <= 0 || w > MAX_W || k <= 0 || k > MAX_K || nres < 0 || nres % w)
        return fail(GBIVF_ERR_INVALID, "bad sizes nres=%d w=%d k=%d", nres, w, k);
    if (nres == 0) return GBIVF_OK;
    if (!residual || !rid_to_ivf || !qid_to_starting_outid || !idxs || !dists)
        return fail(GBIVF_ERR_INVALID, "NULL host buffer");
    const int nq = nres / w;
    int64_t nout = 0;
    for (int q = 0; q < nq; q++) {
        int64_t L = 0;
        for (int j = 0; j < w; j++) {
            int l = rid_to_ivf[(int64_t)q * w + j];
            if (l < 0 || l >= ix->dx.C) return fail(GBIVF_ERR_INVALID, "rid_to_ivf[%d]=%d", q * w + j, l);
            L += ix->h_len[l];
        }
        if (qid_to_starting_outid[q] < 0) return fail(GBIVF_ERR_INVALID, "negative output offset");
        nout = std::max<int64_t>(nout, qid_to_starting_outid[q] + std::min<int64_t>(L, k));
    }
    std::lock_guard<std::mutex> lk(ix->mu);
    DeviceGuard g(ix->device);
    const DevIndex& dx = ix->dx;
    CK(ix->w_res.ensure(sizeof(float) * (size_t)nres * dx.d));
    CK(ix->w_coaidx.ensure(sizeof(int32_t) * (size_t)nres));
    CK(ix->w_start.ensure(sizeof(int32_t) * (size_t)nq));
    CK(ix->w_ids.ensure(sizeof(int32_t) * (size_t)std::max<int64_t>(nout, 1)));
    CK(ix->w_dis.ensure(sizeof(float) * (size_t)std::max<int64_t>(nout, 1)));
    CK(cudaMemcpyAsync(ix->w_res.p, residual, sizeof(float) * (size_t)nres * dx.d, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(ix->w_coaidx.p, rid_to_ivf, sizeof(int32_t) * (size_t)nres, cudaMemcpyHostToDevice, ix->stream));
    CK(cudaMemcpyAsync(ix->w_start.p, qid_to_starting_outid, sizeof(int32_t) * (size_t)nq, cudaMemcpyHostToDevice,
                       ix->stream));
    ScanArgs a;
    a.nq = nq;
    a.w = w;
    a.k = k;
    a.kl = k;
    a.flags = SCAN_SRC_RESIDUAL | SCAN_TABLE_DIRECT | SCAN_OUT_PACKED;
    a.residual = ix->w_res.as<float>();
    a.probes = ix->w_coaidx.as<int32_t>();
    a.out_start = ix->w_start.as<int32_t>();
    a.out_ids = ix->w_ids.as<int32_t>();
    a.out_dis = ix->w_dis.as<float>();
    int rc = run_scan(ix, a, ix->stream);
    if (rc) return rc;
    // copy back only the written ranges
    for (int q = 0; q < nq; q++) {
        int64_t L = 0;
        for (int j = 0; j < w; j++) L += ix->h_len[rid_to_ivf[(int64_t)q * w + j]];
        int64_t cnt = std::min<int64_t>(L, k), o = qid_to_starting_outid[q];
        if (!cnt) continue;
        CK(cudaMemcpyAsync(idxs + o, ix->w_ids.as<int32_t>() + o, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, ix->stream));
        CK(cudaMemcpyAsync(dists + o, ix->w_dis.as<float>() + o, sizeof(float) * cnt, cudaMemcpyDeviceToHost, ix->stream));
    }
    CK(cudaStreamSynchronize(ix->stream));
    return GBIVF_OK;
}

int gbivf_pq_create(gbivf_index** out, int device, int d, int nsq, int ks, const float* pq, const uint8_t* codes,
                    int64_t n) {
    if (n < 0) return fail(GBIVF_ERR_INVALID, "n=%lld", (long long)n);
    if (n > 0x7fffffffLL) return fail(GBIVF_ERR_UNSUPPORTED, "flat PQ limited to 2^31-1 codes");
    if (d <= 0) return fail(GBIVF_ERR_INVALID, "d=%d", d);
    std::vector<float> zero((size_t)d, 0.0f);
    int64_t off[2] = {0, n};
    std::vector<int32_t> ids((size_t)n);
    for (int64_t i = 0; i < n; i++) ids[(size_t)i] = (int32_t)i;
    return create_impl(out, device, d, 1, zero.data(), nsq, ks, pq, off, ids.data(), codes);
}

int gbivf_pq_search(gbivf_index* ix, const float* queries, int nq, int k, float* dis, int32_t* ids) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (ix->dx.C != 1) return fail(GBIVF_ERR_INVALID, "not a flat PQ index (use gbivf_pq_create)");
    if (k > ix->h_len[0]) return fail(GBIVF_ERR_INVALID, "k=%d > n=%d (pq_search needs k <= n)", k, ix->h_len[0]);
    if (nq <= 0) return nq == 0 ? GBIVF_OK : fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    std::vector<int32_t> rid((size_t)nq * k);
    std::vector<float> rdis((size_t)nq * k);
    int rc = gbivf_ivfpq_search(ix, queries, nq, k, 0, 1, 0u, rid.data(), rdis.data());
    if (rc) return rc;
    for (int q = 0; q < nq; q++)
        for (int l = 0; l < k; l++) {  // column-major, 1-based
            dis[(int64_t)nq * l + q] = rdis[(size_t)q * k + l];
            ids[(int64_t)nq * l + q] = rid[(size_t)q * k + l] + 1;
        }
    return GBIVF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Coarse assignment without device allocation.
//
// Some callers cannot call cudaMalloc: a host that hands its plugins a fixed
// device-memory budget and forbids them to allocate, or a serving loop that
// must not take the allocator's device-wide synchronisation on its latency
// path. For them the coarse stage's scratch (query norms and the query x
// centroid distance block) lives in one file-scope device array of
// GBIVF_NOALLOC_SCRATCH_BYTES. Every GPU that loads this library holds the
// array until the process exits. The host resolves the array's device address
// with cudaGetSymbolAddress on the first call made on a device, and again on
// the first call after that device's context was replaced (cudaDeviceReset,
// a new primary context): the module, and with it the array, is loaded anew
// in every context. Such a first call should come before any stream capture.
// All calls share the array: calls that overlap on the GPU (other streams,
// other threads) race on it. The kernels overwrite every scratch byte they
// read, so nothing needs clearing between calls.
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)GBIVF_NOALLOC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mu;
struct NoallocSlot {
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;  // the context the address belongs to
};
NoallocSlot g_noalloc[128];

// scratch bytes of one call: the query norms (rounded up to 256 bytes), then the distance block
size_t noalloc_need(int64_t nq, int C) {
    return ((size_t)nq * sizeof(double) + 255) / 256 * 256 + (size_t)nq * C * sizeof(float);
}

// the largest batch whose scratch fits
int64_t noalloc_max_queries(int C) {
    int64_t nq = (int64_t)((kNoallocScratchBytes - 256) / (sizeof(double) + (size_t)C * sizeof(float)));
    while (nq > 0 && noalloc_need(nq, C) > kNoallocScratchBytes) nq--;
    while (noalloc_need(nq + 1, C) <= kNoallocScratchBytes) nq++;
    return nq;
}

// Unique id of the calling thread's current context, from the driver (resolved through the
// runtime, so the library needs no link against the driver library); 0 when unknown.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" int gbivf_coarse_assign_noalloc(gbivf_index* ix, const float* d_queries, int nq, int w, int32_t* d_coaidx,
                                           float* d_coadis, void* stream) {
    if (!ix) return fail(GBIVF_ERR_INVALID, "index is NULL");
    if (w <= 0 || w > ix->dx.C || w > MAX_W) return fail(GBIVF_ERR_INVALID, "w=%d", w);
    if (nq < 0) return fail(GBIVF_ERR_INVALID, "nq=%d", nq);
    if (nq == 0) return GBIVF_OK;
    if (!d_queries || !d_coaidx || !d_coadis) return fail(GBIVF_ERR_INVALID, "NULL device buffer");
    const DevIndex& dx = ix->dx;
    const size_t norm_bytes = ((size_t)nq * sizeof(double) + 255) / 256 * 256;
    const size_t need = noalloc_need(nq, dx.C);
    if (need > kNoallocScratchBytes)
        return fail(GBIVF_ERR_UNSUPPORTED,
                    "nq=%d with coarsek=%d needs %zu scratch bytes; the no-allocation scratch holds %zu "
                    "(at most %lld queries per call at this coarsek)",
                    nq, dx.C, need, kNoallocScratchBytes, (long long)noalloc_max_queries(dx.C));
    if (ix->device < 0 || ix->device >= 128) return fail(GBIVF_ERR_UNSUPPORTED, "device %d", ix->device);
    DeviceGuard g(ix->device);
    if (!g.ok) return fail(GBIVF_ERR_CUDA, "cudaSetDevice(%d) failed", ix->device);
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        NoallocSlot& slot = g_noalloc[ix->device];
        const unsigned long long ctx = current_context_id();
        if (!slot.ptr || ctx == 0 || ctx != slot.ctx_id) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
            slot.ptr = p;
            slot.ctx_id = ctx;
        }
        base = slot.ptr;
    }
    double* qn = reinterpret_cast<double*>(base);
    float* dist = reinterpret_cast<float*>(static_cast<unsigned char*>(base) + norm_bytes);
    cudaStream_t st = (cudaStream_t)stream;
    CK(launch_norm_d(d_queries, nq, dx.d, qn, st));
    CK(launch_coarse_dist(dx, d_queries, qn, nq, dist, st));
    CK(launch_coarse_select(dist, nq, dx.C, w, d_coaidx, d_coadis, st));
    return GBIVF_OK;
}

// ---------------------------------------------------------------------------
// Index building on the GPU (build_gpu.cu). Synchronous; device buffers.
// ---------------------------------------------------------------------------

extern "C" {

int gbivf_generate_mixture(float* d_out, int64_t n, int d, const float* d_means, int ncomp, const double* d_cdf,
                           float sigma, uint64_t seed, uint64_t stream_id, int64_t row0, void* stream) {
    if (!d_out || !d_means || n < 0 || d <= 0 || d % 2 || ncomp <= 0)
        return fail(GBIVF_ERR_INVALID, "bad mixture arguments");
    CK(gen_mixture(d_out, n, d, d_means, ncomp, d_cdf, sigma, seed, stream_id, row0, (cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_kmeans(const float* d_x, int64_t n, int d, int k, int niter, uint64_t seed, float* d_centroids,
                 void* stream) {
    if (!d_x || !d_centroids || n <= 0 || k <= 0 || niter < 0) return fail(GBIVF_ERR_INVALID, "bad k-means arguments");
    if (d != 128 && d != 8 && d != 16 && d != 32)
        return fail(GBIVF_ERR_UNSUPPORTED, "k-means on the GPU takes d = 128 (tensor cores) or 8, 16, 32");
    CK(kmeans_rows(d_x, n, d, d, k, niter, seed, d_centroids, (cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_assign_flags(const float* d_x, int64_t n, int d, const float* d_centroids, int k, int32_t* d_assign,
                       unsigned flags, void* stream) {
    if (!d_x || !d_centroids || !d_assign || n < 0 || k <= 0) return fail(GBIVF_ERR_INVALID, "bad assign arguments");
    if (flags & ~GBIVF_ASSIGN_BF16) return fail(GBIVF_ERR_INVALID, "unknown flags 0x%x", flags);
    if (d != 128 && d != 8 && d != 16 && d != 32)
        return fail(GBIVF_ERR_UNSUPPORTED, "assignment on the GPU takes d = 128 or 8, 16, 32");
    if (n == 0) return GBIVF_OK;
    cudaError_t e = assign_rows(d_x, n, d, d, d_centroids, k, d_assign, (cudaStream_t)stream,
                                (flags & GBIVF_ASSIGN_BF16) != 0);
    if (e == cudaErrorLaunchTimeout) return fail(GBIVF_ERR_TIMEOUT, "tensor-core assignment: a bounded wait ran out");
    CK(e);
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_assign(const float* d_x, int64_t n, int d, const float* d_centroids, int k, int32_t* d_assign,
                 void* stream) {
    if (!d_x || !d_centroids || !d_assign || n < 0 || k <= 0) return fail(GBIVF_ERR_INVALID, "bad assign arguments");
    if (d != 128 && d != 8 && d != 16 && d != 32)
        return fail(GBIVF_ERR_UNSUPPORTED, "assignment on the GPU takes d = 128 or 8, 16, 32");
    if (n == 0) return GBIVF_OK;
    cudaError_t e = assign_rows(d_x, n, d, d, d_centroids, k, d_assign, (cudaStream_t)stream);
    if (e == cudaErrorLaunchTimeout) return fail(GBIVF_ERR_TIMEOUT, "tensor-core assignment: a bounded wait ran out");
    CK(e);
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_pq_train(const float* d_r, int64_t n, int d, int m, int niter, uint64_t seed, float* d_pq, void* stream) {
    if (!d_r || !d_pq || n <= 0 || m <= 0 || d % m) return fail(GBIVF_ERR_INVALID, "bad PQ training arguments");
    const int ds = d / m;
    if (ds != 8 && ds != 16 && ds != 32) return fail(GBIVF_ERR_UNSUPPORTED, "sub-vector length %d (8, 16, 32)", ds);
    CK(pq_train_rows(d_r, n, d, m, niter, seed, d_pq, (cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_pq_error(const float* d_x, int64_t n, int d, const int32_t* d_coarse, const float* d_coa, int m,
                   const float* d_pq, const uint8_t* d_codes, float* d_out, void* stream) {
    if (!d_x || !d_pq || !d_codes || !d_out || n < 0 || m <= 0 || d % m || (d_coarse && !d_coa))
        return fail(GBIVF_ERR_INVALID, "bad PQ error arguments");
    CK(pq_error_rows(d_x, n, d, d_coarse, d_coa, m, d_pq, d_codes, d_out, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return GBIVF_OK;
}

int gbivf_selftest_wait_timeout(int device, int* timed_out, float* stalled_ms, int* clean_ok) {
    if (!timed_out || !stalled_ms || !clean_ok) return fail(GBIVF_ERR_INVALID, "NULL output");
    *timed_out = 0;
    *stalled_ms = 0.0f;
    *clean_ok = 0;
    DeviceGuard g(device);
    if (!g.ok) return fail(GBIVF_ERR_INVALID, "device %d", device);
    // one CTA of the persistent tensor-core product: 256 zero queries x 128 zero centroids
    const int nq = 256, C = 128;
    struct Bufs {
        void* p[6] = {};
        cudaStream_t st = nullptr;
        cudaEvent_t e[2] = {};
        ~Bufs() {
            for (void* x : p) if (x) cudaFree(x);
            for (cudaEvent_t x : e) if (x) cudaEventDestroy(x);
            if (st) cudaStreamDestroy(st);
        }
    } b;
    const size_t bytes[6] = {coarse_gemm_qtile_bytes(nq), (size_t)C * 128 * 2 * 2, sizeof(double) * nq,
                             sizeof(float) * C, sizeof(float) * nq * C, sizeof(int)};
    for (int i = 0; i < 6; i++) {
        CK(cudaMalloc(&b.p[i], bytes[i]));
        CK(cudaMemset(b.p[i], 0, bytes[i]));
    }
    CK(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b.e[0]));
    CK(cudaEventCreate(&b.e[1]));
    int* d_err = static_cast<int*>(b.p[5]);
    auto run = [&](bool stall, int* h_err) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), b.st);
        if (e == cudaSuccess) e = cudaEventRecord(b.e[0], b.st);
        if (e == cudaSuccess)
            e = launch_coarse_gemm_store(static_cast<uint8_t*>(b.p[0]), static_cast<uint8_t*>(b.p[1]), nq, C,
                                         static_cast<double*>(b.p[2]), static_cast<float*>(b.p[3]),
                                         static_cast<float*>(b.p[4]), C, 1, d_err, b.st, stall);
        if (e == cudaSuccess) e = cudaEventRecord(b.e[1], b.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, b.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b.st);
        return e;
    };
    int h_err = 0;
    CK(run(true, &h_err));
    *timed_out = h_err != 0;
    CK(cudaEventElapsedTime(stalled_ms, b.e[0], b.e[1]));
    // the context must still run work: the same product without the stall
    h_err = 1;
    CK(run(false, &h_err));
    *clean_ok = h_err == 0;
    return GBIVF_OK;
}

int gbivf_pq_encode(const float* d_x, int64_t n, int d, const int32_t* d_coarse, const float* d_coa, int m,
                    const float* d_pq, uint8_t* d_codes, void* stream) {
    if (!d_x || !d_pq || !d_codes || n < 0 || m <= 0 || d % m || (d_coarse && !d_coa))
        return fail(GBIVF_ERR_INVALID, "bad PQ encode arguments");
    const int ds = d / m;
    if (ds != 8 && ds != 16 && ds != 32) return fail(GBIVF_ERR_UNSUPPORTED, "sub-vector length %d (8, 16, 32)", ds);
    if (n == 0) return GBIVF_OK;
    CK(pq_encode_rows(d_x, n, d, d_coarse, d_coa, m, d_pq, d_codes, (cudaStream_t)stream));
    return GBIVF_OK;
}

}  // extern "C"
