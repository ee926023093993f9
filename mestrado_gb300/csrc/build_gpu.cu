// Index building on the GPU: synthetic mixture generation, k-means for the
// coarse quantizer and the sub-quantizers, assignment and PQ encoding.
//
// The reference trains with yael's k-means (sequential/yael_needs/kmeans.c:
// 209-443: Lloyd iterations, float centroid sums) and encodes with exact 1-NN
// (sequential/ivf_pq/ivf_assign.cpp:3-52, pq-utils/pq_assign.cpp:12-53), all
// single-threaded; at 10M-1B base vectors that is days of CPU. Here:
//   * assignment to d = 128 centroids runs on the tensor cores (the split-BF16
//     tcgen05 GEMM of coarse_mma.cu, argmin fused into its epilogue, then a
//     reduction over centroid tiles); smaller dimensions (sub-quantizer
//     spaces) use a SIMT kernel with the centroids staged in shared memory;
//   * centroid sums accumulate in FP64 (atomicAdd on doubles), then divide;
//     an empty cluster is re-seeded with a pseudo-random point;
//   * the generator is counter-based (a 64-bit mix of seed, stream, row and
//     dimension), so any chunk of a data set can be regenerated on its own.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace gbivf {

__device__ __host__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t hash4(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    return mix64(a ^ mix64(b ^ mix64(c ^ mix64(d))));
}

// ---------------------------------------------------------------------------
// mixture generator: x = clip(round(mean[comp] + sigma * N(0,1)), 0, 255)
// ---------------------------------------------------------------------------

__global__ void gen_components_kernel(int32_t* comp, int64_t row0, int64_t n, int ncomp, const double* cdf,
                                      uint64_t seed, uint64_t stream) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t h = hash4(seed, stream, 0xC0FFEEull, (uint64_t)(row0 + i));
    if (!cdf) {
        comp[i] = (int32_t)(h % (uint64_t)ncomp);
        return;
    }
    const double u = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    int lo = 0, hi = ncomp - 1;  // first c with cdf[c] > u
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] > u) hi = mid;
        else lo = mid + 1;
    }
    comp[i] = lo;
}

__global__ void gen_values_kernel(float* out, const int32_t* comp, int64_t row0, int64_t n, int d,
                                  const float* means, float sigma, uint64_t seed, uint64_t stream) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int pairs = d / 2;
    if (t >= n * pairs) return;
    const int64_t i = t / pairs;
    const int j = (int)(t % pairs);
    const uint64_t h = hash4(seed, stream, (uint64_t)(row0 + i), (uint64_t)j);
    const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = ((float)((h >> 16) & 0xFFFFFF) + 0.5f) * (1.0f / 16777216.0f);
    const float rad = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    const float* mu = means + (int64_t)comp[i] * d;
    const float a = fminf(fmaxf(rintf(mu[2 * j] + sigma * rad * cs), 0.0f), 255.0f);
    const float b = fminf(fmaxf(rintf(mu[2 * j + 1] + sigma * rad * sn), 0.0f), 255.0f);
    out[i * d + 2 * j] = a;
    out[i * d + 2 * j + 1] = b;
}

// ---------------------------------------------------------------------------
// assignment
// ---------------------------------------------------------------------------

// per row: the smallest key over the centroid tiles
__global__ void argmin_reduce_kernel(const u64* partial, int64_t n, int tiles, int32_t* assign) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 b = KEY_MAX;
    for (int t = 0; t < tiles; t++) b = min(b, partial[i * tiles + t]);
    assign[i] = (int32_t)key_payload(b);
}

// SIMT nearest centroid for small dimensions: rows of x with stride ld, d <= 32;
// centroids (k x d) staged in shared memory in chunks
constexpr int AS_NT = 256, AS_CHUNK = 256;

template <int D>
__global__ void __launch_bounds__(AS_NT) assign_simt_kernel(const float* __restrict__ x, int64_t n, int64_t ld,
                                                            const float* __restrict__ cent, int k,
                                                            int32_t* __restrict__ assign) {
    __shared__ float sc[AS_CHUNK * D];
    __shared__ float sn[AS_CHUNK];
    const int64_t i = (int64_t)blockIdx.x * AS_NT + threadIdx.x;
    float v[D];
#pragma unroll
    for (int l = 0; l < D; l++) v[l] = i < n ? x[i * ld + l] : 0.0f;
    float best = INFINITY;
    int bi = 0;
    for (int c0 = 0; c0 < k; c0 += AS_CHUNK) {
        const int cn = min(AS_CHUNK, k - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < cn * D; e += AS_NT) sc[e] = cent[(int64_t)c0 * D + e];
        __syncthreads();
        for (int c = threadIdx.x; c < cn; c += AS_NT) {
            float s = 0.0f;
#pragma unroll
            for (int l = 0; l < D; l++) s += sc[c * D + l] * sc[c * D + l];
            sn[c] = s;
        }
        __syncthreads();
        for (int c = 0; c < cn; c++) {
            float dot = 0.0f;
#pragma unroll
            for (int l = 0; l < D; l++) dot += v[l] * sc[c * D + l];
            const float dist = sn[c] - 2.0f * dot;
            if (dist < best) {
                best = dist;
                bi = c0 + c;
            }
        }
    }
    if (i < n) assign[i] = bi;
}

// ---------------------------------------------------------------------------
// centroid update in FP64
// ---------------------------------------------------------------------------

__global__ void kmeans_accum_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int d,
                                    const int32_t* __restrict__ assign, double* __restrict__ sums,
                                    int* __restrict__ counts) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * d) return;
    const int64_t i = t / d;
    const int l = (int)(t % d);
    const int a = assign[i];
    atomicAdd(&sums[(int64_t)a * d + l], (double)x[i * ld + l]);
    if (l == 0) atomicAdd(&counts[a], 1);
}

__global__ void kmeans_finalize_kernel(const double* __restrict__ sums, const int* __restrict__ counts, int k, int d,
                                       float* __restrict__ cent, const float* __restrict__ x, int64_t n, int64_t ld,
                                       uint64_t seed, int iter) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * d) return;
    const int c = (int)(t / d), l = (int)(t % d);
    if (counts[c] > 0) {
        cent[t] = (float)(sums[t] / (double)counts[c]);
    } else {  // empty cluster: re-seed with a pseudo-random point
        const int64_t r = (int64_t)(hash4(seed, 0xE317ull, (uint64_t)iter, (uint64_t)c) % (uint64_t)n);
        cent[t] = x[r * ld + l];
    }
}

__global__ void init_centroids_kernel(const float* __restrict__ x, int64_t n, int64_t ld, int d, int k, uint64_t seed,
                                      float* __restrict__ cent) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * d) return;
    const int c = (int)(t / d), l = (int)(t % d);
    // one pseudo-random point from each of k equal slices of the data
    const uint64_t slice = n >= k ? (uint64_t)(n / k) : 0;
    const uint64_t h = hash4(seed, 0x1D17ull, (uint64_t)c, 0);
    const int64_t r = slice ? (int64_t)((uint64_t)c * slice + h % slice) : (int64_t)(h % (uint64_t)n);
    cent[t] = x[r * ld + l];
}

// residual of a row to its coarse centroid
__global__ void residual_kernel(const float* __restrict__ x, int64_t n, int d, const int32_t* __restrict__ assign,
                                const float* __restrict__ coa, float* __restrict__ r) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * d) return;
    const int64_t i = t / d;
    const int l = (int)(t % d);
    r[t] = x[t] - coa[(int64_t)assign[i] * d + l];
}

// e = x - coa[assign] - c1(codes): the residual error a refinement quantizer encodes
__global__ void pq_error_kernel(const float* __restrict__ x, int64_t n, int d, const int32_t* __restrict__ assign,
                                const float* __restrict__ coa, int m, const float* __restrict__ pq,
                                const uint8_t* __restrict__ codes, float* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * d) return;
    const int64_t i = t / d;
    const int l = (int)(t % d), ds = d / m, s = l / ds;
    const float y = assign ? coa[(int64_t)assign[i] * d + l] : 0.0f;
    out[t] = x[t] - y - pq[((int64_t)s * 256 + codes[i * m + s]) * ds + (l - s * ds)];
}

__global__ void store_codes_kernel(const int32_t* __restrict__ a, int64_t n, int m, int s, uint8_t* __restrict__ codes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) codes[i * m + s] = (uint8_t)a[i];
}

inline unsigned blocks(int64_t work, int nt) { return (unsigned)((work + nt - 1) / nt); }

// nearest centroid for every row: tensor cores for d = 128, SIMT for d <= 32
cudaError_t assign_rows(const float* x, int64_t n, int64_t ld, int d, const float* cent, int k, int32_t* assign,
                        cudaStream_t st, bool hi_only) {
    cudaError_t e = cudaSuccess;
    if (d == 128 && ld == 128) {
        // the persistent tcgen05 GEMM with the argmin epilogue, blocks of up to 2^20 rows
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 1;
        const int64_t bq = std::min<int64_t>(n, 1 << 20), tail = n % bq;
        // partial-result slots for the largest need among the two block sizes used
        size_t slots = (size_t)bq * 2 * coarse_gemm_nsplit((int)bq, k, sms, nullptr);
        if (tail) slots = std::max(slots, (size_t)tail * 2 * coarse_gemm_nsplit((int)tail, k, sms, nullptr));
        void *ctiles = nullptr, *cnorm = nullptr, *qtiles = nullptr, *part = nullptr, *err = nullptr;
        auto cleanup = [&]() {
            for (void* p : {ctiles, cnorm, qtiles, part, err})
                if (p) cudaFree(p);
        };
        const size_t qtb = coarse_gemm_qtile_bytes((int)bq);
        if ((e = cudaMalloc(&ctiles, coarse_mma_tile_bytes(k, true))) != cudaSuccess ||
            (e = cudaMalloc(&cnorm, sizeof(float) * k)) != cudaSuccess ||
            (e = cudaMalloc(&qtiles, qtb)) != cudaSuccess ||
            (e = cudaMalloc(&part, sizeof(u64) * slots)) != cudaSuccess ||
            (e = cudaMalloc(&err, sizeof(int))) != cudaSuccess) {
            cleanup();
            return e;
        }
        e = cudaMemsetAsync(err, 0, sizeof(int), st);
        if (e == cudaSuccess) e = launch_bf16_split_tiles(cent, k, (uint8_t*)ctiles, st);
        if (e == cudaSuccess) e = launch_norm_f(cent, k, d, (float*)cnorm, st);
        for (int64_t r0 = 0; r0 < n && e == cudaSuccess; r0 += bq) {
            const int nb = (int)std::min<int64_t>(bq, n - r0);
            const int ns = coarse_gemm_nsplit(nb, k, sms, nullptr);
            e = launch_bf16_tiles(x + r0 * d, nb, MMA_QUERY_TILE, (uint8_t*)qtiles, st);
            const size_t written = coarse_mma_tile_bytes(nb, false), total = coarse_gemm_qtile_bytes(nb);
            if (e == cudaSuccess && total > written)
                e = cudaMemsetAsync((uint8_t*)qtiles + written, 0, total - written, st);
            if (e == cudaSuccess)
                e = launch_coarse_gemm_argmin((uint8_t*)qtiles, (uint8_t*)ctiles, nb, k, (float*)cnorm, (u64*)part,
                                              sms, (int*)err, st, hi_only);
            if (e == cudaSuccess) {
                argmin_reduce_kernel<<<blocks(nb, 256), 256, 0, st>>>((u64*)part, nb, 2 * ns, assign + r0);
                e = cudaGetLastError();
            }
        }
        int herr = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cleanup();
        if (e == cudaSuccess && herr) e = cudaErrorLaunchTimeout;
        return e;
    }
    switch (d) {
        case 8: assign_simt_kernel<8><<<blocks(n, AS_NT), AS_NT, 0, st>>>(x, n, ld, cent, k, assign); break;
        case 16: assign_simt_kernel<16><<<blocks(n, AS_NT), AS_NT, 0, st>>>(x, n, ld, cent, k, assign); break;
        case 32: assign_simt_kernel<32><<<blocks(n, AS_NT), AS_NT, 0, st>>>(x, n, ld, cent, k, assign); break;
        default: return cudaErrorNotSupported;
    }
    return cudaGetLastError();
}

cudaError_t kmeans_rows(const float* x, int64_t n, int64_t ld, int d, int k, int niter, uint64_t seed, float* cent,
                        cudaStream_t st) {
    void *assign = nullptr, *sums = nullptr, *counts = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&assign, sizeof(int32_t) * n)) != cudaSuccess ||
        (e = cudaMalloc(&sums, sizeof(double) * k * d)) != cudaSuccess ||
        (e = cudaMalloc(&counts, sizeof(int) * k)) != cudaSuccess) {
        for (void* p : {assign, sums, counts})
            if (p) cudaFree(p);
        return e;
    }
    init_centroids_kernel<<<blocks((int64_t)k * d, 256), 256, 0, st>>>(x, n, ld, d, k, seed, cent);
    e = cudaGetLastError();
    for (int it = 0; it < niter && e == cudaSuccess; it++) {
        e = assign_rows(x, n, ld, d, cent, k, (int32_t*)assign, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(sums, 0, sizeof(double) * k * d, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * k, st);
        if (e == cudaSuccess) {
            kmeans_accum_kernel<<<blocks(n * d, 256), 256, 0, st>>>(x, n, ld, d, (int32_t*)assign, (double*)sums,
                                                                      (int*)counts);
            kmeans_finalize_kernel<<<blocks((int64_t)k * d, 256), 256, 0, st>>>((double*)sums, (int*)counts, k, d, cent,
                                                                                 x, n, ld, seed, it);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (void* p : {assign, sums, counts}) cudaFree(p);
    return e;
}

cudaError_t gen_mixture(float* out, int64_t n, int d, const float* means, int ncomp, const double* cdf, float sigma,
                        uint64_t seed, uint64_t stream_id, int64_t row0, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (d % 2) return cudaErrorInvalidValue;
    void* comp = nullptr;
    cudaError_t e = cudaMalloc(&comp, sizeof(int32_t) * n);
    if (e != cudaSuccess) return e;
    gen_components_kernel<<<blocks(n, 256), 256, 0, st>>>((int32_t*)comp, row0, n, ncomp, cdf, seed, stream_id);
    gen_values_kernel<<<blocks(n * (d / 2), 256), 256, 0, st>>>(out, (int32_t*)comp, row0, n, d, means, sigma, seed,
                                                                 stream_id);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(comp);
    return e;
}

cudaError_t pq_train_rows(const float* r, int64_t n, int d, int m, int niter, uint64_t seed, float* pq,
                          cudaStream_t st) {
    const int ds = d / m;
    for (int s = 0; s < m; s++) {
        cudaError_t e = kmeans_rows(r + s * ds, n, d, ds, 256, niter, seed + 1 + s, pq + (int64_t)s * 256 * ds, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t pq_encode_rows(const float* x, int64_t n, int d, const int32_t* coarse, const float* coa, int m,
                           const float* pq, uint8_t* codes, cudaStream_t st) {
    const int ds = d / m;
    const int64_t chunk = std::min<int64_t>(n, 1 << 22);
    void *res = nullptr, *a = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&res, sizeof(float) * chunk * d)) != cudaSuccess ||
        (e = cudaMalloc(&a, sizeof(int32_t) * chunk)) != cudaSuccess) {
        if (res) cudaFree(res);
        return e;
    }
    for (int64_t r0 = 0; r0 < n && e == cudaSuccess; r0 += chunk) {
        const int64_t nb = std::min(chunk, n - r0);
        const float* src = x + r0 * d;
        if (coarse) {
            residual_kernel<<<blocks(nb * d, 256), 256, 0, st>>>(src, nb, d, coarse + r0, coa, (float*)res);
            e = cudaGetLastError();
            src = (const float*)res;
        }
        for (int s = 0; s < m && e == cudaSuccess; s++) {
            e = assign_rows(src + s * ds, nb, d, ds, pq + (int64_t)s * 256 * ds, 256, (int32_t*)a, st);
            if (e == cudaSuccess) {
                store_codes_kernel<<<blocks(nb, 256), 256, 0, st>>>((int32_t*)a, nb, m, s, codes + r0 * m);
                e = cudaGetLastError();
            }
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(res);
    cudaFree(a);
    return e;
}

cudaError_t pq_error_rows(const float* x, int64_t n, int d, const int32_t* coarse, const float* coa, int m,
                          const float* pq, const uint8_t* codes, float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    pq_error_kernel<<<blocks(n * d, 256), 256, 0, st>>>(x, n, d, coarse, coa, m, pq, codes, out);
    return cudaGetLastError();
}

}  // namespace gbivf
