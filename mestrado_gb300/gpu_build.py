"""Build large IVF-PQ indexes on the GPU, through the engine's C ABI.

The reference trains and encodes on one CPU thread (ivfpq_new + ivfpq_assign,
sequential/ivf_test.cpp:52-59); at 10M+ base vectors that is impractical, so
this driver runs every step on the GPU:

1. mixture data (gbivf_generate_mixture: counter-based, chunked);
2. coarse k-means (gbivf_kmeans: tensor-core assignment, FP64 centroid sums);
3. residuals of the training set, then m sub-quantizer k-means (gbivf_pq_train);
4. base vectors: nearest coarse centroid (gbivf_assign), PQ codes of the
   residuals (gbivf_pq_encode);
5. lists bucketed by coarse centroid with ids ascending (stable sort on the
   host, as the reference's ivec_sort_index orders them);
6. optionally, refinement codes: a second product quantizer trained on and
   encoding the residual errors x - y_list - c1(codes) (gbivf_pq_error).

Device buffers are torch tensors (memory only); all compute is the engine's.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .ivfdata import IVFPQData
from .synth import Mixture


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def zipf_cdf(ncomp: int, s: float) -> np.ndarray:
    w = 1.0 / np.arange(1, ncomp + 1, dtype=np.float64) ** s
    c = np.cumsum(w)
    return c / c[-1]


class GpuMixture:
    """A Mixture whose vectors are generated on the GPU in chunks."""

    def __init__(self, mx: Mixture, device="cuda"):
        import torch

        self.mx = mx
        self.lib = _lib.load()
        self.means = torch.from_numpy(mx.means()).to(device)
        self.cdf = torch.from_numpy(zipf_cdf(mx.ncomp, mx.zipf)).to(device) if mx.zipf else None
        self.device = device

    def generate(self, n: int, stream_id: int, row0: int = 0, out=None, chunk: int = 1 << 24):
        import torch

        d = self.mx.d
        if out is None:
            out = torch.empty((n, d), dtype=torch.float32, device=self.device)
        s = torch.cuda.current_stream().cuda_stream
        for r in range(0, n, chunk):
            nb = min(chunk, n - r)
            check(self.lib.gbivf_generate_mixture(
                C.c_void_p(out.data_ptr() + r * d * 4), nb, d, _ptr(self.means), self.mx.ncomp,
                _ptr(self.cdf) if self.cdf is not None else C.c_void_p(0), float(self.mx.sigma),
                self.mx.seed, stream_id, row0 + r, C.c_void_p(s)))
        return out


def train_quantizers(train, coarsek: int, m: int, niter: int = 10, seed: int = 0):
    """(coarse centroids, pq centroids) as device tensors."""
    import torch

    lib = _lib.load()
    n, d = train.shape
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    coa = torch.empty((coarsek, d), dtype=torch.float32, device=train.device)
    check(lib.gbivf_kmeans(_ptr(train), n, d, coarsek, niter, seed, _ptr(coa), s))
    assign = torch.empty(n, dtype=torch.int32, device=train.device)
    check(lib.gbivf_assign(_ptr(train), n, d, _ptr(coa), coarsek, _ptr(assign), s))
    res = train - coa[assign.long()]
    pq = torch.empty((m, 256, d // m), dtype=torch.float32, device=train.device)
    check(lib.gbivf_pq_train(_ptr(res), n, d, m, niter, seed + 1, _ptr(pq), s))
    return coa, pq


def encode_base(base, coa, pq, chunk: int = 1 << 24):
    """(coarse assignment, codes) of the base set, device tensors."""
    import torch

    lib = _lib.load()
    n, d = base.shape
    m = pq.shape[0]
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assign = torch.empty(n, dtype=torch.int32, device=base.device)
    codes = torch.empty((n, m), dtype=torch.uint8, device=base.device)
    for r in range(0, n, chunk):
        nb = min(chunk, n - r)
        xb = base[r:r + nb]
        ab = assign[r:r + nb]
        check(lib.gbivf_assign(_ptr(xb), nb, d, _ptr(coa), coa.shape[0], _ptr(ab), s))
        check(lib.gbivf_pq_encode(_ptr(xb), nb, d, _ptr(ab), _ptr(coa), m, _ptr(pq), _ptr(codes[r:r + nb]), s))
    return assign, codes


def residual_error(x, assign, coa, pq, codes):
    """x - coa[assign] - c1(codes) on the GPU (the refinement quantizer's input)."""
    import torch

    lib = _lib.load()
    n, d = x.shape
    out = torch.empty_like(x)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(lib.gbivf_pq_error(_ptr(x), n, d, _ptr(assign), _ptr(coa), pq.shape[0], _ptr(pq), _ptr(codes), _ptr(out), s))
    return out


def train_refine(train, coa, pq, m2: int, niter: int = 10, seed: int = 0):
    """Refinement codebook (m2 x 256 x d/m2) trained on the residual errors of
    the training set (a second product quantizer; no counterpart in the reference)."""
    import torch

    lib = _lib.load()
    assign, codes = encode_base(train, coa, pq)
    err = residual_error(train, assign, coa, pq, codes)
    n, d = train.shape
    pq2 = torch.empty((m2, 256, d // m2), dtype=torch.float32, device=train.device)
    check(lib.gbivf_pq_train(_ptr(err), n, d, m2, niter, seed + 7, _ptr(pq2),
                             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return pq2


def encode_refine(base, assign, codes, coa, pq, pq2, chunk: int = 1 << 22):
    """Refinement codes of the base set (n x m2 uint8, device)."""
    import torch

    lib = _lib.load()
    n, d = base.shape
    m2 = pq2.shape[0]
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    codes2 = torch.empty((n, m2), dtype=torch.uint8, device=base.device)
    for r in range(0, n, chunk):
        nb = min(chunk, n - r)
        err = residual_error(base[r:r + nb], assign[r:r + nb], coa, pq, codes[r:r + nb])
        check(lib.gbivf_pq_encode(_ptr(err), nb, d, C.c_void_p(0), C.c_void_p(0), m2, _ptr(pq2),
                                  _ptr(codes2[r:r + nb]), s))
    return codes2


def bucket(assign: np.ndarray, codes: np.ndarray, coarsek: int, codes2: np.ndarray | None = None):
    order = np.argsort(assign, kind="stable")
    counts = np.bincount(assign, minlength=coarsek)
    off = np.zeros(coarsek + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    c2 = None if codes2 is None else np.ascontiguousarray(codes2[order])
    return off, order.astype(np.int32), np.ascontiguousarray(codes[order]), c2


def build_index_gpu(base, train, coarsek: int, m: int, niter: int = 10, seed: int = 0, m2: int = 0) -> IVFPQData:
    """An index built on the GPU; with m2 > 0 also m2 x 256 refinement codes."""
    coa, pq = train_quantizers(train, coarsek, m, niter, seed)
    assign, codes = encode_base(base, coa, pq)
    pq2 = codes2 = None
    if m2:
        pq2 = train_refine(train, coa, pq, m2, niter, seed)
        codes2 = encode_refine(base, assign, codes, coa, pq, pq2)
    off, ids, codes_h, codes2_h = bucket(assign.cpu().numpy(), codes.cpu().numpy(), coarsek,
                                         None if codes2 is None else codes2.cpu().numpy())
    out = IVFPQData(coa=coa.cpu().numpy(), pq=pq.cpu().numpy(), list_off=off, ids=ids, codes=codes_h,
                    pq2=None if pq2 is None else pq2.cpu().numpy(), codes2=codes2_h)
    out.validate()
    return out


def build_index_streaming(gm: GpuMixture, nbase: int, train, coarsek: int, m: int, m2: int = 0, niter: int = 10,
                          seed: int = 0, chunk: int = 1 << 24, bf16_assign: bool = True, log=None):
    """An index over a generated base too large to hold in memory (1B x 128
    floats is 512 GB): chunks of the base are generated, assigned, PQ-encoded
    and refinement-encoded on the fly; the lists are bucketed on the GPU (a
    stable sort by list) and the index is created from those device arrays.
    Returns (GpuIndex, list_off)."""
    import time

    import torch

    from .engine import GpuIndex

    lib = _lib.load()
    dev = train.device
    d = train.shape[1]
    t0 = time.time()
    coa, pq = train_quantizers(train, coarsek, m, niter, seed)
    pq2 = train_refine(train, coa, pq, m2, niter, seed) if m2 else None
    torch.cuda.synchronize()
    if log:
        log(f"quantizers trained in {time.time() - t0:.1f}s")
    assign = torch.empty(nbase, dtype=torch.int32, device=dev)
    codes = torch.empty((nbase, m), dtype=torch.uint8, device=dev)
    codes2 = torch.empty((nbase, m2), dtype=torch.uint8, device=dev) if m2 else None
    buf = torch.empty((min(chunk, nbase), d), dtype=torch.float32, device=dev)
    err = torch.empty_like(buf) if m2 else None
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    t1 = time.time()
    for r in range(0, nbase, chunk):
        nb = min(chunk, nbase - r)
        x = gm.generate(nb, stream_id=1, row0=r, out=buf[:nb])
        a = assign[r:r + nb]
        check(lib.gbivf_assign_flags(_ptr(x), nb, d, _ptr(coa), coarsek, _ptr(a), 1 if bf16_assign else 0, s))
        check(lib.gbivf_pq_encode(_ptr(x), nb, d, _ptr(a), _ptr(coa), m, _ptr(pq), _ptr(codes[r:r + nb]), s))
        if m2:
            e = err[:nb]
            check(lib.gbivf_pq_error(_ptr(x), nb, d, _ptr(a), _ptr(coa), m, _ptr(pq), _ptr(codes[r:r + nb]),
                                     _ptr(e), s))
            check(lib.gbivf_pq_encode(_ptr(e), nb, d, C.c_void_p(0), C.c_void_p(0), m2, _ptr(pq2),
                                      _ptr(codes2[r:r + nb]), s))
    del buf, err
    torch.cuda.synchronize()
    if log:
        log(f"{nbase:,} vectors generated, assigned and encoded in {time.time() - t1:.1f}s")
    order = torch.sort(assign, stable=True).indices
    counts = torch.bincount(assign, minlength=coarsek).cpu().numpy()
    off = np.zeros(coarsek + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    del assign
    ids = order.to(torch.int32)
    codes_s = codes[order]
    del codes
    codes2_s = codes2[order] if m2 else None
    del codes2, order
    torch.cuda.empty_cache()
    gi = GpuIndex.from_device(coa.cpu().numpy(), pq.cpu().numpy(), off, ids, codes_s,
                              None if pq2 is None else pq2.cpu().numpy(), codes2_s, device=dev.index or 0)
    del ids, codes_s, codes2_s
    torch.cuda.empty_cache()
    if log:
        log(f"index created in {time.time() - t0:.1f}s in all")
    return gi, off


def exact_topk_streaming(gm: GpuMixture, nbase: int, queries, k: int, chunk: int = 1 << 24):
    """Brute-force top-k over a generated base, chunk by chunk (evaluation only;
    exact in FP32 for byte-valued vectors, as exact_topk)."""
    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    nq, d = queries.shape
    dev = queries.device
    qn = (queries * queries).sum(1, keepdim=True)
    best_d = torch.full((nq, k), float("inf"), device=dev)
    best_i = torch.full((nq, k), -1, dtype=torch.int64, device=dev)
    buf = torch.empty((min(chunk, nbase), d), dtype=torch.float32, device=dev)
    for r in range(0, nbase, chunk):
        nb = min(chunk, nbase - r)
        x = gm.generate(nb, stream_id=1, row0=r, out=buf[:nb])
        dist = qn + (x * x).sum(1)[None, :] - 2.0 * (queries @ x.T)
        vd, vi = torch.topk(dist, min(k, nb), dim=1, largest=False)
        cd = torch.cat([best_d, vd], 1)
        ci = torch.cat([best_i, vi + r], 1)
        sel = torch.topk(cd, k, dim=1, largest=False).indices
        best_d, best_i = torch.gather(cd, 1, sel), torch.gather(ci, 1, sel)
    return best_i.cpu().numpy()


def exact_topk(base, queries, k: int, batch: int = 256):
    """Brute-force top-k by squared L2 on the GPU. For byte-valued vectors (d <=
    256) every product and partial sum is an integer below 2^24, so FP32 gives
    the exact distances (the same as FP64). Evaluation only."""
    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    bn = torch.empty(base.shape[0], dtype=torch.float32, device=base.device)
    for r in range(0, base.shape[0], 1 << 22):
        blk = base[r:r + (1 << 22)]
        bn[r:r + len(blk)] = (blk * blk).sum(1)
    out = np.empty((queries.shape[0], k), np.int64)
    for s in range(0, queries.shape[0], batch):
        q = queries[s:s + batch]
        dist = (q * q).sum(1, keepdim=True) + bn[None, :] - 2.0 * (q @ base.T)
        out[s:s + len(q)] = torch.topk(dist, k, dim=1, largest=False).indices.cpu().numpy()
    return out
