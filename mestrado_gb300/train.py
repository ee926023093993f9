"""Index training and filling for benchmark inputs (host side, numpy).

Produces the same kind of index as the reference's ``ivfpq_new`` +
``ivfpq_assign`` (sequential/ivf_pq/ivf_new.cpp:4-33,
sequential/ivf_pq/ivf_assign.cpp:3-52):

1. coarse k-means on the training set (C centroids);
2. residuals of the training set to their nearest coarse centroid;
3. one k-means of ks=256 centroids per sub-space of the residuals (the PQ);
4. base vectors: nearest coarse centroid, residual, PQ code per sub-space;
5. lists bucketed by coarse centroid, ids ascending inside each list (the
   reference sorts by list with a stable index sort, sorting.c:254-258).

Lloyd iterations in float32 with float64 centroid sums; the reference's
k-means++ initialisation and exact iteration count are not reproduced (the
search engine is checked on indexes built by the reference itself; this
trainer only makes benchmark-sized indexes).
"""
from __future__ import annotations

import numpy as np

from .ivfdata import IVFPQData


def _nearest(x: np.ndarray, cent: np.ndarray, chunk: int = 1 << 15) -> np.ndarray:
    cn = (cent.astype(np.float32) ** 2).sum(1)
    out = np.empty(len(x), np.int64)
    ct = np.ascontiguousarray(cent.T, np.float32)
    for s in range(0, len(x), chunk):
        xc = x[s:s + chunk]
        d = cn[None, :] - 2.0 * (xc @ ct)
        out[s:s + chunk] = d.argmin(1)
    return out


def kmeans(x: np.ndarray, k: int, niter: int = 20, seed: int = 0) -> np.ndarray:
    """Lloyd's k-means; empty clusters are re-seeded from random points."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    rng = np.random.default_rng(seed)
    cent = x[rng.choice(n, size=k, replace=n < k)].copy()
    for _ in range(niter):
        a = _nearest(x, cent)
        order = np.argsort(a, kind="stable")
        counts = np.bincount(a, minlength=k)
        nz = np.nonzero(counts)[0]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])[nz]
        sums = np.add.reduceat(x[order].astype(np.float64), starts, axis=0)
        cent[nz] = (sums / counts[nz, None]).astype(np.float32)
        empty = np.nonzero(counts == 0)[0]
        if len(empty):
            cent[empty] = x[rng.choice(n, size=len(empty), replace=False)]
    return cent


def train_ivfpq(train: np.ndarray, coarsek: int, nsq: int, ks: int = 256, niter: int = 20,
                seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Coarse centroids (C x d) and PQ centroids (nsq x ks x ds)."""
    train = np.ascontiguousarray(train, np.float32)
    d = train.shape[1]
    if d % nsq:
        raise ValueError("d must be a multiple of nsq")
    ds = d // nsq
    coa = kmeans(train, coarsek, niter, seed)
    res = train - coa[_nearest(train, coa)]
    pq = np.empty((nsq, ks, ds), np.float32)
    for s in range(nsq):
        pq[s] = kmeans(res[:, s * ds:(s + 1) * ds], ks, niter, seed + 1 + s)
    return coa, pq


def encode(base: np.ndarray, coa: np.ndarray, pq: np.ndarray, chunk: int = 1 << 18):
    """(list assignment, uint8 codes) of base vectors."""
    nsq, ks, ds = pq.shape
    assign = np.empty(len(base), np.int64)
    codes = np.empty((len(base), nsq), np.uint8)
    for s0 in range(0, len(base), chunk):
        x = np.ascontiguousarray(base[s0:s0 + chunk], np.float32)
        a = _nearest(x, coa)
        r = x - coa[a]
        assign[s0:s0 + len(x)] = a
        for s in range(nsq):
            codes[s0:s0 + len(x), s] = _nearest(np.ascontiguousarray(r[:, s * ds:(s + 1) * ds]), pq[s])
    return assign, codes


def bucket(assign: np.ndarray, codes: np.ndarray, coarsek: int, ids: np.ndarray | None = None):
    """Lists in coarse-centroid order, ids ascending inside each list."""
    if ids is None:
        ids = np.arange(len(assign), dtype=np.int32)
    order = np.argsort(assign, kind="stable")
    counts = np.bincount(assign, minlength=coarsek)
    off = np.zeros(coarsek + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    return off, ids[order].astype(np.int32), codes[order]


def build_index(train: np.ndarray, base: np.ndarray, coarsek: int, nsq: int, niter: int = 20,
                seed: int = 0) -> IVFPQData:
    coa, pq = train_ivfpq(train, coarsek, nsq, niter=niter, seed=seed)
    assign, codes = encode(base, coa, pq)
    off, ids, codes = bucket(assign, codes, coarsek)
    out = IVFPQData(coa=coa, pq=pq, list_off=off, ids=ids, codes=np.ascontiguousarray(codes))
    out.validate()
    return out
