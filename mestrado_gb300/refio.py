"""The reference's file formats and its recall statistic, on the host.

* TEXMEX vector files (`.fvecs`, `.bvecs`, `.ivecs`): each vector is an int32
  dimension followed by that many float32 / uint8 / int32 values
  (sequential/yael_needs/vector.c:296-414). `.bvecs` are widened to float32
  as `b2fvecs_read` does; an offset in whole blocks of n vectors follows
  `my_bvecs_read` (parallel/pq-utils/pq_test_load_vectors.cpp:275-325).
* The parallel2 index on disk (parallel2/ivf_pq/ivf_training.cpp:93-160,
  parallel2/genivf.cpp:62-86, parallel2/ivf_pq/ivf_search.cpp:293-321):
  `<train>/header` holds 8 int32 (nsq, ks, ds, centroidsn = ks*ds,
  centroidsd = nsq, coarsek, coa_centroidsn = coarsek, coa_centroidsd = d);
  `<train>/pq_centroids` is float32 [nsq][ks][ds]; `<train>/coa_centroids`
  is float32 [coarsek][d]; `<ivf>/<j>` for each list j holds int32 coarsek,
  idstam, ids[idstam], codes.n, codes.d, codes[n*d] (row-major, one code per
  int32).
* R@r as `pq_test_compute_stats` / `pq_test_compute_stats2` print it
  (sequential/pq-utils/pq_test_compute_stats.cpp:3-149): per query the rank
  of its first ground-truth neighbour in the returned list (k+1 when absent),
  then, for r in 1, 2, 5, ..., 10000 with r <= k, the percentage of queries
  whose rank is below r. The ground truth is the first column of the
  `.ivecs` file (pq_test_load_vectors.cpp:157-161).
"""
from __future__ import annotations

import os

import numpy as np

from .ivfdata import IVFPQData

R_AT = (1, 2, 5, 10, 20, 50, 100, 200, 500, 1000, 2000, 5000, 10000)


# ---------------------------------------------------------------------------
# TEXMEX vector files
# ---------------------------------------------------------------------------

def _xvecs_read(path: str, dtype, n: int | None, offset: int) -> np.ndarray:
    item = np.dtype(dtype).itemsize
    with open(path, "rb") as f:
        head = np.fromfile(f, dtype=np.int32, count=1)
        if head.size == 0:
            return np.zeros((0, 0), dtype)
        d = int(head[0])
        if d <= 0:
            raise ValueError(f"{path}: bad vector dimension {d}")
        rec = 4 + d * item
        total = os.path.getsize(path) // rec
        start = offset * (n if n is not None else 0)
        count = total - start if n is None else min(n, max(total - start, 0))
        f.seek(start * rec)
        raw = np.fromfile(f, dtype=np.uint8, count=count * rec)
    raw = raw[: (raw.size // rec) * rec].reshape(-1, rec)
    dims = raw[:, :4].copy().view(np.int32).ravel()
    if np.any(dims != d):
        raise ValueError(f"{path}: unexpected vector dimension (expected {d})")
    return raw[:, 4:].copy().view(dtype).reshape(-1, d)


def read_fvecs(path: str, n: int | None = None) -> np.ndarray:
    """float32 vectors, n x d (all of them when n is None)."""
    return _xvecs_read(path, np.float32, n, 0)


def read_bvecs(path: str, n: int | None = None, offset: int = 0) -> np.ndarray:
    """uint8 vectors widened to float32, n x d; `offset` skips offset*n vectors."""
    return _xvecs_read(path, np.uint8, n, offset).astype(np.float32)


def read_ivecs(path: str, n: int | None = None) -> np.ndarray:
    """int32 vectors, n x d."""
    return _xvecs_read(path, np.int32, n, 0)


def _xvecs_write(path: str, a: np.ndarray, dtype) -> None:
    a = np.ascontiguousarray(a, dtype=dtype)
    n, d = a.shape
    rec = np.empty((n, 4 + d * a.itemsize), np.uint8)
    rec[:, :4] = np.full((n, 1), d, np.int32).view(np.uint8)
    rec[:, 4:] = a.view(np.uint8).reshape(n, -1)
    rec.tofile(path)


def write_fvecs(path: str, a: np.ndarray) -> None:
    _xvecs_write(path, a, np.float32)


def write_bvecs(path: str, a: np.ndarray) -> None:
    _xvecs_write(path, a, np.uint8)


def write_ivecs(path: str, a: np.ndarray) -> None:
    _xvecs_write(path, a, np.int32)


def ground_truth_first(gnd: np.ndarray) -> np.ndarray:
    """The reference keeps only the first ground-truth neighbour per query."""
    return np.ascontiguousarray(np.asarray(gnd)[:, 0], np.int32)


# ---------------------------------------------------------------------------
# R@r
# ---------------------------------------------------------------------------

def r_at(ids: np.ndarray, gnd_first: np.ndarray, k: int, layout: str = "row0") -> dict:
    """{r: percentage} as the reference prints it.

    layout "row0": ids nq x k row-major, 0-based (ivfpq_search output,
    pq_test_compute_stats2); "col1": ids k x nq column-major, 1-based
    (pq_search output, pq_test_compute_stats)."""
    gnd = np.asarray(gnd_first, np.int64)
    nq = gnd.shape[0]
    if layout == "row0":
        m = np.asarray(ids, np.int64).reshape(nq, k)
        hit = m == gnd[:, None]
    elif layout == "col1":
        m = np.asarray(ids, np.int64).reshape(k, nq).T
        hit = m == (gnd[:, None] + 1)
    else:
        raise ValueError(f"layout {layout!r}")
    # the last matching slot wins, as the reference's loop overwrites the rank
    rank = np.where(hit.any(axis=1), k - 1 - np.argmax(hit[:, ::-1], axis=1), k + 1)
    out = {}
    for r in R_AT:
        if r <= k:
            out[r] = float(np.count_nonzero((rank < r) & (rank < k))) / nq * 100.0
    return out


# ---------------------------------------------------------------------------
# parallel2 index files
# ---------------------------------------------------------------------------

def read_parallel2_index(train_dir: str, ivf_dir: str) -> IVFPQData:
    """An index trained and assigned by the reference's parallel2 tools
    (`header`, `pq_centroids`, `coa_centroids`, one file per list)."""
    hdr = np.fromfile(os.path.join(train_dir, "header"), dtype=np.int32)
    if hdr.size != 8:
        raise ValueError(f"{train_dir}/header: expected 8 int32, found {hdr.size}")
    nsq, ks, ds, cn, cd, coarsek, coan, coad = (int(v) for v in hdr)
    if cn != ks * ds or cd != nsq or coan != coarsek:
        raise ValueError(f"inconsistent header {hdr.tolist()}")
    if ks > 256:
        raise ValueError(f"ks = {ks}: codes above 255 cannot be held as bytes")
    pq = np.fromfile(os.path.join(train_dir, "pq_centroids"), dtype=np.float32)
    coa = np.fromfile(os.path.join(train_dir, "coa_centroids"), dtype=np.float32)
    if pq.size != nsq * ks * ds or coa.size != coarsek * coad:
        raise ValueError("centroid files do not match the header")
    sizes, ids, codes = [], [], []
    for j in range(coarsek):
        a = np.fromfile(os.path.join(ivf_dir, str(j)), dtype=np.int32)
        if a.size < 2:
            raise ValueError(f"{ivf_dir}/{j}: truncated")
        n = int(a[1])
        lid = a[2:2 + n]
        cn_, cd_ = int(a[2 + n]), int(a[3 + n])
        if cn_ != n or cd_ != nsq:
            raise ValueError(f"{ivf_dir}/{j}: codes {cn_} x {cd_} for {n} ids and nsq = {nsq}")
        lc = a[4 + n:4 + n + n * nsq]
        if lc.size != n * nsq:
            raise ValueError(f"{ivf_dir}/{j}: truncated codes")
        sizes.append(n)
        ids.append(lid)
        codes.append(lc)
    allc = np.concatenate(codes) if codes else np.zeros(0, np.int32)
    ix = IVFPQData.from_reference_lists(coa.reshape(coarsek, coad), pq.reshape(nsq, ks, ds),
                                        np.array(sizes, np.int64),
                                        np.concatenate(ids) if ids else np.zeros(0, np.int32),
                                        allc.reshape(-1, nsq))
    ix.validate()
    return ix


def write_parallel2_index(ix: IVFPQData, train_dir: str, ivf_dir: str) -> None:
    """The inverse of read_parallel2_index, byte for byte the reference's layout."""
    os.makedirs(train_dir, exist_ok=True)
    os.makedirs(ivf_dir, exist_ok=True)
    m, ks, ds = ix.pq.shape
    C, d = ix.coa.shape
    np.array([m, ks, ds, ks * ds, m, C, C, d], np.int32).tofile(os.path.join(train_dir, "header"))
    np.ascontiguousarray(ix.pq, np.float32).tofile(os.path.join(train_dir, "pq_centroids"))
    np.ascontiguousarray(ix.coa, np.float32).tofile(os.path.join(train_dir, "coa_centroids"))
    for j in range(C):
        b, e = int(ix.list_off[j]), int(ix.list_off[j + 1])
        n = e - b
        parts = [np.array([C, n], np.int32), ix.ids[b:e].astype(np.int32), np.array([n, m], np.int32),
                 ix.codes[b:e].astype(np.int32).ravel()]
        np.concatenate(parts).tofile(os.path.join(ivf_dir, str(j)))
