"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the IVF-PQ search path.

Python bindings for two checkers:

* ``liboracle.so``: the plain-C restatement of rafaelms101/mestrado's
  sequential search (``ivfpq_oracle.c``), used by the tests, the smoke check
  and the benchmark's CPU-baseline leg;
* ``_ref/libref_seq.so`` (only where the reference sources exist): the
  reference's own code, used to pin the restatement and to write the golden
  fixtures.

Nothing in the product (``mestrado_gb300``) imports this package.

An index is any object with the attributes ``d, coarsek, m, ks`` (ints),
``coa`` (C x d float32), ``pq`` (m x ks x ds float32), ``list_off`` (C+1
int64), ``ids`` (n int32) and ``codes`` (n x m uint8).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

TIES_HEAP, TIES_KEYED = 0, 1
TABLE_EXPANSION, TABLE_DIRECT = 0, 1

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class _OrcIndex(C.Structure):
    _fields_ = [
        ("d", C.c_int), ("coarsek", C.c_int), ("m", C.c_int), ("ks", C.c_int),
        ("coa", C.c_void_p), ("pq", C.c_void_p), ("list_off", C.c_void_p),
        ("ids", C.c_void_p), ("codes", C.c_void_p),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = C.CDLL(path)
        _lib.orc_ivfpq_search.restype = C.c_int
        _lib.orc_pq_search.restype = C.c_int
        _lib.orc_core_cpu.restype = C.c_int
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _pin(ix):
    """Keep contiguous copies alive and build the C struct."""
    arrs = (
        _c(ix.coa, np.float32), _c(ix.pq, np.float32), _c(ix.list_off, np.int64),
        _c(ix.ids, np.int32), _c(ix.codes, np.uint8),
    )
    s = _OrcIndex(int(ix.d), int(ix.coarsek), int(ix.m), int(ix.ks),
                  *(a.ctypes.data for a in arrs))
    return s, arrs


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def ivfpq_search(ix, queries, k, w, kl=None, base=None, rerank=True, ties=TIES_HEAP,
                 table_mode=TABLE_EXPANSION, nthreads=1, stages=False):
    """Restated ivfpq_search (sequential/ivf_pq/ivf_search.cpp:9-153).

    Returns (ids, dis) or, with stages=True, (ids, dis, coaidx, coadis,
    adc_ids, adc_dis)."""
    q = _c(queries, np.float32)
    nq = q.shape[0]
    if kl is None:
        kl = k
    kk = kl if rerank else k
    ids = np.empty((nq, k), np.int32)
    dis = np.empty((nq, k), np.float32)
    st = [None] * 4
    if stages:
        st = [np.empty((nq, w), np.int32), np.empty((nq, w), np.float32),
              np.empty((nq, kk), np.int32), np.empty((nq, kk), np.float32)]
    b = _c(base, np.float32) if base is not None else None
    s, keep = _pin(ix)
    rc = lib().orc_ivfpq_search(
        C.byref(s), _ptr(q), C.c_int(nq), _ptr(b), C.c_int(k), C.c_int(kl), C.c_int(w),
        C.c_int(1 if rerank else 0), C.c_int(ties), C.c_int(table_mode), _ptr(ids), _ptr(dis),
        *(_ptr(a) for a in st), C.c_int(nthreads))
    del keep
    if rc != 0:
        raise RuntimeError(f"orc_ivfpq_search failed ({rc})")
    return (ids, dis, *st) if stages else (ids, dis)


def search_batched(ix, queries, w_per_q, k_per_q, ties=TIES_KEYED, nthreads=1):
    """The engine's uneven batch (gbivf_search_batched) restated: per-query nprobe and k, no
    re-rank. Returns (ids, dis, offsets): query q's results are ids[offsets[q]:offsets[q+1]]."""
    q = _c(queries, np.float32)
    wq = _c(w_per_q, np.int32)
    kq = _c(k_per_q, np.int32)
    off = np.zeros(len(kq) + 1, np.int64)
    np.cumsum(kq, out=off[1:])
    ids = np.empty(int(off[-1]), np.int32)
    dis = np.empty(int(off[-1]), np.float32)
    s, keep = _pin(ix)
    lib().orc_ivfpq_search_batched.restype = C.c_int
    rc = lib().orc_ivfpq_search_batched(C.byref(s), _ptr(q), C.c_int(q.shape[0]), _ptr(wq), _ptr(kq),
                                        _ptr(off), C.c_int(ties), _ptr(ids), _ptr(dis), C.c_int(nthreads))
    del keep
    if rc != 0:
        raise RuntimeError(f"orc_ivfpq_search_batched failed ({rc})")
    return ids, dis, off


def pq_search(d, m, ks, pq, codes, queries, k, nthreads=1):
    """Restated pq_search: column-major (k x nq) dis and 1-based ids."""
    q = _c(queries, np.float32)
    codes = _c(codes, np.uint8)
    pq = _c(pq, np.float32)
    nq = q.shape[0]
    dis = np.empty((k, nq), np.float32)
    ids = np.empty((k, nq), np.int32)
    rc = lib().orc_pq_search(C.c_int(d), C.c_int(m), C.c_int(ks), _ptr(pq), _ptr(codes),
                             C.c_int64(codes.shape[0]), _ptr(q), C.c_int(nq), C.c_int(k),
                             _ptr(dis), _ptr(ids), C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"orc_pq_search failed ({rc})")
    return dis, ids


def core_cpu(ix, residual, rid_to_ivf, qid_to_starting_outid, nout, k, w, nthreads=1):
    """Restated parallel2 core_cpu: packed (idxs, dists) of length nout."""
    r = _c(residual, np.float32)
    rid = _c(rid_to_ivf, np.int32)
    qs = _c(qid_to_starting_outid, np.int32)
    idxs = np.full(nout, -1, np.int32)
    dists = np.full(nout, np.nan, np.float32)
    s, keep = _pin(ix)
    rc = lib().orc_core_cpu(C.byref(s), _ptr(r), C.c_int(r.shape[0]), _ptr(rid), _ptr(qs),
                            _ptr(idxs), _ptr(dists), C.c_int(k), C.c_int(w), C.c_int(nthreads))
    del keep
    if rc != 0:
        raise RuntimeError(f"orc_core_cpu failed ({rc})")
    return idxs, dists


def knn_full(mat2, mat1, k, ties=TIES_HEAP):
    m2 = _c(mat2, np.float32)
    m1 = _c(mat1, np.float32)
    vw = np.empty((m1.shape[0], k), np.int32)
    vd = np.empty((m1.shape[0], k), np.float32)
    lib().orc_knn_full(C.c_int(m1.shape[0]), C.c_int(m2.shape[0]), C.c_int(m2.shape[1]),
                       C.c_int(k), _ptr(m2), _ptr(m1), _ptr(vw), _ptr(vd), C.c_int(ties))
    return vw, vd


def cross_distances(a, b):
    """dist2[j, i] = ||a_i - b_j||^2 in the reference's arithmetic."""
    a = _c(a, np.float32)
    b = _c(b, np.float32)
    out = np.empty((b.shape[0], a.shape[0]), np.float32)
    lib().orc_cross_distances(C.c_int(a.shape[1]), C.c_int(a.shape[0]), C.c_int(b.shape[0]),
                              _ptr(a), C.c_int(a.shape[1]), _ptr(b), C.c_int(b.shape[1]),
                              _ptr(out), C.c_int(a.shape[0]))
    return out


# ---------------------------------------------------------------------------
# the reference itself (only where its sources exist)
# ---------------------------------------------------------------------------

def ref_available() -> bool:
    return _build.reference_available()


def ref():
    global _ref
    if _ref is None:
        path = _build.build_reference()
        if path is None:
            raise RuntimeError("reference sources not present on this machine")
        _ref = C.CDLL(path)
        _ref.ref_l2.restype = C.c_float
    return _ref


def ref_build_index(train, base, coarsek, nsq):
    """ivfpq_new + ivfpq_assign of the reference. One call per process."""
    tr = _c(train, np.float32)
    bs = _c(base, np.float32)
    d = tr.shape[1]
    coa = np.empty((coarsek, d), np.float32)
    pq = np.empty((nsq, 256, d // nsq), np.float32)
    sizes = np.empty(coarsek, np.int32)
    ids = np.empty(bs.shape[0], np.int32)
    codes = np.empty((bs.shape[0], nsq), np.int32)
    ks = ref().ref_build_index(_ptr(tr), C.c_int(tr.shape[0]), _ptr(bs), C.c_int(bs.shape[0]),
                               C.c_int(d), C.c_int(coarsek), C.c_int(nsq), _ptr(coa), _ptr(pq),
                               _ptr(sizes), _ptr(ids), _ptr(codes))
    assert ks == 256
    return coa, pq, sizes, ids, codes


def ref_build_pq(train, base, nsq):
    """pq_new + pq_assign of the reference (flat PQ, as pq_test runs them)."""
    tr = _c(train, np.float32)
    bs = _c(base, np.float32)
    d = tr.shape[1]
    pq = np.empty((nsq, 256, d // nsq), np.float32)
    codes = np.empty((bs.shape[0], nsq), np.int32)
    ks = ref().ref_build_pq(_ptr(tr), C.c_int(tr.shape[0]), _ptr(bs), C.c_int(bs.shape[0]),
                            C.c_int(d), C.c_int(nsq), _ptr(pq), _ptr(codes))
    assert ks == 256
    return pq, codes


def _ref_index_args(ix, codes_i32):
    sizes = np.diff(np.asarray(ix.list_off)).astype(np.int32)
    return (C.c_int(ix.d), C.c_int(ix.coarsek), C.c_int(ix.m), _ptr(_c(ix.coa, np.float32)),
            _ptr(_c(ix.pq, np.float32)), _ptr(sizes), _ptr(_c(ix.ids, np.int32)),
            _ptr(codes_i32)), sizes


def ref_ivfpq_search(ix, queries, base, k, kl, w):
    codes = _c(ix.codes, np.int32)
    args, keep = _ref_index_args(ix, codes)
    q = _c(queries, np.float32)
    b = _c(base, np.float32)
    ids = np.empty((q.shape[0], k), np.int32)
    ref().ref_ivfpq_search(*args, _ptr(q), C.c_int(q.shape[0]), _ptr(b), C.c_int(b.shape[0]),
                           C.c_int(k), C.c_int(kl), C.c_int(w), _ptr(ids))
    del keep
    return ids


def ref_adc_stage(ix, queries, kl, w):
    codes = _c(ix.codes, np.int32)
    args, keep = _ref_index_args(ix, codes)
    q = _c(queries, np.float32)
    nq = q.shape[0]
    coaidx = np.empty((nq, w), np.int32)
    coadis = np.empty((nq, w), np.float32)
    adc_ids = np.empty((nq, kl), np.int32)
    adc_dis = np.empty((nq, kl), np.float32)
    ref().ref_adc_stage(*args, _ptr(q), C.c_int(nq), C.c_int(kl), C.c_int(w), _ptr(coaidx),
                        _ptr(coadis), _ptr(adc_ids), _ptr(adc_dis))
    del keep
    return coaidx, coadis, adc_ids, adc_dis


def ref_pq_search(d, nsq, pq, codes, queries, k):
    q = _c(queries, np.float32)
    cb = _c(codes, np.int32)
    nq = q.shape[0]
    dis = np.empty((k, nq), np.float32)
    ids = np.empty((k, nq), np.int32)
    ref().ref_pq_search(C.c_int(d), C.c_int(nsq), _ptr(_c(pq, np.float32)), _ptr(cb),
                        C.c_int(cb.shape[0]), _ptr(q), C.c_int(nq), C.c_int(k), _ptr(dis), _ptr(ids))
    return dis, ids


def ref_l2(a, b):
    a = _c(a, np.float32)
    b = _c(b, np.float32)
    return float(ref().ref_l2(C.c_int(a.shape[0]), _ptr(a), _ptr(b)))
