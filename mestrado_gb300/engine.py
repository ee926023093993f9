"""Python mirror of the reference's IVF-PQ search entry points, on the GPU.

Each function keeps the reference's name, argument meaning and output
convention, and runs through the C ABI (include/gbivf.h):

* :func:`ivfpq_search` -- ``ivfpq_search(ivfpq, ivf, vquery, vbase, k, kl, w,
  ids, dis)`` (sequential/ivf_pq/ivf_search.cpp:9);
* :func:`pq_search` -- ``pq_search(pq, codebook, vquery, k, dis, ids)``
  (sequential/pq-utils/pq_search.cpp:10);
* :func:`core_gpu` -- ``core_gpu(PQ, residual, ivf, ivf_size, rid_to_ivf,
  qid_to_starting_outid, idxs, dists, k, w)`` (parallel2/ivf_pq/mycuda.cu:119).

Errors raise :class:`GbivfError` (the reference exits the process instead).
"""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np

from . import _lib
from ._lib import GBIVF_PROFILE, GBIVF_RERANK, GBIVF_TABLE_DIRECT, GbivfError, check  # noqa: F401
from .ivfdata import IVFPQData


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


class GpuIndex:
    """An IVF-PQ index resident in GPU memory (the handle owns it)."""

    def __init__(self, data: IVFPQData, device: int = 0, base: np.ndarray | None = None):
        data.validate()
        self.lib = _lib.load()
        self.data = data
        self.device = device
        h = C.c_void_p()
        keep = [_c(data.coa, np.float32), _c(data.pq, np.float32), _c(data.list_off, np.int64),
                _c(data.ids, np.int32), _c(data.codes, np.uint8)]
        check(self.lib.gbivf_index_create(C.byref(h), device, data.d, data.coarsek, _p(keep[0]), data.m,
                                          data.ks, _p(keep[1]), _p(keep[2]), _p(keep[3]), _p(keep[4])))
        self.h = h
        self.base_rows = 0
        if data.pq2 is not None:
            p2, c2 = _c(data.pq2, np.float32), _c(data.codes2, np.uint8)
            check(self.lib.gbivf_index_set_refine(h, data.pq2.shape[0], 256, _p(p2), _p(c2)))
        if base is not None:
            self.set_base(base)

    @classmethod
    def from_device(cls, coa, pq, list_off, d_ids, d_codes, pq2=None, d_codes2=None, device: int = 0) -> "GpuIndex":
        """An index whose lists are already in device memory (torch tensors in list
        order: d_ids n int32, d_codes n x m uint8, optional refinement codebook pq2
        (host) and codes d_codes2 n x m2): no host copy of the codes."""
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.data = None
        self.device = device
        self.base_rows = 0
        h = C.c_void_p()
        keep = [_c(coa, np.float32), _c(pq, np.float32), _c(list_off, np.int64)]
        check(self.lib.gbivf_index_create_device(C.byref(h), device, coa.shape[1], coa.shape[0], _p(keep[0]),
                                                 pq.shape[0], pq.shape[1], _p(keep[1]), _p(keep[2]),
                                                 C.c_void_p(d_ids.data_ptr()), C.c_void_p(d_codes.data_ptr())))
        self.h = h
        if pq2 is not None:
            p2 = _c(pq2, np.float32)
            check(self.lib.gbivf_index_set_refine_device(h, pq2.shape[0], 256, _p(p2),
                                                         C.c_void_p(d_codes2.data_ptr())))
        return self

    @classmethod
    def from_handle(cls, h: C.c_void_p, device: int = 0) -> "GpuIndex":
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.data = None
        self.device = device
        self.h = h
        return self

    def set_base(self, base: np.ndarray) -> None:
        b = _c(base, np.float32)
        check(self.lib.gbivf_index_set_base(self.h, _p(b), b.shape[0], b.shape[1]))
        self.base_rows = b.shape[0]
        self.base_key = None

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gbivf_index_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dims(self):
        d, c, m, ks = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        n = C.c_int64()
        check(self.lib.gbivf_index_dims(self.h, C.byref(d), C.byref(c), C.byref(m), C.byref(ks), C.byref(n)))
        return d.value, c.value, m.value, ks.value, n.value

    # -- searches ---------------------------------------------------------
    @staticmethod
    def _scan_flag(mixed_scan):
        """mixed_scan: False (exact form), True (precision form) or "auto" (the engine's choice)."""
        if mixed_scan == "auto":
            return _lib.GBIVF_MIXED_SCAN_AUTO
        return _lib.GBIVF_MIXED_SCAN if mixed_scan else 0

    @staticmethod
    def _order_flag(scan_order):
        """scan_order: None (the engine's choice), "lists" (list by list) or "queries" (query by query)."""
        if scan_order is None:
            return 0
        return {"lists": _lib.GBIVF_LIST_SCAN, "queries": _lib.GBIVF_QUERY_SCAN}[scan_order]

    def scan_form(self):
        """(tuned, mixed): the scan form mixed_scan="auto" resolves to on this index."""
        t, m = C.c_int(), C.c_int()
        check(self.lib.gbivf_index_scan_form(self.h, C.byref(t), C.byref(m)))
        return bool(t.value), bool(m.value)

    def search(self, queries, k, w, kl=None, rerank=False, direct=False, out=None, mixed_coarse=False,
               mixed_scan=False, refine=False, scan_order=None):
        """ivfpq_search: (ids nq x k int32, dis nq x k float32). ``out`` may
        pass preallocated (ids, dis) host arrays (e.g. pinned memory)."""
        q = _c(queries, np.float32)
        nq = q.shape[0]
        if out is None:
            ids = np.empty((nq, k), np.int32)
            dis = np.empty((nq, k), np.float32)
        else:
            ids, dis = out
            assert ids.shape == (nq, k) and ids.dtype == np.int32 and ids.flags.c_contiguous
            assert dis.shape == (nq, k) and dis.dtype == np.float32 and dis.flags.c_contiguous
        flags = (GBIVF_RERANK if rerank else 0) | (GBIVF_TABLE_DIRECT if direct else 0)
        flags |= _lib.GBIVF_MIXED_COARSE if mixed_coarse else 0
        flags |= self._scan_flag(mixed_scan)
        flags |= _lib.GBIVF_RERANK_REFINE if refine else 0
        flags |= self._order_flag(scan_order)
        check(self.lib.gbivf_ivfpq_search(self.h, _p(q), nq, k, kl if kl is not None else k, w, flags,
                                          _p(ids), _p(dis)))
        return ids, dis

    def search_device(self, d_queries_ptr, nq, k, w, d_ids_ptr, d_dis_ptr, kl=None, rerank=False,
                      stream_ptr=0, profile=False, mixed_coarse=False, mixed_scan=False, refine=False,
                      scan_order=None):
        """Device-pointer search (pointers as ints), enqueued on stream_ptr."""
        flags = (GBIVF_RERANK if rerank else 0) | (GBIVF_PROFILE if profile else 0)
        flags |= _lib.GBIVF_MIXED_COARSE if mixed_coarse else 0
        flags |= self._scan_flag(mixed_scan)
        flags |= _lib.GBIVF_RERANK_REFINE if refine else 0
        flags |= self._order_flag(scan_order)
        check(self.lib.gbivf_ivfpq_search_device(self.h, C.c_void_p(d_queries_ptr), nq, k,
                                                 kl if kl is not None else k, w, flags, C.c_void_p(d_ids_ptr),
                                                 C.c_void_p(d_dis_ptr), C.c_void_p(stream_ptr)))

    def search_batched(self, queries, w_per_q, k_per_q, mixed_coarse=False, mixed_scan=False, out=None,
                       scan_order=None):
        """Uneven batch: per-query nprobe and k. Returns (ids, dis, offsets):
        query q's results are ids[offsets[q]:offsets[q+1]]. ``out`` may pass preallocated
        (ids, dis) host arrays of sum(k_per_q) entries (e.g. pinned memory)."""
        q = _c(queries, np.float32)
        wq = _c(w_per_q, np.int32)
        kq = _c(k_per_q, np.int32)
        off = np.zeros(len(kq) + 1, np.int64)
        np.cumsum(kq, out=off[1:])
        if out is None:
            ids = np.empty(int(off[-1]), np.int32)
            dis = np.empty(int(off[-1]), np.float32)
        else:
            ids, dis = out
            assert ids.shape == (int(off[-1]),) and ids.dtype == np.int32 and ids.flags.c_contiguous
            assert dis.shape == (int(off[-1]),) and dis.dtype == np.float32 and dis.flags.c_contiguous
        flags = (_lib.GBIVF_MIXED_COARSE if mixed_coarse else 0) | self._scan_flag(mixed_scan)
        flags |= self._order_flag(scan_order)
        check(self.lib.gbivf_search_batched(self.h, _p(q), q.shape[0], _p(wq), _p(kq), flags, _p(ids), _p(dis)))
        return ids, dis, off

    def search_batched_device(self, d_queries_ptr, nq, d_w_ptr, d_k_ptr, d_off_ptr, max_w, max_k, d_ids_ptr,
                              d_dis_ptr, stream_ptr=0, profile=False, mixed_coarse=False, mixed_scan=False,
                              scan_order=None):
        """Uneven batch on device buffers (pointers as ints), enqueued on stream_ptr."""
        flags = (GBIVF_PROFILE if profile else 0) | (_lib.GBIVF_MIXED_COARSE if mixed_coarse else 0)
        flags |= self._scan_flag(mixed_scan) | self._order_flag(scan_order)
        check(self.lib.gbivf_search_batched_device(self.h, C.c_void_p(d_queries_ptr), nq, C.c_void_p(d_w_ptr),
                                                   C.c_void_p(d_k_ptr), C.c_void_p(d_off_ptr), max_w, max_k, flags,
                                                   C.c_void_p(d_ids_ptr), C.c_void_p(d_dis_ptr),
                                                   C.c_void_p(stream_ptr)))

    def capture_graph(self, d_queries_ptr, nq, k, w, d_ids_ptr, d_dis_ptr, kl=None, rerank=False,
                      mixed_coarse=False, d_w_ptr=0, d_k_ptr=0, d_off_ptr=0, stream_ptr=0, mixed_scan=False,
                      refine=False, scan_order=None):
        """Capture a device-buffer search as a CUDA graph (see gbivf_graph_capture)."""
        flags = (GBIVF_RERANK if rerank else 0) | (_lib.GBIVF_MIXED_COARSE if mixed_coarse else 0)
        flags |= self._scan_flag(mixed_scan)
        flags |= _lib.GBIVF_RERANK_REFINE if refine else 0
        flags |= self._order_flag(scan_order)
        g = C.c_void_p()
        check(self.lib.gbivf_graph_capture(self.h, C.c_void_p(d_queries_ptr), nq, k, kl if kl is not None else k, w,
                                           flags, C.c_void_p(d_ids_ptr), C.c_void_p(d_dis_ptr), C.c_void_p(d_w_ptr),
                                           C.c_void_p(d_k_ptr), C.c_void_p(d_off_ptr), C.c_void_p(stream_ptr),
                                           C.byref(g)))
        return SearchGraph(self.lib, g)

    def autotune(self, d_queries_ptr, nq, k, w, kl=None, rerank=False, mixed_coarse=False, scan_form=False):
        """Pick the fastest scan kernel for this index; returns (choice, times_ms). With
        scan_form=True also time both scan forms for mixed_scan="auto" (see scan_form())."""
        flags = (GBIVF_RERANK if rerank else 0) | (_lib.GBIVF_MIXED_COARSE if mixed_coarse else 0)
        flags |= _lib.GBIVF_MIXED_SCAN_AUTO if scan_form else 0
        ch = C.c_int()
        t = (C.c_float * 4)()
        check(self.lib.gbivf_index_autotune(self.h, C.c_void_p(d_queries_ptr), nq, k, kl if kl is not None else k, w,
                                            flags, C.byref(ch), t))
        return ch.value, list(t)

    def last_stage_ms(self):
        """(coarse_ms, scan_ms) of the last search made with profile=True."""
        a, b = C.c_float(), C.c_float()
        check(self.lib.gbivf_last_stage_ms(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_stages_ms(self):
        """(coarse_ms, scan_kernel_ms, finalize_ms) of the last search made with profile=True."""
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        check(self.lib.gbivf_last_stages_ms(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def last_scan_parts(self):
        """(parts_ms, counters) of the last profiled search's scan stage (gbivf_last_scan_parts):
        planning, first pass, grouping, list-centric scan, selection, overflow pass, finalize; and
        pairs scanned list by list, work items, overflowed queries, 1 if it ran list by list."""
        p = (C.c_float * 7)()
        c = (C.c_int64 * 4)()
        check(self.lib.gbivf_last_scan_parts(self.h, p, c))
        names = ["plan", "first_pass", "grouping", "list_scan", "select", "overflow_pass", "finalize"]
        return dict(zip(names, list(p))), dict(zip(["pairs", "items", "overflowed", "list_scan"], list(c)))

    def last_unproven(self):
        """Queries of the last precision-form search whose result was not proven identical to the
        exact form's (gbivf_last_unproven); 0 after a search in the exact form."""
        n = C.c_int64()
        check(self.lib.gbivf_last_unproven(self.h, C.byref(n)))
        return n.value

    def coarse_assign(self, queries, w, mixed=False, stats=False, full=False):
        """knn_full over the coarse centroids: (coaidx, coadis) nq x w. With
        mixed=True the tensor-core form runs, with full=True the full-block
        selection instead of the large-C filter (same results either way);
        stats=True also returns the number of centroids re-checked exactly and
        the number of queries that took all centroids exactly."""
        q = _c(queries, np.float32)
        nq = q.shape[0]
        idx = np.empty((nq, w), np.int32)
        dis = np.empty((nq, w), np.float32)
        nc, nf = C.c_int64(0), C.c_int64(0)
        flags = (_lib.GBIVF_MIXED_COARSE if mixed else 0) | (_lib.GBIVF_COARSE_FULL if full else 0)
        check(self.lib.gbivf_coarse_assign_flags(self.h, _p(q), nq, w, flags, _p(idx), _p(dis), C.byref(nc)))
        check(self.lib.gbivf_last_coarse_stats(self.h, None, C.byref(nf)))
        return (idx, dis, nc.value, nf.value) if stats else (idx, dis)

    def core_gpu(self, residual, rid_to_ivf, qid_to_starting_outid, nout, k, w):
        r = _c(residual, np.float32)
        rid = _c(rid_to_ivf, np.int32)
        qs = _c(qid_to_starting_outid, np.int32)
        idxs = np.full(nout, -1, np.int32)
        dists = np.full(nout, np.nan, np.float32)
        check(self.lib.gbivf_core_gpu(self.h, _p(r), r.shape[0], _p(rid), _p(qs), _p(idxs), _p(dists), k, w))
        return idxs, dists


class SearchGraph:
    """A captured search; launch() replays it on a stream."""

    def __init__(self, lib, h):
        self.lib = lib
        self.h = h

    def launch(self, stream_ptr=0):
        check(self.lib.gbivf_graph_launch(self.h, C.c_void_p(stream_ptr)))

    def kernel_count(self) -> int:
        """Kernel launches per replay."""
        n = C.c_int()
        check(self.lib.gbivf_graph_kernel_count(self.h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbivf_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuPQ(GpuIndex):
    """A flat PQ codebook resident in GPU memory (pq_search)."""

    def __init__(self, pq: np.ndarray, codes: np.ndarray, device: int = 0):
        self.lib = _lib.load()
        self.data = None
        self.device = device
        pqc = _c(pq, np.float32)
        cb = _c(codes, np.uint8)
        m, ks, ds = pqc.shape
        h = C.c_void_p()
        check(self.lib.gbivf_pq_create(C.byref(h), device, m * ds, m, ks, _p(pqc), _p(cb), cb.shape[0]))
        self.h = h
        self.d = m * ds

    def pq_search(self, queries, k):
        q = _c(queries, np.float32)
        nq = q.shape[0]
        dis = np.empty((k, nq), np.float32)
        ids = np.empty((k, nq), np.int32)
        check(self.lib.gbivf_pq_search(self.h, _p(q), nq, k, _p(dis), _p(ids)))
        return dis, ids


def _content_key(a: np.ndarray) -> tuple:
    """Shape and a digest of the bytes: tells one base from another even when the caller refills
    the same array in place (the reference rewrites vectors in place, ivf_assign.cpp:15)."""
    a = np.ascontiguousarray(a, np.float32)
    return a.shape, hashlib.blake2b(memoryview(a).cast("B"), digest_size=16).digest()


def ivfpq_search(index: GpuIndex, vquery, vbase, k, kl, w):
    """The reference signature's semantics: always re-ranks kl -> k against
    vbase (uploaded again whenever its contents change). Returns (ids, dis)."""
    key = _content_key(vbase)
    if getattr(index, "base_key", None) != key:
        index.set_base(vbase)
        index.base_key = key
    return index.search(vquery, k, w, kl=kl, rerank=True)


def pq_search(pq, codebook, vquery, k):
    """pq_search with the reference's outputs: (dis, ids), k x nq, ids 1-based."""
    return GpuPQ(pq, codebook).pq_search(vquery, k)
