"""The reference-signature shims (include/gbivf_refcompat*.h).

CPU: the shims export the reference's exact mangled symbols, and -- where
the reference sources exist -- the reference's own sequential driver
(sequential/ivf_test.cpp) links against the shim instead of ivf_search.o.
GPU: the shim entry points, called with structs laid out as the
reference's, return what the C ABI returns."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from mestrado_gb300 import build as engine_build
from oracle import build as oracle_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SEQ = oracle_build.REF_SEQ  # the reference tree's location is known to the oracle's build recipe only
SEQ_SYMS = ["_Z12ivfpq_search5ivfpqP3ivf3matS2_iiiPiPf", "_Z9pq_search6pqtipo4matI3matiPfPi"]
PAR2_SYMS = ["_Z8core_gpu6pqtipo3matP3ivfiPiS3_4matIS0_ii", "_Z19preallocate_gpu_mem6pqtipoP3ivfi",
             "_Z18deallocate_gpu_memv"]


def shim(name):
    engine_build.build()
    return os.path.join(engine_build.LIBDIR, name)


def test_shims_export_reference_symbols():
    for lib, syms in (("libgbivf_refcompat_seq.so", SEQ_SYMS), ("libgbivf_refcompat_par2.so", PAR2_SYMS)):
        h = C.CDLL(shim(lib))
        for s in syms:
            assert hasattr(h, s), (lib, s)


@pytest.mark.skipif(not os.path.isdir(REF_SEQ), reason="reference sources not present")
def test_reference_driver_links_against_shim(tmp_path):
    """Link sequential/ivf_test.cpp with the reference's objects minus
    ivf_search.o plus the shim: the reference's ivfpq_search resolves to gbivf."""
    from oracle import build as ob

    ob.build_reference()
    cxx = ["g++", "-std=gnu++11", "-O2", "-w", "-DFINTEGER=int", "-I", REF_SEQ]
    subprocess.run([*cxx, "-c", os.path.join(REF_SEQ, "ivf_test.cpp"), "-o", str(tmp_path / "t.o")], check=True)
    subprocess.run([*cxx, "-c", os.path.join(REF_SEQ, "pq-utils", "pq_test_compute_stats.cpp"), "-o",
                    str(tmp_path / "s.o")], check=True)
    objs = [os.path.join(ob.REF_DIR, f) for f in os.listdir(ob.REF_DIR)
            if f.endswith(".o") and "ivf_search" not in f and "ref_harness" not in f]
    shim("libgbivf_refcompat_seq.so")
    exe = str(tmp_path / "ivfpq_test_gbivf")
    r = subprocess.run(["g++", "-o", exe, str(tmp_path / "t.o"), str(tmp_path / "s.o"), *objs,
                        "-L", engine_build.LIBDIR, "-lgbivf_refcompat_seq", "-lgbivf",
                        f"-Wl,-rpath,{engine_build.LIBDIR}", "-lm", "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", exe], capture_output=True, text=True).stdout
    assert f"U {SEQ_SYMS[0]}" in nm  # taken from the shim, not defined in the executable


# --- calls through the shims (GPU) -----------------------------------------

class Mat(C.Structure):
    _fields_ = [("mat", C.POINTER(C.c_float)), ("n", C.c_int), ("d", C.c_int)]


class MatI(C.Structure):
    _fields_ = [("mat", C.POINTER(C.c_int)), ("n", C.c_int), ("d", C.c_int)]


class PqSeq(C.Structure):
    _fields_ = [("nsq", C.c_int), ("ks", C.c_int), ("ds", C.c_int), ("centroids", C.POINTER(C.POINTER(C.c_float))),
                ("centroidsn", C.c_int), ("centroidsd", C.c_int)]


class PqPar2(C.Structure):
    _fields_ = [("nsq", C.c_int), ("ks", C.c_int), ("ds", C.c_int), ("centroids", C.POINTER(C.c_float)),
                ("centroidsn", C.c_int), ("centroidsd", C.c_int)]


class Ivfpq(C.Structure):
    _fields_ = [("pq", PqSeq), ("coarsek", C.c_int), ("coa_centroids", C.POINTER(C.c_float)),
                ("coa_centroidsn", C.c_int), ("coa_centroidsd", C.c_int)]


class Ivf(C.Structure):
    _fields_ = [("ids", C.POINTER(C.c_int)), ("idstam", C.c_int), ("codes", MatI)]


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def ref_structs(ix, keep):
    """ivfpq_t and ivf_t[] as the reference's ivfpq_new / ivfpq_assign leave them."""
    cents = (C.POINTER(C.c_float) * ix.m)()
    for s in range(ix.m):
        a = np.ascontiguousarray(ix.pq[s])
        keep.append(a)
        cents[s] = fptr(a)
    keep.append(cents)
    coa = np.ascontiguousarray(ix.coa)
    keep.append(coa)
    pq = PqSeq(ix.m, ix.ks, ix.ds, cents, ix.ks * ix.ds, ix.m)
    top = Ivfpq(pq, ix.coarsek, fptr(coa), ix.coarsek, ix.d)
    lists = (Ivf * ix.coarsek)()
    for l in range(ix.coarsek):
        b, e = int(ix.list_off[l]), int(ix.list_off[l + 1])
        ids = np.ascontiguousarray(ix.ids[b:e], np.int32)
        codes = np.ascontiguousarray(ix.codes[b:e].astype(np.int32))
        keep += [ids, codes]
        lists[l] = Ivf(iptr(ids), e - b, MatI(iptr(codes), e - b, ix.m))
    keep.append(lists)
    return top, lists


@pytest.mark.gpu
def test_ivfpq_search_through_shim():
    from mestrado_gb300.engine import GpuIndex
    from tests import golden_cases

    g = golden_cases.load("cfg1")
    lib = C.CDLL(shim("libgbivf_refcompat_seq.so"))
    f = getattr(lib, SEQ_SYMS[0])
    f.argtypes = [Ivfpq, C.POINTER(Ivf), Mat, Mat, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                  C.POINTER(C.c_float)]
    f.restype = None
    keep = []
    top, lists = ref_structs(g.ix, keep)
    q = np.ascontiguousarray(g.queries)
    base = np.ascontiguousarray(g.base)
    for k, kl in ((100, 100), (10, 100)):
        ids = np.empty((len(q), k), np.int32)
        dis = np.empty((len(q), k), np.float32)
        f(top, lists, Mat(fptr(q), len(q), 128), Mat(fptr(base), len(base), 128), k, kl, 4, iptr(ids), fptr(dis))
        gi = GpuIndex(g.ix, base=g.base)
        e_ids, e_dis = gi.search(q, k, 4, kl=kl, rerank=True)
        gi.close()
        np.testing.assert_array_equal(ids, e_ids)
        np.testing.assert_array_equal(dis.view(np.uint32), e_dis.view(np.uint32))


@pytest.mark.gpu
def test_pq_search_through_shim():
    from mestrado_gb300.engine import GpuPQ
    from tests import golden_cases

    g = golden_cases.load("cfg1")
    lib = C.CDLL(shim("libgbivf_refcompat_seq.so"))
    f = getattr(lib, SEQ_SYMS[1])
    f.argtypes = [PqSeq, MatI, Mat, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int)]
    f.restype = None
    pqc, codes = g.z["flat_pq"], g.z["flat_codes"]
    keep = []
    cents = (C.POINTER(C.c_float) * 8)()
    for s in range(8):
        a = np.ascontiguousarray(pqc[s])
        keep.append(a)
        cents[s] = fptr(a)
    cb = np.ascontiguousarray(codes.astype(np.int32))
    q = np.ascontiguousarray(g.queries)
    k = 100
    dis = np.empty((k, len(q)), np.float32)
    ids = np.empty((k, len(q)), np.int32)
    f(PqSeq(8, 256, 16, cents, 256 * 16, 8), MatI(iptr(cb), len(cb), 8), Mat(fptr(q), len(q), 128), k,
      fptr(dis), iptr(ids))
    e_dis, e_ids = GpuPQ(pqc, codes).pq_search(q, k)
    np.testing.assert_array_equal(ids, e_ids)
    np.testing.assert_array_equal(dis.view(np.uint32), e_dis.view(np.uint32))


@pytest.mark.gpu
def test_core_gpu_through_shim():
    import oracle
    from tests import golden_cases

    g = golden_cases.load("m16")
    ix = g.ix
    lib = C.CDLL(shim("libgbivf_refcompat_par2.so"))
    pre, core, dealloc = (getattr(lib, s) for s in (PAR2_SYMS[1], PAR2_SYMS[0], PAR2_SYMS[2]))
    pre.argtypes = [PqPar2, C.POINTER(Ivf), C.c_int]
    core.argtypes = [PqPar2, Mat, C.POINTER(Ivf), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), MatI, Mat,
                     C.c_int, C.c_int]
    for fn in (pre, core, dealloc):
        fn.restype = None
    keep = []
    _, lists = ref_structs(ix, keep)
    flat = np.ascontiguousarray(ix.pq.reshape(-1))
    pq = PqPar2(ix.m, ix.ks, ix.ds, fptr(flat), ix.ks * ix.ds, ix.m)
    pre(pq, lists, ix.coarsek)
    w, k = g.meta["w"], 20
    coaidx = g.z["ref_coaidx"]
    res = np.ascontiguousarray((g.queries[:, None, :] - ix.coa[coaidx]).reshape(-1, 128), np.float32)
    rid = np.ascontiguousarray(coaidx.reshape(-1), np.int32)
    cnt = np.minimum(ix.list_sizes()[coaidx].sum(1), k)
    start = np.ascontiguousarray(np.concatenate([[0], np.cumsum(cnt)[:-1]]), np.int32)
    nout = int(cnt.sum())
    idxs = np.full(nout, -1, np.int32)
    dists = np.full(nout, np.nan, np.float32)
    core(pq, Mat(fptr(res), len(res), 128), lists, ix.coarsek, iptr(rid), iptr(start), MatI(iptr(idxs), nout, 1),
         Mat(fptr(dists), nout, 1), k, w)
    dealloc()
    o_idxs, o_dists = oracle.core_cpu(ix, res, rid, start, nout, k, w)
    np.testing.assert_array_equal(idxs, o_idxs)
    np.testing.assert_array_equal(dists.view(np.uint32), o_dists.view(np.uint32))
