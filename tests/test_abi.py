"""The C ABI library: builds, loads, exports every declared symbol, and
rejects bad arguments with a status code (CPU only; no compute calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mestrado_gb300 import _lib
from mestrado_gb300.ivfdata import IVFPQData

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            out |= set(re.findall(r"\b(gbivf_\w+)\s*\(", txt))
    return out


def test_header_declares_the_binding_list():
    assert declared_symbols() == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.gbivf_version() >= 1


def test_invalid_arguments_return_status():
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.gbivf_index_create(C.byref(h), 0, 8, 2, None, 2, 4, None, None, None, None) == 1
    assert b"NULL" in lib.gbivf_last_error()
    coa = np.zeros((2, 8), np.float32)
    pq = np.zeros((2, 300, 4), np.float32)
    off = np.zeros(3, np.int64)
    rc = lib.gbivf_index_create(C.byref(h), 0, 8, 2, coa.ctypes.data, 2, 300, pq.ctypes.data,
                                off.ctypes.data, None, None)
    assert rc == 4 and b"ks" in lib.gbivf_last_error()  # ks > 256 unsupported
    assert lib.gbivf_ivfpq_search(None, None, 1, 1, 1, 1, 0, None, None) == 1
    assert lib.gbivf_index_destroy(None) == 0
    # the reporting entry points of the batched engine
    n = C.c_int64()
    assert lib.gbivf_last_unproven(None, C.byref(n)) == 1
    assert lib.gbivf_last_scan_parts(None, None, None) == 1
    k = C.c_int()
    assert lib.gbivf_graph_kernel_count(None, C.byref(k)) == 1
    assert lib.gbivf_index_scan_form(None, C.byref(k), C.byref(k)) == 1
    assert lib.gbivf_last_stages_ms(None, None, None, None) == 1


def test_codes_out_of_range_rejected():
    lib = _lib.load()
    h = C.c_void_p()
    coa = np.zeros((1, 8), np.float32)
    pq = np.zeros((2, 4, 4), np.float32)
    off = np.array([0, 1], np.int64)
    ids = np.zeros(1, np.int32)
    codes = np.array([[0, 9]], np.uint8)
    rc = lib.gbivf_index_create(C.byref(h), 0, 8, 1, coa.ctypes.data, 2, 4, pq.ctypes.data,
                                off.ctypes.data, ids.ctypes.data, codes.ctypes.data)
    assert rc == 1 and b"code" in lib.gbivf_last_error()


def test_reference_lists_conversion():
    sizes = np.array([2, 0, 1], np.int32)
    codes = np.array([[1, 2], [3, 4], [5, 6]], np.int32)
    d = IVFPQData.from_reference_lists(np.zeros((3, 4), np.float32), np.zeros((2, 8, 2), np.float32),
                                       sizes, np.array([7, 8, 9], np.int32), codes)
    assert d.list_off.tolist() == [0, 2, 2, 3]
    assert d.codes.dtype == np.uint8 and d.codes.tolist() == codes.tolist()
    with pytest.raises(ValueError):
        IVFPQData.from_reference_lists(np.zeros((1, 4), np.float32), np.zeros((2, 8, 2), np.float32),
                                       np.array([1], np.int32), np.array([0], np.int32),
                                       np.array([[300, 0]], np.int32))
