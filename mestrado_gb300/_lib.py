"""ctypes binding of the engine's C ABI (include/gbivf.h).

The library is built in-tree (``mestrado_gb300/lib/libgbivf.so``); loading
fails loudly if it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

GBIVF_OK = 0
GBIVF_RERANK = 0x1
GBIVF_TABLE_DIRECT = 0x2
GBIVF_MIXED_COARSE = 0x4
GBIVF_COARSE_FULL = 0x8
GBIVF_MIXED_SCAN = 0x10
GBIVF_RERANK_REFINE = 0x20
GBIVF_MIXED_SCAN_AUTO = 0x40
GBIVF_LIST_SCAN = 0x80
GBIVF_QUERY_SCAN = 0x200
GBIVF_PROFILE = 0x100

_lib = None

# every symbol declared in include/gbivf.h
EXPORTS = [
    "gbivf_last_error", "gbivf_version", "gbivf_index_create", "gbivf_index_create_from_lists",
    "gbivf_index_set_base", "gbivf_index_destroy", "gbivf_index_dims", "gbivf_ivfpq_search",
    "gbivf_ivfpq_search_device", "gbivf_coarse_assign", "gbivf_core_gpu", "gbivf_pq_create",
    "gbivf_pq_search", "gbivf_last_stage_ms", "gbivf_coarse_assign_noalloc", "gbivf_coarse_assign_flags",
    "gbivf_search_batched", "gbivf_search_batched_device", "gbivf_graph_capture", "gbivf_graph_launch",
    "gbivf_graph_destroy", "gbivf_graph_kernel_count", "gbivf_index_autotune", "gbivf_generate_mixture", "gbivf_kmeans", "gbivf_assign",
    "gbivf_pq_train", "gbivf_pq_encode", "gbivf_last_coarse_stats", "gbivf_coarse_assign_device",
    "gbivf_index_set_refine", "gbivf_index_set_refine_device", "gbivf_pq_error", "gbivf_index_create_device",
    "gbivf_assign_flags", "gbivf_last_stages_ms", "gbivf_last_scan_parts", "gbivf_last_unproven", "gbivf_selftest_wait_timeout", "gbivf_index_scan_form",
]


class GbivfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbivf error {code}: {msg}")
        self.code = code


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libgbivf.so (building it first if asked and absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"GPU engine library missing: {path} (run mestrado_gb300.build)")
        path = _build.build()
    lib = C.CDLL(path)
    vp, i32, i64, u32 = C.c_void_p, C.c_int, C.c_int64, C.c_uint
    lib.gbivf_last_error.restype = C.c_char_p
    lib.gbivf_version.restype = i32
    lib.gbivf_index_create.argtypes = [C.POINTER(vp), i32, i32, i32, vp, i32, i32, vp, vp, vp, vp]
    lib.gbivf_index_create_from_lists.argtypes = [C.POINTER(vp), i32, i32, i32, vp, i32, i32, vp, vp, vp, vp]
    lib.gbivf_index_set_base.argtypes = [vp, vp, i64, i32]
    lib.gbivf_index_destroy.argtypes = [vp]
    lib.gbivf_index_dims.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.gbivf_ivfpq_search.argtypes = [vp, vp, i32, i32, i32, i32, u32, vp, vp]
    lib.gbivf_ivfpq_search_device.argtypes = [vp, vp, i32, i32, i32, i32, u32, vp, vp, vp]
    lib.gbivf_coarse_assign.argtypes = [vp, vp, i32, i32, vp, vp]
    lib.gbivf_core_gpu.argtypes = [vp, vp, i32, vp, vp, vp, vp, i32, i32]
    lib.gbivf_pq_create.argtypes = [C.POINTER(vp), i32, i32, i32, i32, vp, vp, i64]
    lib.gbivf_pq_search.argtypes = [vp, vp, i32, i32, vp, vp]
    lib.gbivf_last_stage_ms.argtypes = [vp, vp, vp]
    lib.gbivf_last_stages_ms.argtypes = [vp, vp, vp, vp]
    lib.gbivf_last_scan_parts.argtypes = [vp, vp, vp]
    lib.gbivf_last_unproven.argtypes = [vp, vp]
    lib.gbivf_index_scan_form.argtypes = [vp, vp, vp]
    lib.gbivf_selftest_wait_timeout.argtypes = [C.c_int, vp, vp, vp]
    lib.gbivf_coarse_assign_noalloc.argtypes = [vp, vp, i32, i32, vp, vp, vp]
    lib.gbivf_coarse_assign_flags.argtypes = [vp, vp, i32, i32, u32, vp, vp, vp]
    lib.gbivf_last_coarse_stats.argtypes = [vp, vp, vp]
    lib.gbivf_coarse_assign_device.argtypes = [vp, vp, i32, i32, u32, vp, vp, vp]
    lib.gbivf_index_set_refine.argtypes = [vp, i32, i32, vp, vp]
    lib.gbivf_index_set_refine_device.argtypes = [vp, i32, i32, vp, vp]
    lib.gbivf_pq_error.argtypes = [vp, i64, i32, vp, vp, i32, vp, vp, vp, vp]
    lib.gbivf_index_create_device.argtypes = [C.POINTER(vp), i32, i32, i32, vp, i32, i32, vp, vp, vp, vp]
    lib.gbivf_assign_flags.argtypes = [vp, i64, i32, vp, i32, vp, u32, vp]
    lib.gbivf_search_batched.argtypes = [vp, vp, i32, vp, vp, u32, vp, vp]
    lib.gbivf_search_batched_device.argtypes = [vp, vp, i32, vp, vp, vp, i32, i32, u32, vp, vp, vp]
    lib.gbivf_graph_kernel_count.argtypes = [vp, vp]
    lib.gbivf_graph_capture.argtypes = [vp, vp, i32, i32, i32, i32, u32, vp, vp, vp, vp, vp, vp, C.POINTER(vp)]
    lib.gbivf_graph_launch.argtypes = [vp, vp]
    lib.gbivf_graph_destroy.argtypes = [vp]
    lib.gbivf_index_autotune.argtypes = [vp, vp, i32, i32, i32, i32, u32, vp, vp]
    u64 = C.c_uint64
    lib.gbivf_generate_mixture.argtypes = [vp, i64, i32, vp, i32, vp, C.c_float, u64, u64, i64, vp]
    lib.gbivf_kmeans.argtypes = [vp, i64, i32, i32, i32, u64, vp, vp]
    lib.gbivf_assign.argtypes = [vp, i64, i32, vp, i32, vp, vp]
    lib.gbivf_pq_train.argtypes = [vp, i64, i32, i32, i32, u64, vp, vp]
    lib.gbivf_pq_encode.argtypes = [vp, i64, i32, vp, vp, i32, vp, vp, vp]
    for name in EXPORTS:
        if name != "gbivf_last_error":
            getattr(lib, name).restype = i32
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != GBIVF_OK:
        msg = _lib.gbivf_last_error().decode(errors="replace") if _lib else "?"
        raise GbivfError(rc, msg)
