"""gbivf_coarse_assign_noalloc: the coarse stage for callers that cannot
allocate device memory (a plugin host with a fixed device-memory budget, or
a serving loop that must not take cudaMalloc's synchronisation). Its scratch
is a fixed file-scope device array, so the call itself allocates nothing.

Checked through the C ABI against the allocating entry point
(gbivf_coarse_assign), bit for bit -- the tolerance of every coarse test
here -- on two calls in a row with different batches, plus the rejection of
a batch larger than the scratch. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _index(seed=3, C_=1024, d=128, m=8):
    from mestrado_gb300.ivfdata import IVFPQData

    rng = np.random.default_rng(seed)
    coa = rng.uniform(0, 120, (C_, d)).astype(np.float32)
    pq = rng.normal(0, 10, (m, 256, d // m)).astype(np.float32)
    off = np.zeros(C_ + 1, np.int64)  # empty lists: only the coarse stage is used
    ix = IVFPQData(coa=coa, pq=pq, list_off=off, ids=np.zeros(0, np.int32),
                   codes=np.zeros((0, m), np.uint8))
    ix.validate()
    return ix, rng


def test_noalloc_matches_allocating_coarse_assign():
    import torch

    from mestrado_gb300 import _lib
    from mestrado_gb300.engine import GpuIndex

    lib = _lib.load()
    ix, rng = _index()
    gi = GpuIndex(ix)
    stream = torch.cuda.current_stream().cuda_stream
    for nq, w in ((3000, 16), (1777, 5)):  # two calls in a row, different shapes
        q = np.rint(np.clip(rng.normal(60, 30, (nq, 128)), 0, 255)).astype(np.float32)
        d_q = torch.from_numpy(q).cuda()
        d_idx = torch.full((nq, w), -7, dtype=torch.int32, device="cuda")
        d_dis = torch.full((nq, w), -7.0, dtype=torch.float32, device="cuda")
        rc = lib.gbivf_coarse_assign_noalloc(gi.h, C.c_void_p(d_q.data_ptr()), nq, w,
                                             C.c_void_p(d_idx.data_ptr()), C.c_void_p(d_dis.data_ptr()),
                                             C.c_void_p(stream))
        _lib.check(rc)
        torch.cuda.synchronize()
        ref_idx, ref_dis = gi.coarse_assign(q, w)
        np.testing.assert_array_equal(d_idx.cpu().numpy(), ref_idx)
        np.testing.assert_array_equal(d_dis.cpu().numpy().view(np.uint32), ref_dis.view(np.uint32))

    # the largest batch that fits (4,088 queries at coarsek = 1024: 16 MiB exactly) runs; one more
    # query is refused with a clear error naming that limit
    limit = 4088
    q = np.rint(np.clip(rng.normal(60, 30, (limit + 1, 128)), 0, 255)).astype(np.float32)
    d_q = torch.from_numpy(q).cuda()
    d_idx = torch.empty((limit + 1, 4), dtype=torch.int32, device="cuda")
    d_dis = torch.empty((limit + 1, 4), dtype=torch.float32, device="cuda")
    rc = lib.gbivf_coarse_assign_noalloc(gi.h, C.c_void_p(d_q.data_ptr()), limit, 4, C.c_void_p(d_idx.data_ptr()),
                                         C.c_void_p(d_dis.data_ptr()), C.c_void_p(stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    ref_idx, _ = gi.coarse_assign(q[:limit], 4)
    np.testing.assert_array_equal(d_idx[:limit].cpu().numpy(), ref_idx)
    too_many = lib.gbivf_coarse_assign_noalloc(gi.h, C.c_void_p(d_q.data_ptr()), limit + 1, 4,
                                               C.c_void_p(d_idx.data_ptr()), C.c_void_p(d_dis.data_ptr()),
                                               C.c_void_p(stream))
    assert too_many == 4
    msg = lib.gbivf_last_error()
    assert b"scratch" in msg and b"at most 4088 queries" in msg, msg
    gi.close()


def test_noalloc_matches_filtered_coarse_stage():
    """At coarsek >= 16,384 the allocating call takes the large-C filter (a sampled bound, then
    exact re-checks); the allocation-free call always selects over the full distance block. Both
    are exact, so they agree bit for bit."""
    import torch

    from mestrado_gb300 import _lib
    from mestrado_gb300.engine import GpuIndex

    lib = _lib.load()
    ix, rng = _index(seed=5, C_=16384)
    gi = GpuIndex(ix)
    stream = torch.cuda.current_stream().cuda_stream
    for nq, w in ((240, 32), (97, 64)):
        q = np.rint(np.clip(rng.normal(60, 30, (nq, 128)), 0, 255)).astype(np.float32)
        d_q = torch.from_numpy(q).cuda()
        d_idx = torch.full((nq, w), -7, dtype=torch.int32, device="cuda")
        d_dis = torch.full((nq, w), -7.0, dtype=torch.float32, device="cuda")
        _lib.check(lib.gbivf_coarse_assign_noalloc(gi.h, C.c_void_p(d_q.data_ptr()), nq, w,
                                                   C.c_void_p(d_idx.data_ptr()), C.c_void_p(d_dis.data_ptr()),
                                                   C.c_void_p(stream)))
        torch.cuda.synchronize()
        ref_idx, ref_dis = gi.coarse_assign(q, w)
        np.testing.assert_array_equal(d_idx.cpu().numpy(), ref_idx)
        np.testing.assert_array_equal(d_dis.cpu().numpy().view(np.uint32), ref_dis.view(np.uint32))
    gi.close()
