"""Selection stress (GB300): ADC top-k of the engine vs the oracle's keyed
rule on synthetic indexes built to stress the block selection -- lists
whose codes repeat a few rows (many equal distances, resolved by position),
k from 1 to 2000 (the persistent kernel up to 1024, the general one above),
and a d=96 index that only the general kernel takes."""
import numpy as np
import pytest

import oracle
from mestrado_gb300.ivfdata import IVFPQData

pytestmark = pytest.mark.gpu


def make_index(seed, d=128, m=8, C=6, sizes=(5000, 3000, 1, 0, 7000, 800), distinct_rows=None):
    rng = np.random.default_rng(seed)
    ds = d // m
    coa = rng.uniform(0, 100, (C, d)).astype(np.float32)
    pq = rng.normal(0, 10, (m, 256, ds)).astype(np.float32)
    off = np.zeros(C + 1, np.int64)
    off[1:] = np.cumsum(sizes[:C])
    n = int(off[-1])
    if distinct_rows:
        rows = rng.integers(0, 256, (distinct_rows, m), dtype=np.uint8)
        codes = rows[rng.integers(0, distinct_rows, n)]
    else:
        codes = rng.integers(0, 256, (n, m), dtype=np.uint8)
    ids = rng.permutation(n).astype(np.int32)
    ix = IVFPQData(coa=coa, pq=pq, list_off=off, ids=ids, codes=np.ascontiguousarray(codes))
    ix.validate()
    q = rng.uniform(0, 100, (40, d)).astype(np.float32)
    return ix, q


KERNELS = {"persistent512": {"GBIVF_SCAN_THREADS": "512"}, "persistent1024": {"GBIVF_SCAN_THREADS": "1024"},
           "general": {"GBIVF_SCAN_KERNEL": "general"}}


@pytest.mark.parametrize("variant", sorted(KERNELS))
@pytest.mark.parametrize("distinct", [None, 3])
@pytest.mark.parametrize("k", [1, 7, 100, 1000, 2000])
def test_topk_vs_oracle(k, distinct, variant, monkeypatch):
    from mestrado_gb300.engine import GpuIndex

    for key, val in KERNELS[variant].items():
        monkeypatch.setenv(key, val)
    ix, q = make_index(7, distinct_rows=distinct)
    gi = GpuIndex(ix)
    for w in (1, 3, 6):
        ids, dis = gi.search(q, k, w)
        o_ids, o_dis = oracle.ivfpq_search(ix, q, k=k, w=w, rerank=False, ties=oracle.TIES_KEYED)
        np.testing.assert_array_equal(ids, o_ids)
        np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    gi.close()


def test_general_kernel_shape():
    from mestrado_gb300.engine import GpuIndex

    ix, q = make_index(11, d=96, m=12, sizes=(900, 2500, 0, 40, 3000, 100))
    gi = GpuIndex(ix)
    for k, w in ((10, 2), (300, 6)):
        ids, dis = gi.search(q, k, w)
        o_ids, o_dis = oracle.ivfpq_search(ix, q, k=k, w=w, rerank=False, ties=oracle.TIES_KEYED)
        np.testing.assert_array_equal(ids, o_ids)
        np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    gi.close()


@pytest.mark.parametrize("variant", sorted(KERNELS))
@pytest.mark.parametrize("m", [4, 8, 16])
def test_direct_tables_other_m(m, variant, monkeypatch):
    """core_gpu's direct tables with m = 4, 8, 16 on every scan kernel."""
    from mestrado_gb300.engine import GpuIndex

    for key, val in KERNELS[variant].items():
        monkeypatch.setenv(key, val)
    ix, q = make_index(5, m=m)
    gi = GpuIndex(ix)
    w, k = 4, 50
    # expansion tables with re-rank-free search on the same kernel
    ids, dis = gi.search(q, k, w)
    o_ids, o_dis = oracle.ivfpq_search(ix, q, k=k, w=w, rerank=False, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    coaidx = np.argsort(((q[:, None, :] - ix.coa[None]) ** 2).sum(-1), axis=1)[:, :w].astype(np.int32)
    res = (q[:, None, :] - ix.coa[coaidx]).reshape(-1, 128).astype(np.float32)
    cnt = np.minimum(ix.list_sizes()[coaidx].sum(1), k)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
    idxs, dists = gi.core_gpu(res, coaidx.reshape(-1), start, int(cnt.sum()), k, w)
    o_idxs, o_dists = oracle.core_cpu(ix, res, coaidx.reshape(-1), start, int(cnt.sum()), k, w)
    np.testing.assert_array_equal(idxs, o_idxs)
    np.testing.assert_array_equal(dists.view(np.uint32), o_dists.view(np.uint32))
    gi.close()
