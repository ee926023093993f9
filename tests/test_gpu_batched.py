"""Batched engine (GB300): uneven per-query nprobe and k in one launch
sequence, CUDA-graph capture and replay, and the scan-kernel autotuner.
Every result is compared with the oracle (keyed tie rule), query by query."""
import numpy as np
import pytest

import oracle
from tests import golden_cases

pytestmark = pytest.mark.gpu

KERNELS = {"persistent512": {"GBIVF_SCAN_THREADS": "512"}, "persistent1024": {"GBIVF_SCAN_THREADS": "1024"},
           "general": {"GBIVF_SCAN_KERNEL": "general"}}


def oracle_one(ix, q, k, w):
    ids, dis = oracle.ivfpq_search(ix, q[None, :], k=k, w=w, rerank=False, ties=oracle.TIES_KEYED)
    return ids[0], dis[0]


@pytest.mark.parametrize("variant", sorted(KERNELS))
@pytest.mark.parametrize("name", ["cfg1", "m16"])
def test_uneven_batch_vs_oracle(name, variant, monkeypatch):
    from mestrado_gb300.engine import GpuIndex

    for key, val in KERNELS[variant].items():
        monkeypatch.setenv(key, val)
    g = golden_cases.load(name)
    rng = np.random.default_rng(5)
    nq = len(g.queries)
    wq = rng.integers(1, g.ix.coarsek + 1, nq).astype(np.int32)
    kq = rng.choice([1, 10, 100, 1000], nq).astype(np.int32)
    gi = GpuIndex(g.ix)
    for mixed in (False, True):
        ids, dis, off = gi.search_batched(g.queries, wq, kq, mixed_coarse=mixed)
        for i in range(nq):
            o_ids, o_dis = oracle_one(g.ix, g.queries[i], int(kq[i]), int(wq[i]))
            np.testing.assert_array_equal(ids[off[i]:off[i + 1]], o_ids)
            np.testing.assert_array_equal(dis[off[i]:off[i + 1]].view(np.uint32), o_dis.view(np.uint32))
    gi.close()


def test_graph_capture_and_replay():
    import torch

    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix, base=g.base)
    nq, k, kl, w = 50, 10, 100, 4
    d_q = torch.from_numpy(g.queries[:nq].copy()).cuda()
    d_ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    d_dis = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    graph = gi.capture_graph(d_q.data_ptr(), nq, k, w, d_ids.data_ptr(), d_dis.data_ptr(), kl=kl, rerank=True,
                             stream_ptr=s.cuda_stream)
    for part in (slice(0, 50), slice(50, 100)):  # new queries in the same buffer, replay
        d_q.copy_(torch.from_numpy(g.queries[part].copy()))
        torch.cuda.synchronize()
        graph.launch(s.cuda_stream)
        s.synchronize()
        e_ids, e_dis = gi.search(g.queries[part], k, w, kl=kl, rerank=True)
        np.testing.assert_array_equal(d_ids.cpu().numpy(), e_ids)
        np.testing.assert_array_equal(d_dis.cpu().numpy().view(np.uint32), e_dis.view(np.uint32))
    graph.close()
    gi.close()


def test_graph_of_uneven_batch():
    import torch

    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("m16")
    gi = GpuIndex(g.ix)
    nq = len(g.queries)
    rng = np.random.default_rng(9)
    wq = rng.integers(1, 9, nq).astype(np.int32)
    kq = rng.choice([1, 10, 100], nq).astype(np.int32)
    off = np.concatenate([[0], np.cumsum(kq)]).astype(np.int64)
    d_q = torch.from_numpy(g.queries.copy()).cuda()
    d_w = torch.from_numpy(wq).cuda()
    d_k = torch.from_numpy(kq).cuda()
    d_off = torch.from_numpy(off[:-1].copy()).cuda()
    d_ids = torch.empty(int(off[-1]), dtype=torch.int32, device="cuda")
    d_dis = torch.empty(int(off[-1]), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    graph = gi.capture_graph(d_q.data_ptr(), nq, int(kq.max()), int(wq.max()), d_ids.data_ptr(), d_dis.data_ptr(),
                             d_w_ptr=d_w.data_ptr(), d_k_ptr=d_k.data_ptr(), d_off_ptr=d_off.data_ptr(),
                             stream_ptr=s.cuda_stream)
    d_ids.fill_(-5)
    graph.launch(s.cuda_stream)
    s.synchronize()
    e_ids, e_dis, e_off = gi.search_batched(g.queries, wq, kq)
    np.testing.assert_array_equal(d_ids.cpu().numpy(), e_ids)
    np.testing.assert_array_equal(d_dis.cpu().numpy().view(np.uint32), e_dis.view(np.uint32))
    graph.close()
    gi.close()


def test_autotune_picks_a_kernel_and_keeps_results(tmp_path, monkeypatch):
    import torch

    from mestrado_gb300.engine import GpuIndex

    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("GBIVF_TUNE_CACHE", str(cache))
    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix)
    d_q = torch.from_numpy(g.queries.copy()).cuda()
    before = gi.search(g.queries, 100, 4)
    choice, times = gi.autotune(d_q.data_ptr(), len(g.queries), 100, 4)
    assert choice in (0, 1, 512, 1024)  # 1: the list-centric pipeline
    assert all(t > 0 for t in times)
    after = gi.search(g.queries, 100, 4)
    np.testing.assert_array_equal(before[0], after[0])
    assert cache.read_text().strip().endswith(str(choice))
    choice2, times2 = gi.autotune(d_q.data_ptr(), len(g.queries), 100, 4)  # served from the cache file
    assert choice2 == choice and times2 == [-1.0, -1.0, -1.0, -1.0]
    gi.close()
