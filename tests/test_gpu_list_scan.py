"""The list-centric scan (GBIVF_LIST_SCAN): the batch's (query, probe) pairs
grouped by list, G queries per work item, a first pass over each query's
nearest probes for its threshold, emission of the keys below it, exact
selection, and the overflow pass.

Exact form: its results must be the per-query scan's bit for bit (ids and
distances) and the oracle's (keyed tie rule). Precision form: its approximate
sums run in a row-rotated order (rot_codes.cuh), so its candidate sets may
differ from the per-query kernel's in the last bits; what must hold is what
the form promises -- every returned distance is the exact one (bit-identical
to the exact form's for the same id), the ids are the exact form's on every
query that the form reports as proven (all but gbivf_last_unproven of them)
and on at least 99% of the queries. Covered on the golden cases, on uneven batches with
k up to 1000, on a GPU-built index with a few thousand queries, through the
overflow pass (a tiny emission buffer) and inside a CUDA graph (a replay
returns exactly what the direct call returns)."""
import numpy as np
import pytest

import oracle
from tests import golden_cases

pytestmark = pytest.mark.gpu


def _same(a, b, what):
    np.testing.assert_array_equal(a[0], b[0], err_msg=f"{what}: ids")
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32), err_msg=f"{what}: distances")


def _rows(x, off):
    """Rows of a result: (nq, k) arrays, or packed arrays with offsets."""
    if off is None:
        return [x[i] for i in range(len(x))]
    return [x[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def _precision(m, e, what, off=None, unproven=0):
    """The precision form's result m against the exact form's e: the same distance bits for every id both
    return, the same ids on every query but (at most) the `unproven` ones and on at least 99% of them."""
    mi, md, ei, ed = _rows(m[0], off), _rows(m[1], off), _rows(e[0], off), _rows(e[1], off)
    same = 0
    for q in range(len(mi)):
        same += int(np.array_equal(mi[q], ei[q]))
        ex = dict(zip(ei[q].tolist(), ed[q].view(np.uint32).tolist()))
        for i, d in zip(mi[q].tolist(), md[q].view(np.uint32).tolist()):
            assert i < 0 or i not in ex or ex[i] == d, f"{what}: query {q} id {i} distance differs"
    assert same >= 0.99 * len(mi), f"{what}: identical rows {same} of {len(mi)}"
    assert len(mi) - same <= unproven, f"{what}: {len(mi) - same} rows differ, {unproven} not proven"


@pytest.mark.parametrize("name", ["cfg1", "m16"])
def test_golden_cases_list_equals_query_and_oracle(name):
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load(name)
    gi = GpuIndex(g.ix, base=g.base)
    w = g.meta["w"]
    for k, kl, rerank in ((100, 100, True), (10, 60, True), (1, 1, False), (37, 37, False)):
        what = f"{name} k={k} kl={kl} rerank={rerank}"
        lst = gi.search(g.queries, k, w, kl=kl, rerank=rerank, scan_order="lists")
        _same(lst, gi.search(g.queries, k, w, kl=kl, rerank=rerank, scan_order="queries"), what)
        o = oracle.ivfpq_search(g.ix, g.queries, k=k, kl=kl, w=w, base=g.base if rerank else None, rerank=rerank,
                                ties=oracle.TIES_KEYED)
        _same(lst, o, f"{what} vs oracle")
        mix = gi.search(g.queries, k, w, kl=kl, rerank=rerank, mixed_scan=True, scan_order="lists")
        _precision(mix, lst, f"{what} precision form", unproven=gi.last_unproven())
    gi.close()


def test_list_scan_needs_d128():
    from mestrado_gb300._lib import GbivfError
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("small")  # d = 32
    gi = GpuIndex(g.ix)
    with pytest.raises(GbivfError):
        gi.search(g.queries, 5, 3, scan_order="lists")
    gi.close()


@pytest.mark.parametrize("name", ["cfg1", "m16"])
def test_uneven_batches(name):
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load(name)
    rng = np.random.default_rng(9)
    nq = len(g.queries)
    wq = rng.integers(1, g.ix.coarsek + 1, nq).astype(np.int32)
    kq = rng.choice([1, 10, 100, 1000], nq).astype(np.int32)
    gi = GpuIndex(g.ix)
    lst = gi.search_batched(g.queries, wq, kq, scan_order="lists")
    _same(lst[:2], gi.search_batched(g.queries, wq, kq, scan_order="queries")[:2], name)
    o_ids, o_dis, _ = oracle.search_batched(g.ix, g.queries, wq, kq)
    _same(lst[:2], (o_ids, o_dis), f"{name} vs oracle")
    mix = gi.search_batched(g.queries, wq, kq, mixed_coarse=True, mixed_scan=True, scan_order="lists")
    _precision(mix[:2], lst[:2], f"{name} precision form", off=lst[2], unproven=gi.last_unproven())
    gi.close()


def _gpu_index(nbase=600_000, C=2048, m=16, nq=4096, seed=3):
    import torch

    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    gm = GpuMixture(Mixture(d=128, ncomp=C, seed=seed, zipf=1.1))
    base = gm.generate(nbase, stream_id=1)
    train = gm.generate(100_000, stream_id=2)
    ix = build_index_gpu(base, train, C, m, niter=4, seed=seed)
    q = gm.generate(nq, stream_id=3).cpu().numpy()
    del base, train
    torch.cuda.empty_cache()
    return ix, q


@pytest.fixture(scope="module")
def built():
    return _gpu_index()


def test_gpu_built_index_list_equals_query(built):
    from mestrado_gb300.engine import GpuIndex

    ix, q = built
    rng = np.random.default_rng(4)
    wq = np.clip(np.floor(np.exp(rng.uniform(0.0, np.log(129), len(q)))), 1, 128).astype(np.int32)
    kq = rng.choice([1, 10, 100, 1000], len(q)).astype(np.int32)
    gi = GpuIndex(ix)
    lst = gi.search_batched(q, wq, kq, scan_order="lists")
    _same(lst[:2], gi.search_batched(q, wq, kq, scan_order="queries")[:2], "exact form")
    mix = gi.search_batched(q, wq, kq, mixed_coarse=True, mixed_scan=True, scan_order="lists")
    u = gi.last_unproven()
    print(f"precision form: {u} of {len(q)} queries not proven")
    _precision(mix[:2], lst[:2], "precision form", off=lst[2], unproven=u)
    # and a uniform batch with re-rank-free k = 100, w = 32
    lst = gi.search(q, 100, 32, scan_order="lists")
    qry = gi.search(q, 100, 32, scan_order="queries")
    _same(lst, qry, "uniform")
    gi.close()


def test_overflow_pass(built, monkeypatch):
    """With an emission buffer of 16 keys most queries overflow and are scanned again query by
    query; the results do not change."""
    import torch

    from mestrado_gb300.engine import GpuIndex

    ix, q = built
    q = q[:1536]
    rng = np.random.default_rng(6)
    wq = rng.integers(1, 65, len(q)).astype(np.int32)
    kq = rng.choice([10, 100, 1000], len(q)).astype(np.int32)
    ref = GpuIndex(ix)
    expect = ref.search_batched(q, wq, kq, scan_order="queries")
    ref.close()
    monkeypatch.setenv("GBIVF_LIST_SCAN_CAP", "16")
    gi = GpuIndex(ix)
    off = expect[2]
    d_q = torch.from_numpy(q).cuda()
    d_w, d_k = torch.from_numpy(wq).cuda(), torch.from_numpy(kq).cuda()
    d_off = torch.from_numpy(off[:-1].copy()).cuda()
    d_ids = torch.empty(int(off[-1]), dtype=torch.int32, device="cuda")
    d_dis = torch.empty(int(off[-1]), dtype=torch.float32, device="cuda")
    for mixed in (False, True):
        gi.search_batched_device(d_q.data_ptr(), len(q), d_w.data_ptr(), d_k.data_ptr(), d_off.data_ptr(),
                                 int(wq.max()), int(kq.max()), d_ids.data_ptr(), d_dis.data_ptr(), profile=True,
                                 mixed_scan=mixed, scan_order="lists")
        torch.cuda.synchronize()
        parts, counters = gi.last_scan_parts()
        assert counters["list_scan"] == 1 and counters["overflowed"] > len(q) // 4, counters
        got = (d_ids.cpu().numpy(), d_dis.cpu().numpy())
        if mixed:
            _precision(got, expect[:2], "overflow, precision form", off=off, unproven=gi.last_unproven())
        else:
            _same(got, expect[:2], "overflow, exact form")
    gi.close()


def test_graph_replay_list_scan(built):
    import torch

    from mestrado_gb300.engine import GpuIndex

    ix, q = built
    nq = 2048
    rng = np.random.default_rng(8)
    wq = rng.integers(1, 97, nq).astype(np.int32)
    kq = rng.choice([1, 10, 100, 1000], nq).astype(np.int32)
    gi = GpuIndex(ix)
    expect = gi.search_batched(q[:nq], wq, kq, mixed_coarse=True, mixed_scan=True, scan_order="lists")
    off = expect[2]
    d_q = torch.from_numpy(q[:nq].copy()).cuda()
    d_w, d_k = torch.from_numpy(wq).cuda(), torch.from_numpy(kq).cuda()
    d_off = torch.from_numpy(off[:-1].copy()).cuda()
    d_ids = torch.empty(int(off[-1]), dtype=torch.int32, device="cuda")
    d_dis = torch.empty(int(off[-1]), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    graph = gi.capture_graph(d_q.data_ptr(), nq, int(kq.max()), int(wq.max()), d_ids.data_ptr(), d_dis.data_ptr(),
                             mixed_coarse=True, mixed_scan=True, d_w_ptr=d_w.data_ptr(), d_k_ptr=d_k.data_ptr(),
                             d_off_ptr=d_off.data_ptr(), stream_ptr=s.cuda_stream, scan_order="lists")
    assert graph.kernel_count() > 5
    for _ in range(2):
        d_ids.fill_(-5)
        graph.launch(s.cuda_stream)
        s.synchronize()
        _same((d_ids.cpu().numpy(), d_dis.cpu().numpy()), expect[:2], "graph replay")
    graph.close()
    gi.close()
