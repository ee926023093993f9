"""Precision form of the scan (GB300): FP16 approximate tables summed in FP32,
then, of the alpha*k best, those within the tables' error bound of the k-th
exact distance re-scored in the reference's FP32 arithmetic. Every returned
distance must be the plain form's for that id; ids match the plain form's on
every query the form reports as proven, and may differ elsewhere only where a
true neighbour fell outside the approximate selection."""
import numpy as np
import pytest

from tests import golden_cases

pytestmark = pytest.mark.gpu


def compare(a_ids, a_dis, b_ids, b_dis):
    """(fraction of identical rows, every matching id carries the same distance bits)."""
    a_ids, b_ids = np.atleast_2d(a_ids), np.atleast_2d(b_ids)
    a_dis, b_dis = np.atleast_2d(a_dis), np.atleast_2d(b_dis)
    same_rows = np.mean([np.array_equal(x, y) for x, y in zip(a_ids, b_ids)])
    ok = True
    for ia, da, ib, db in zip(a_ids, a_dis, b_ids, b_dis):
        pa = {int(i): float(d) for i, d in zip(ia, da) if i >= 0}
        for i, d in zip(ib, db):
            if i >= 0 and int(i) in pa and np.float32(pa[int(i)]).view(np.uint32) != np.float32(d).view(np.uint32):
                ok = False
    return same_rows, ok


@pytest.mark.parametrize("name", ["cfg1", "m16"])
@pytest.mark.parametrize("rerank", [False, True])
def test_mixed_scan_golden(name, rerank):
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load(name)
    gi = GpuIndex(g.ix, base=g.base)
    w = g.meta["w"]
    for k, kl in ((100, 100), (10, 100), (1, 50)):
        a = gi.search(g.queries, k, w, kl=kl, rerank=rerank)
        b = gi.search(g.queries, k, w, kl=kl, rerank=rerank, mixed_scan=True)
        same, ok = compare(a[0], a[1], b[0], b[1])
        u = gi.last_unproven()
        print(f"[{name} rerank={rerank} k={k}] identical rows {same:.4f}, {u} not proven")
        assert ok, "a returned distance differs from the plain form's"
        assert same >= 0.99
        assert round((1.0 - same) * len(g.queries)) <= u
    gi.close()


def test_mixed_scan_uneven_batch_and_both_mixed_forms():
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("m16")
    rng = np.random.default_rng(9)
    nq = len(g.queries)
    wq = rng.integers(1, g.ix.coarsek + 1, nq).astype(np.int32)
    kq = rng.choice([1, 10, 100, 1000], nq).astype(np.int32)
    gi = GpuIndex(g.ix)
    a_ids, a_dis, off = gi.search_batched(g.queries, wq, kq)
    b_ids, b_dis, _ = gi.search_batched(g.queries, wq, kq, mixed_coarse=True, mixed_scan=True)
    u = gi.last_unproven()
    rows = [(a_ids[off[i]:off[i + 1]], a_dis[off[i]:off[i + 1]], b_ids[off[i]:off[i + 1]], b_dis[off[i]:off[i + 1]])
            for i in range(nq)]
    same = np.mean([np.array_equal(r[0], r[2]) for r in rows])
    ok = all(compare(r[0], r[1], r[2], r[3])[1] for r in rows)
    print(f"uneven: identical rows {same:.4f}, {u} not proven")
    assert ok and same >= 0.99
    assert round((1.0 - same) * nq) <= u
    gi.close()


def test_mixed_scan_on_gpu_built_zipf_index():
    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    gm = GpuMixture(Mixture(d=128, ncomp=512, seed=13, zipf=1.1))
    base = gm.generate(300000, stream_id=1)
    train = gm.generate(60000, stream_id=2)
    q = gm.generate(300, stream_id=3).cpu().numpy()
    ix = build_index_gpu(base, train, coarsek=1024, m=16, niter=4, seed=2)
    gi = GpuIndex(ix)
    for k, w in ((100, 32), (1000, 64)):
        a = gi.search(q, k, w)
        b = gi.search(q, k, w, mixed_scan=True, mixed_coarse=True)
        u = gi.last_unproven()
        same, ok = compare(a[0], a[1], b[0], b[1])
        assert round((1.0 - same) * len(q)) <= u
        recall = np.mean([len(set(x) & set(y)) / k for x, y in zip(a[0], b[0])])
        print(f"k={k} w={w}: identical rows {same:.4f}, overlap with plain {recall:.5f}")
        assert ok
        assert recall >= 0.998
    gi.close()


def test_unproven_count_follows_the_last_search():
    """gbivf_last_unproven: 0 after an exact-form search; after a precision-form search with an
    approximate selection of max(alpha * k, k + 64), a count between 0 and the number of queries."""
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("m16")
    gi = GpuIndex(g.ix)
    w = g.meta["w"]
    gi.search(g.queries, 10, w, mixed_scan=True)
    u = gi.last_unproven()
    assert 0 <= u <= len(g.queries)
    gi.search(g.queries, 10, w)
    assert gi.last_unproven() == 0
    gi.close()


def test_mixed_scan_rejects_direct_tables():
    from mestrado_gb300.engine import GbivfError, GpuIndex

    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix)
    with pytest.raises(GbivfError) as e:
        gi.search(g.queries, 10, 4, direct=True, mixed_scan=True)
    assert e.value.code == 4
    gi.close()


@pytest.fixture(scope="module")
def long_list_indexes():
    """GPU-built indexes with few, long lists (~4,700 codes each on average), m = 4, 8 and 16, so
    that probes span several code chunks and more code groups than the precision form stages."""
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    gm = GpuMixture(Mixture(d=128, ncomp=64, seed=21))
    base = gm.generate(300000, stream_id=1)
    train = gm.generate(40000, stream_id=2)
    q = gm.generate(200, stream_id=3).cpu().numpy()
    out = {m: build_index_gpu(base, train, coarsek=64, m=m, niter=4, seed=3) for m in (4, 8, 16)}
    return out, q


@pytest.mark.parametrize("threads", ["512", "1024"])
@pytest.mark.parametrize("m", [4, 8, 16])
def test_mixed_scan_long_lists_every_shape(long_list_indexes, m, threads, monkeypatch):
    """Every sub-quantizer count and block size of the precision form (at 1024 threads and m = 4
    each thread holds a single table entry; past 1024 code groups a probe's codes come from global
    memory instead of the stage): distances bit-identical to the plain form's for every shared id."""
    from mestrado_gb300.engine import GpuIndex

    monkeypatch.setenv("GBIVF_SCAN_THREADS", threads)
    ixs, q = long_list_indexes
    gi = GpuIndex(ixs[m])
    for k, w in ((10, 3), (100, 8), (1000, 8)):  # (k = 1000 at m = 4: a wide second re-score round)
        a = gi.search(q, k, w)
        b = gi.search(q, k, w, mixed_scan=True)
        u = gi.last_unproven()
        same, ok = compare(a[0], a[1], b[0], b[1])
        print(f"m={m} threads={threads} k={k} w={w}: identical rows {same:.4f}, {u} not proven")
        assert round((1.0 - same) * len(q)) <= u
        assert ok, "a returned distance differs from the plain form's"
        assert same >= 0.99
    gi.close()


@pytest.mark.parametrize("m", [8, 16])
def test_auto_scan_form_default_then_tuned(long_list_indexes, m):
    """mixed_scan="auto" returns exactly what the form it resolves to returns: before tuning the
    precision form when m = 16 and the exact form otherwise; after the autotuner timed both forms,
    the faster one (reported by scan_form()). Combined with an explicit form it is rejected."""
    import torch

    from mestrado_gb300.engine import GbivfError, GpuIndex

    ixs, q = long_list_indexes
    gi = GpuIndex(ixs[m])
    k, w = 50, 6
    exact = gi.search(q, k, w)
    mixed = gi.search(q, k, w, mixed_scan=True)

    def same(a, b):
        return np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))

    assert gi.scan_form() == (False, m == 16)
    assert same(gi.search(q, k, w, mixed_scan="auto"), mixed if m == 16 else exact)
    d_q = torch.from_numpy(q).cuda()
    gi.autotune(d_q.data_ptr(), len(q), k, w, scan_form=True)
    tuned, form_mixed = gi.scan_form()
    print(f"m={m}: tuned scan form {'precision' if form_mixed else 'exact'}")
    assert tuned
    assert same(gi.search(q, k, w, mixed_scan="auto"), mixed if form_mixed else exact)
    ids, dis, off = gi.search_batched(q, np.full(len(q), w, np.int32), np.full(len(q), k, np.int32),
                                      mixed_scan="auto")
    ref = mixed if form_mixed else exact
    np.testing.assert_array_equal(ids.reshape(len(q), k), ref[0])
    from mestrado_gb300._lib import GBIVF_MIXED_SCAN, GBIVF_MIXED_SCAN_AUTO, check

    with pytest.raises(GbivfError) as e:
        check(gi.lib.gbivf_ivfpq_search(gi.h, q.ctypes.data, len(q), k, k, w, GBIVF_MIXED_SCAN | GBIVF_MIXED_SCAN_AUTO,
                                        ids.ctypes.data, dis.ctypes.data))
    assert e.value.code == 1
    gi.close()
