"""GPU engine parity (GB300): the CUDA path, called through the C ABI,
against the CPU oracle on the same seeded inputs and against the golden
outputs of the reference itself.

* vs the oracle with the keyed tie rule (the engine's own rule): every
  coarse list, ADC distance, id and re-rank distance must be bit-identical;
* vs the reference's golden outputs: distances bit-identical, ids equal up to
  ties (the reference orders ties by qsort / heap slot), counts printed.
"""
import numpy as np
import pytest

import oracle
from oracle.compare import compare_ranked, set_differs
from tests import golden_cases

pytestmark = pytest.mark.gpu

NAMES = golden_cases.NAMES


@pytest.fixture(scope="module")
def engine():
    from mestrado_gb300 import engine as e

    return e


_idx_cache = {}


def gpu_index(engine, name):
    if name not in _idx_cache:
        g = golden_cases.load(name)
        _idx_cache[name] = engine.GpuIndex(g.ix, base=g.base)
    return _idx_cache[name]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", NAMES)
def test_coarse_assign_bit_exact(engine, name):
    g = golden_cases.load(name)
    ix = gpu_index(engine, name)
    w = g.meta["w"]
    co, cd = ix.coarse_assign(g.queries, w)
    np.testing.assert_array_equal(co, g.z["ref_coaidx"])
    np.testing.assert_array_equal(bits(cd), bits(g.z["ref_coadis"]))


@pytest.mark.parametrize("name", NAMES)
def test_adc_topk_vs_oracle_and_reference(engine, name):
    g = golden_cases.load(name)
    ix = gpu_index(engine, name)
    w = g.meta["w"]
    kl = g.z["ref_adc_ids"].shape[1]
    ids, dis = ix.search(g.queries, kl, w, rerank=False)
    o_ids, o_dis = oracle.ivfpq_search(g.ix, g.queries, k=kl, w=w, rerank=False, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(bits(dis), bits(o_dis))
    ref_ids, ref_dis = g.z["ref_adc_ids"], g.z["ref_adc_dis"]
    ref_dis = np.where(ref_ids >= 0, ref_dis, np.inf).astype(np.float32)
    rep = compare_ranked(ids, dis, ref_ids, ref_dis)
    print(f"[{name}] GPU ADC top-{kl} vs reference: {rep}")
    assert rep.ok, str(rep)


@pytest.mark.parametrize("name", NAMES)
def test_ivfpq_search_rerank_vs_oracle_and_reference(engine, name):
    g = golden_cases.load(name)
    ix = gpu_index(engine, name)
    w = g.meta["w"]
    for k, kl in g.meta["searches"]:
        ids, dis = ix.search(g.queries, k, w, kl=kl, rerank=True)
        o_ids, o_dis = oracle.ivfpq_search(g.ix, g.queries, k=k, kl=kl, w=w, base=g.base,
                                           ties=oracle.TIES_KEYED)
        np.testing.assert_array_equal(ids, o_ids)
        np.testing.assert_array_equal(bits(dis), bits(o_dis))
        ref_ids = g.z[f"ref_ids_k{k}_kl{kl}"]
        ref_dis = g.z[f"ref_dis_k{k}_kl{kl}"]
        a_ids, _ = ix.search(g.queries, kl, w, rerank=False)
        upstream = set_differs(np.where(a_ids >= 0, a_ids, -1), g.z["ref_adc_ids"][:, :kl])
        rep = compare_ranked(ids, dis, ref_ids, ref_dis, upstream=upstream)
        print(f"[{name}] GPU ivfpq_search k={k} kl={kl} vs reference: {rep}")
        assert rep.ok, str(rep)


def test_reference_entry_point_semantics(engine):
    g = golden_cases.load("cfg1")
    ix = gpu_index(engine, "cfg1")
    ids, _ = engine.ivfpq_search(ix, g.queries, g.base, 100, 100, 4)
    o_ids, _ = oracle.ivfpq_search(g.ix, g.queries, k=100, kl=100, w=4, base=g.base, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)


def test_pq_search_flat(engine):
    g = golden_cases.load("cfg1")
    k = g.meta["flat"]["k"]
    pq, codes = g.z["flat_pq"], g.z["flat_codes"]
    dis, ids = engine.pq_search(pq, codes, g.queries, k)
    o_dis, o_ids = oracle.pq_search(g.meta["d"], g.meta["m"], 256, pq, codes, g.queries, k)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(bits(dis), bits(o_dis))
    rep = compare_ranked(ids.T, dis.T, g.z["ref_flat_ids"].T, g.z["ref_flat_dis"].T)
    print(f"[cfg1] GPU pq_search vs reference: {rep}")
    assert rep.ok, str(rep)


@pytest.mark.parametrize("name", NAMES)
def test_core_gpu_vs_oracle(engine, name):
    g = golden_cases.load(name)
    ix = gpu_index(engine, name)
    w, k = g.meta["w"], 10
    coaidx = g.z["ref_coaidx"]
    # residuals as parallel2's assign rank builds them (ivf_assign.cpp:36-41)
    res = (g.queries[:, None, :] - g.ix.coa[coaidx]).reshape(-1, g.meta["d"]).astype(np.float32)
    rid = coaidx.reshape(-1).astype(np.int32)
    sizes = g.ix.list_sizes()
    cnt = np.minimum(sizes[coaidx].sum(1), k)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
    nout = int(cnt.sum())
    idxs, dists = ix.core_gpu(res, rid, start, nout, k, w)
    o_idxs, o_dists = oracle.core_cpu(g.ix, res, rid, start, nout, k, w)
    np.testing.assert_array_equal(idxs, o_idxs)
    np.testing.assert_array_equal(bits(dists), bits(o_dists))


def test_index_from_reference_lists(engine):
    """gbivf_index_create_from_lists: the reference's ivf_t layout (int32 codes)."""
    import ctypes as C

    from mestrado_gb300 import _lib

    g = golden_cases.load("m16")
    lib = _lib.load()
    ix = g.ix
    sizes = ix.list_sizes()
    keep = []
    pq_ptrs = (C.c_void_p * ix.m)()
    for s in range(ix.m):
        a = np.ascontiguousarray(ix.pq[s])
        keep.append(a)
        pq_ptrs[s] = a.ctypes.data
    id_ptrs = (C.c_void_p * ix.coarsek)()
    code_ptrs = (C.c_void_p * ix.coarsek)()
    for l in range(ix.coarsek):
        a = np.ascontiguousarray(ix.ids[ix.list_off[l]:ix.list_off[l + 1]])
        b = np.ascontiguousarray(ix.codes[ix.list_off[l]:ix.list_off[l + 1]].astype(np.int32))
        keep += [a, b]
        id_ptrs[l] = a.ctypes.data
        code_ptrs[l] = b.ctypes.data
    coa = np.ascontiguousarray(ix.coa)
    h = C.c_void_p()
    _lib.check(lib.gbivf_index_create_from_lists(C.byref(h), 0, ix.d, ix.coarsek, coa.ctypes.data, ix.m, ix.ks,
                                                 pq_ptrs, sizes.ctypes.data, id_ptrs, code_ptrs))
    gi = engine.GpuIndex.from_handle(h)
    ids, dis = gi.search(g.queries, 50, g.meta["w"])
    o_ids, o_dis = oracle.ivfpq_search(g.ix, g.queries, k=50, w=g.meta["w"], rerank=False, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(bits(dis), bits(o_dis))
    gi.close()


def test_errors_are_status_codes(engine):
    g = golden_cases.load("small")
    ix = gpu_index(engine, "small")
    with pytest.raises(engine.GbivfError) as e:
        ix.search(g.queries, 5, g.ix.coarsek + 1)
    assert e.value.code == 1
    bare = engine.GpuIndex(g.ix)
    with pytest.raises(engine.GbivfError):
        bare.search(g.queries, 5, 2, kl=10, rerank=True)  # no base set
    bare.close()
    with pytest.raises(engine.GbivfError) as e:
        ix.search(g.queries, 5000, 2)
    assert e.value.code == 4


def test_short_candidate_lists_pad(engine):
    """L < k: the reference asserts (nn.c:468); the engine pads -1 / +inf."""
    g = golden_cases.load("small")
    ix = gpu_index(engine, "small")
    ids, dis = ix.search(g.queries, 200, 1, kl=300, rerank=True)
    o_ids, o_dis = oracle.ivfpq_search(g.ix, g.queries, k=200, kl=300, w=1, base=g.base, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(bits(dis), bits(o_dis))
    assert (ids == -1).any() and np.isinf(dis[ids == -1]).all()


def test_empty_query_batch(engine):
    ix = gpu_index(engine, "small")
    ids, dis = ix.search(np.zeros((0, 32), np.float32), 5, 2)
    assert ids.shape == (0, 5)
