"""Pin the CPU oracle against outputs of the reference itself (CPU only).

The golden fixtures hold the reference's own results on seeded inputs
(tests/golden/make_golden.py). The oracle with the reference's heap tie rule
must reproduce the coarse k-min and every ADC distance bit for bit; ids may
differ only where distances tie (counted and printed)."""
import numpy as np
import pytest

import oracle
from oracle.compare import compare_ranked, set_differs
from tests import golden_cases

NAMES = golden_cases.NAMES


@pytest.mark.parametrize("name", NAMES)
def test_fixture_inputs_regenerate(name):
    g = golden_cases.load(name)
    assert g.queries.shape == (g.meta["nq"], g.meta["d"])
    assert np.all(g.queries == np.rint(g.queries)) and g.queries.min() >= 0 and g.queries.max() <= 255


@pytest.mark.parametrize("name", NAMES)
def test_oracle_coarse_bit_exact(name):
    g = golden_cases.load(name)
    w = g.meta["w"]
    kl = g.z["ref_adc_ids"].shape[1]
    _, _, co, cd, _, _ = oracle.ivfpq_search(g.ix, g.queries, k=1, kl=kl, w=w, base=g.base,
                                              stages=True)
    np.testing.assert_array_equal(co, g.z["ref_coaidx"])
    np.testing.assert_array_equal(cd.view(np.uint32), g.z["ref_coadis"].view(np.uint32))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_adc_matches_reference(name):
    g = golden_cases.load(name)
    w = g.meta["w"]
    kl = g.z["ref_adc_ids"].shape[1]
    _, _, _, _, ai, ad = oracle.ivfpq_search(g.ix, g.queries, k=1, kl=kl, w=w, base=g.base,
                                              stages=True)
    ref_ai, ref_ad = g.z["ref_adc_ids"], g.z["ref_adc_dis"]
    valid = ref_ai >= 0
    np.testing.assert_array_equal(ai >= 0, valid)
    # every ADC distance of the k-min, bit for bit
    np.testing.assert_array_equal(ad[valid].view(np.uint32), ref_ad[valid].view(np.uint32))
    rep = compare_ranked(ai, np.where(valid, ad, np.inf), ref_ai, np.where(valid, ref_ad, np.inf))
    print(f"[{name}] ADC k-min vs reference: {rep}")
    assert rep.ok, str(rep)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_search_matches_reference(name):
    g = golden_cases.load(name)
    w = g.meta["w"]
    for k, kl in g.meta["searches"]:
        ids, dis, _, _, ai, _ = oracle.ivfpq_search(g.ix, g.queries, k=k, kl=kl, w=w,
                                                    base=g.base, stages=True)
        ref_ids = g.z[f"ref_ids_k{k}_kl{kl}"]
        ref_dis = g.z[f"ref_dis_k{k}_kl{kl}"]
        # ADC candidate sets that differ by a boundary tie propagate
        ref_ai = g.z["ref_adc_ids"][:, :kl]
        upstream = set_differs(ai, ref_ai)
        # the reference re-rank distance of each returned id, bit for bit
        np.testing.assert_array_equal(dis[~upstream].view(np.uint32), ref_dis[~upstream].view(np.uint32))
        rep = compare_ranked(ids, dis, ref_ids, ref_dis, upstream=upstream)
        print(f"[{name}] ivfpq_search k={k} kl={kl} vs reference: {rep}")
        assert rep.ok, str(rep)


def test_oracle_pq_search_matches_reference():
    g = golden_cases.load("cfg1")
    k = g.meta["flat"]["k"]
    pq, codes = g.z["flat_pq"], g.z["flat_codes"]
    dis, ids = oracle.pq_search(g.meta["d"], g.meta["m"], 256, pq, codes, g.queries, k)
    np.testing.assert_array_equal(dis.view(np.uint32), g.z["ref_flat_dis"].view(np.uint32))
    # column-major, 1-based (sequential/pq-utils/pq_search.cpp:58-63)
    rep = compare_ranked(ids.T, dis.T, g.z["ref_flat_ids"].T, g.z["ref_flat_dis"].T)
    print(f"[cfg1] pq_search vs reference: {rep}")
    assert rep.ok, str(rep)
    assert ids.min() >= 1


def test_oracle_keyed_and_heap_agree_up_to_ties():
    g = golden_cases.load("cfg1")
    a = oracle.ivfpq_search(g.ix, g.queries, k=100, kl=100, w=4, base=g.base, ties=oracle.TIES_HEAP)
    b = oracle.ivfpq_search(g.ix, g.queries, k=100, kl=100, w=4, base=g.base, ties=oracle.TIES_KEYED)
    rep = compare_ranked(a[0], a[1], b[0], b[1])
    assert rep.ok, str(rep)


def test_knn_full_tie_rule():
    # equal distances: the heap keeps the earlier label while filling, then
    # orders by value and heap slot; the keyed rule orders by (value, index)
    base = np.zeros((6, 4), np.float32)
    base[:, 0] = [3, 1, 1, 2, 1, 5]
    q = np.zeros((1, 4), np.float32)
    ih, dh = oracle.knn_full(base, q, 3, ties=oracle.TIES_HEAP)
    ik, dk = oracle.knn_full(base, q, 3, ties=oracle.TIES_KEYED)
    assert sorted(ih[0].tolist()) == [1, 2, 4] and ik[0].tolist() == [1, 2, 4]
    assert dh[0].tolist() == dk[0].tolist() == [1.0, 1.0, 1.0]
