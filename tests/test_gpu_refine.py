"""Refinement-code re-rank (GB300): the kl ADC candidates re-ranked by the
distance to their refined reconstruction y + c1(codes) + c2(codes2). Checked
against a numpy restatement (FP32 in the defined order: sequential partial
sums over the eight blocks of 16 dimensions, then the partials summed in
block order) applied to the oracle's keyed ADC top-kl."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def refined_reference(ix, q, adc_ids, k):
    """Per query: candidates in ADC order -> (dist, adc rank) keyed top-k."""
    row_of = np.empty(ix.n, np.int64)
    row_of[ix.ids] = np.arange(ix.n)
    list_of = np.searchsorted(ix.list_off, np.arange(ix.n), side="right") - 1
    m, ds = ix.m, ix.ds
    m2 = ix.pq2.shape[0]
    ds2 = 128 // m2
    out_ids, out_dis = [], []
    for qi in range(q.shape[0]):
        cand = adc_ids[qi][adc_ids[qi] >= 0]
        rows = row_of[cand]
        lists = list_of[rows]
        dist = np.zeros(len(cand), np.float32)
        for blk in range(8):
            part = np.zeros(len(cand), np.float32)
            for t in range(16 * blk, 16 * blk + 16):
                s, s2 = t // ds, t // ds2
                y = ix.coa[lists, t]
                a = ix.pq[s, ix.codes[rows, s], t - s * ds]
                b = ix.pq2[s2, ix.codes2[rows, s2], t - s2 * ds2]
                e = ((np.float32(q[qi, t]) - y) - a) - b
                part = part + e * e
            dist = dist + part
        order = np.lexsort((np.arange(len(cand)), dist))[:k]
        out_ids.append(cand[order])
        out_dis.append(dist[order])
    return np.array(out_ids), np.array(out_dis)


def built_index(m2=8, m=8):
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=128, seed=31, zipf=1.1))
    base = g.generate(60000, stream_id=1)
    train = g.generate(30000, stream_id=2)
    q = g.generate(40, stream_id=3).cpu().numpy()
    ix = build_index_gpu(base, train, coarsek=128, m=m, niter=5, seed=4, m2=m2)
    return ix, q, base.cpu().numpy()


def test_refined_rerank_matches_reference():
    from mestrado_gb300.engine import GpuIndex

    ix, q, base = built_index()
    assert ix.codes2.shape == (ix.n, 8)
    gi = GpuIndex(ix)
    k, kl, w = 10, 200, 16
    adc_ids, _ = oracle.ivfpq_search(ix, q, k=kl, kl=kl, w=w, rerank=False, ties=oracle.TIES_KEYED)
    r_ids, r_dis = refined_reference(ix, q, adc_ids, k)
    for mixed in (False, True):
        ids, dis = gi.search(q, k, w, kl=kl, refine=True, mixed_scan=mixed, mixed_coarse=mixed)
        np.testing.assert_array_equal(ids, r_ids)
        np.testing.assert_array_equal(dis.view(np.uint32), r_dis.view(np.uint32))
    # the refined distances approximate the true ones much better than the ADC distances
    true = ((q[:, None, :].astype(np.float64) - base[ids]) ** 2).sum(-1)
    err_refined = np.abs(dis - true).mean()
    adc_top, adc_dis = gi.search(q, k, w)
    err_adc = np.abs(adc_dis - ((q[:, None, :].astype(np.float64) - base[adc_top]) ** 2).sum(-1)).mean()
    print(f"mean |refined - true| {err_refined:.1f}, mean |adc - true| {err_adc:.1f}")
    assert err_refined < err_adc
    gi.close()


@pytest.mark.parametrize("m,m2", [(16, 16), (4, 16), (16, 4)])
def test_refined_rerank_other_shapes(m, m2):
    """Sub-vector lengths other than 16: a lane's 16 dimensions span two sub-quantizers (ds = 8)
    or half of one (ds = 32), for the PQ codes and the refinement codes alike."""
    from mestrado_gb300.engine import GpuIndex

    ix, q, _ = built_index(m2=m2, m=m)
    gi = GpuIndex(ix)
    k, kl, w = 10, 100, 12
    adc_ids, _ = oracle.ivfpq_search(ix, q, k=kl, kl=kl, w=w, rerank=False, ties=oracle.TIES_KEYED)
    r_ids, r_dis = refined_reference(ix, q, adc_ids, k)
    for mixed in (False, True):
        ids, dis = gi.search(q, k, w, kl=kl, refine=True, mixed_scan=mixed, mixed_coarse=mixed)
        np.testing.assert_array_equal(ids, r_ids)
        np.testing.assert_array_equal(dis.view(np.uint32), r_dis.view(np.uint32))
    gi.close()


def test_refine_flag_rules():
    from mestrado_gb300.engine import GbivfError, GpuIndex
    from tests import golden_cases

    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix, base=g.base)
    with pytest.raises(GbivfError):  # no refinement codes on this index
        gi.search(g.queries, 10, 4, kl=100, refine=True)
    gi.close()
    ix, q, base = built_index()
    gi = GpuIndex(ix, base=base)
    with pytest.raises(GbivfError):  # raw and refined re-rank together
        gi.search(q, 10, 4, kl=100, refine=True, rerank=True)
    with pytest.raises(GbivfError):  # kl < k
        gi.search(q, 50, 4, kl=10, refine=True)
    gi.close()
