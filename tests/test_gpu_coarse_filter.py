"""Large-C coarse stage (GB300): the sample-bound candidate filter, plain and
tensor-core forms, must return the full selection's probe lists and coarse
distances bit for bit -- including the queries for which the sample bound is
too low or the candidates overflow, which take all C centroids exactly."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def index_with(coa):
    from mestrado_gb300.ivfdata import IVFPQData

    C = coa.shape[0]
    rng = np.random.default_rng(C)
    return IVFPQData(coa=np.ascontiguousarray(coa, np.float32),
                     pq=rng.normal(0, 10, (8, 256, 16)).astype(np.float32),
                     list_off=np.zeros(C + 1, np.int64), ids=np.zeros(0, np.int32),
                     codes=np.zeros((0, 8), np.uint8))


def mixture_centroids(C, nq, seed):
    from mestrado_gb300.synth import Mixture

    mx = Mixture(d=128, ncomp=512, seed=seed)
    means = mx.means()
    # centroids as noisy copies of data points (byte-valued data, float centroids)
    coa = mx.train(C, means) + np.random.default_rng(seed).normal(0, 2, (C, 128)).astype(np.float32)
    return coa.astype(np.float32), mx.queries(nq, means)


def all_forms(gi, q, w):
    """{form: (idx, dis, rechecked, fallbacks)} of the four coarse forms."""
    out = {}
    for name, mixed, full in (("plain_full", False, True), ("plain_filter", False, False),
                              ("mixed_full", True, True), ("mixed_filter", True, False)):
        out[name] = gi.coarse_assign(q, w, mixed=mixed, full=full, stats=True)
    return out


def assert_same(forms, ref="plain_full"):
    ri, rd = forms[ref][0], forms[ref][1]
    for name, (idx, dis, _, _) in forms.items():
        np.testing.assert_array_equal(idx, ri, err_msg=name)
        np.testing.assert_array_equal(dis.view(np.uint32), rd.view(np.uint32), err_msg=name)


@pytest.mark.parametrize("C,w", [(16384, 1), (16384, 64), (32768, 256), (40000, 1024)])
def test_filter_equals_full_selection(C, w):
    from mestrado_gb300.engine import GpuIndex

    coa, q = mixture_centroids(C, 300, seed=C + w)
    gi = GpuIndex(index_with(coa))
    forms = all_forms(gi, q, w)
    assert_same(forms)
    # and the oracle's knn_full with the same keyed ties, on a few queries
    o_idx, o_dis = oracle.knn_full(coa, q[:20], w, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(forms["mixed_filter"][0][:20], o_idx)
    np.testing.assert_array_equal(forms["mixed_filter"][1][:20].view(np.uint32), o_dis.view(np.uint32))
    for name in ("plain_filter", "mixed_filter"):
        _, _, rechecked, fallbacks = forms[name]
        print(f"C={C} w={w} {name}: {rechecked / len(q):.0f} exact per query, {fallbacks} fallbacks")
        assert fallbacks <= len(q) // 100
        assert rechecked <= len(q) * (8 * w + 4096)
    gi.close()


def test_overflowing_candidates_fall_back():
    """4 distinct centroids, 4096 copies each: every query's bound admits
    4096 candidates, above the 1024 slots, so every query takes all C."""
    from mestrado_gb300.engine import GpuIndex

    rng = np.random.default_rng(5)
    distinct = rng.uniform(0, 255, (4, 128)).astype(np.float32)
    coa = np.tile(distinct, (4096, 1))
    q = np.rint(rng.uniform(0, 255, (50, 128))).astype(np.float32)
    gi = GpuIndex(index_with(coa))
    forms = all_forms(gi, q, 1)
    assert_same(forms)
    for name in ("plain_filter", "mixed_filter"):
        assert forms[name][3] == len(q), name
    # the nearest distinct centroid's first copy (keyed ties: lowest id)
    d = ((q[:, None, :].astype(np.float64) - distinct[None]) ** 2).sum(-1)
    np.testing.assert_array_equal(forms["plain_full"][0][:, 0], d.argmin(1))
    gi.close()


def test_low_sample_bound_falls_back():
    """The sampled centroids (the first 4096 of 16384) sit next to the
    queries and the rest far away, so the sample bound admits fewer than w
    centroids of the whole set and every query takes all C."""
    from mestrado_gb300.engine import GpuIndex

    rng = np.random.default_rng(6)
    centre = rng.uniform(100, 150, 128).astype(np.float32)
    near = centre + rng.normal(0, 3, (4096, 128)).astype(np.float32)
    far = centre + 60.0 + rng.normal(0, 3, (12288, 128)).astype(np.float32)
    coa = np.concatenate([near, far]).astype(np.float32)
    q = np.rint(centre + rng.normal(0, 2, (40, 128))).astype(np.float32)
    gi = GpuIndex(index_with(coa))
    w = 1024  # above the sample rank r (520), so the count would have to come from the far set
    forms = all_forms(gi, q, w)
    assert_same(forms)
    for name in ("plain_filter", "mixed_filter"):
        assert forms[name][3] == len(q), name
    gi.close()


def test_filtered_search_equals_full_search():
    """A whole search on a 16,384-list index: filter and full selection give
    the same results, plain and mixed."""
    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=256, seed=21))
    base = g.generate(200000, stream_id=1)
    train = g.generate(100000, stream_id=2)
    q = g.generate(200, stream_id=3).cpu().numpy()
    ix = build_index_gpu(base, train, coarsek=16384, m=8, niter=4, seed=3)
    gi = GpuIndex(ix)
    ref = gi.search(q, 50, 32)
    for mixed in (False, True):
        got = gi.search(q, 50, 32, mixed_coarse=mixed)
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1].view(np.uint32), ref[1].view(np.uint32))
    o_ids, o_dis = oracle.ivfpq_search(ix, q[:25], k=50, kl=50, w=32, rerank=False, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ref[0][:25], o_ids)
    np.testing.assert_array_equal(ref[1][:25].view(np.uint32), o_dis.view(np.uint32))
    gi.close()
