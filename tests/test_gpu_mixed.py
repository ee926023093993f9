"""Mixed-precision coarse stage (GB300 tensor cores): the BF16 tcgen05 GEMM
with the exact FP32 re-check must give the plain path's probe lists and
coarse distances bit for bit, and the same search results."""
import numpy as np
import pytest

from tests import golden_cases

pytestmark = pytest.mark.gpu


def synthetic(C, nq, seed):
    from mestrado_gb300.ivfdata import IVFPQData
    from mestrado_gb300.synth import Mixture
    from mestrado_gb300.train import kmeans

    mx = Mixture(d=128, ncomp=max(8, C // 4), seed=seed)
    means = mx.means()
    train = mx.train(max(4 * C, 2000), means)
    coa = kmeans(train, C, niter=3, seed=seed)
    q = mx.queries(nq, means)
    rng = np.random.default_rng(seed)
    ix = IVFPQData(coa=coa, pq=rng.normal(0, 10, (8, 256, 16)).astype(np.float32),
                   list_off=np.zeros(C + 1, np.int64), ids=np.zeros(0, np.int32), codes=np.zeros((0, 8), np.uint8))
    return ix, q


def check_coarse(gi, q, w):
    a_idx, a_dis = gi.coarse_assign(q, w)
    b_idx, b_dis, ncand, _ = gi.coarse_assign(q, w, mixed=True, stats=True)
    np.testing.assert_array_equal(b_idx, a_idx)
    np.testing.assert_array_equal(b_dis.view(np.uint32), a_dis.view(np.uint32))
    return ncand / len(q)


@pytest.mark.parametrize("name", ["cfg1", "m16"])
def test_mixed_coarse_golden(name):
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load(name)
    gi = GpuIndex(g.ix)
    per_q = check_coarse(gi, g.queries, g.meta["w"])
    np.testing.assert_array_equal(gi.coarse_assign(g.queries, g.meta["w"], mixed=True)[0], g.z["ref_coaidx"])
    print(f"[{name}] mixed coarse: {per_q:.1f} centroids re-checked per query of {g.ix.coarsek}")
    gi.close()


@pytest.mark.parametrize("C,nq,w", [(1000, 300, 1), (1000, 300, 16), (1024, 1000, 100), (4096, 777, 32)])
def test_mixed_coarse_synthetic(C, nq, w):
    from mestrado_gb300.engine import GpuIndex

    ix, q = synthetic(C, nq, seed=C + w)
    gi = GpuIndex(ix)
    per_q = check_coarse(gi, q, w)
    print(f"C={C} nq={nq} w={w}: {per_q:.1f} centroids re-checked per query")
    gi.close()


def test_mixed_search_equals_plain():
    from mestrado_gb300.engine import GpuIndex

    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix, base=g.base)
    for k, kl in ((100, 100), (10, 100)):
        a = gi.search(g.queries, k, 4, kl=kl, rerank=True)
        b = gi.search(g.queries, k, 4, kl=kl, rerank=True, mixed_coarse=True)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    gi.close()


def test_mixed_needs_d128():
    from mestrado_gb300.engine import GbivfError, GpuIndex

    g = golden_cases.load("small")
    gi = GpuIndex(g.ix)
    with pytest.raises(GbivfError) as e:
        gi.coarse_assign(g.queries, 3, mixed=True)
    assert e.value.code == 4
    gi.close()
