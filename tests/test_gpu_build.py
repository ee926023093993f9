"""GPU index building (GB300): generator, assignment, k-means, PQ encoding,
and an index built on the GPU searched with parity against the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def lib():
    from mestrado_gb300 import _lib

    return _lib.load()


def test_generator_is_chunk_invariant_and_byte_valued():
    from mestrado_gb300.gpu_build import GpuMixture
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=50, seed=4, zipf=1.1))
    whole = g.generate(1000, stream_id=7).cpu().numpy()
    a = g.generate(400, stream_id=7).cpu().numpy()
    b = g.generate(600, stream_id=7, row0=400).cpu().numpy()
    np.testing.assert_array_equal(whole, np.concatenate([a, b]))
    assert whole.min() >= 0 and whole.max() <= 255 and np.all(whole == np.rint(whole))
    other = g.generate(1000, stream_id=8).cpu().numpy()
    assert not np.array_equal(whole, other)


@pytest.mark.parametrize("d,k", [(128, 1000), (16, 256), (32, 100)])
def test_assign_is_nearest(d, k):
    import torch

    from mestrado_gb300._lib import check

    rng = np.random.default_rng(d + k)
    x = np.rint(rng.uniform(0, 255, (3000, d))).astype(np.float32)
    c = rng.uniform(0, 255, (k, d)).astype(np.float32)
    dx, dc = torch.from_numpy(x).cuda(), torch.from_numpy(c).cuda()
    a = torch.empty(3000, dtype=torch.int32, device="cuda")
    check(lib().gbivf_assign(C.c_void_p(dx.data_ptr()), 3000, d, C.c_void_p(dc.data_ptr()), k,
                             C.c_void_p(a.data_ptr()), C.c_void_p(0)))
    a = a.cpu().numpy()
    dist = ((x[:, None, :].astype(np.float64) - c[None].astype(np.float64)) ** 2).sum(-1)
    best = dist.min(1)
    got = dist[np.arange(3000), a]
    assert np.all(got <= best * (1 + 1e-5) + 1e-3)  # the nearest, up to near-ties
    assert (a == dist.argmin(1)).mean() > 0.99


def test_kmeans_objective_matches_host_trainer():
    import torch

    from mestrado_gb300._lib import check
    from mestrado_gb300.synth import Mixture
    from mestrado_gb300.train import kmeans

    mx = Mixture(d=128, ncomp=64, seed=3)
    x = mx.train(20000)
    k = 64
    dx = torch.from_numpy(x).cuda()
    cent = torch.empty((k, 128), dtype=torch.float32, device="cuda")
    check(lib().gbivf_kmeans(C.c_void_p(dx.data_ptr()), 20000, 128, k, 15, 1, C.c_void_p(cent.data_ptr()),
                             C.c_void_p(0)))
    cg = cent.cpu().numpy()
    ch = kmeans(x, k, niter=15, seed=1)

    def obj(c):
        return ((x[:, None, :].astype(np.float64) - c[None]) ** 2).sum(-1).min(1).mean()

    assert obj(cg) <= 1.05 * obj(ch)


def test_index_built_on_gpu_searches_with_parity():
    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=128, seed=11, zipf=1.1))
    base = g.generate(60000, stream_id=1)
    train = g.generate(20000, stream_id=2)
    q = g.generate(64, stream_id=3).cpu().numpy()
    ix = build_index_gpu(base, train, coarsek=256, m=8, niter=8, seed=5)
    sizes = ix.list_sizes()
    assert sizes.sum() == 60000 and sizes.max() > 2 * sizes.mean()  # uneven lists
    gi = GpuIndex(ix, base=base.cpu().numpy())
    ids, dis = gi.search(q, 20, 16, kl=100, rerank=True)
    o_ids, o_dis = oracle.ivfpq_search(ix, q, k=20, kl=100, w=16, base=base.cpu().numpy(), ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    gi.close()
