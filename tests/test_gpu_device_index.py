"""Indexes created from device-resident lists (GB300): the same search results
as the host upload path, the refinement codes placed in the same rows, and the
streaming builder for bases too large to hold."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_created_index_equals_host_created():
    import torch

    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=64, seed=8, zipf=1.1))
    base = g.generate(40000, stream_id=1)
    train = g.generate(20000, stream_id=2)
    q = g.generate(50, stream_id=3).cpu().numpy()
    ix = build_index_gpu(base, train, coarsek=100, m=8, niter=4, seed=1, m2=8)
    a = GpuIndex(ix)
    b = GpuIndex.from_device(ix.coa, ix.pq, ix.list_off, torch.from_numpy(ix.ids).cuda(),
                             torch.from_numpy(ix.codes).cuda(), ix.pq2, torch.from_numpy(ix.codes2).cuda())
    for kw in (dict(k=20, w=8), dict(k=10, w=16, kl=200, refine=True), dict(k=10, w=16, kl=200, refine=True,
                                                                             mixed_scan=True)):
        ra, rb = a.search(q, **kw), b.search(q, **kw)
        np.testing.assert_array_equal(ra[0], rb[0])
        np.testing.assert_array_equal(ra[1].view(np.uint32), rb[1].view(np.uint32))
    a.close()
    b.close()


def test_streaming_build_recall():
    import torch

    from mestrado_gb300.gpu_build import GpuMixture, build_index_streaming, exact_topk, exact_topk_streaming
    from mestrado_gb300.synth import Mixture

    g = GpuMixture(Mixture(d=128, ncomp=256, seed=12))
    train = g.generate(40000, stream_id=2)
    q = g.generate(64, stream_id=3)
    gi, off = build_index_streaming(g, 300000, train, coarsek=512, m=8, m2=8, niter=4, seed=3, chunk=70000)
    assert off[-1] == 300000
    base = g.generate(300000, stream_id=1)
    gt = exact_topk(base, q, 10)
    np.testing.assert_array_equal(exact_topk_streaming(g, 300000, q, 10, chunk=70000)[:, 0], gt[:, 0])
    qh = q.cpu().numpy()
    ids, _ = gi.search(qh, 10, 32, kl=500, refine=True)
    adc, _ = gi.search(qh, 10, 32)
    r_ref = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(ids, gt)])
    r_adc = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(adc, gt)])
    print(f"recall@10: ADC {r_adc:.3f}, refined re-rank {r_ref:.3f}")
    assert r_ref > r_adc
    gi.close()
