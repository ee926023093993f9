"""The oracle's uneven batch (per-query nprobe and k, packed outputs) is the
uniform oracle query by query: each query's row equals orc_ivfpq_search
without re-rank at that query's (w, k), padded with -1 / +inf where the
probed lists hold fewer than k candidates."""
import numpy as np

import oracle
from tests import golden_cases


def test_batched_oracle_is_the_uniform_oracle_per_query():
    g = golden_cases.load("small")
    ix, q = g.ix, g.queries[:40]
    rng = np.random.default_rng(4)
    wq = rng.integers(1, ix.coarsek + 1, len(q)).astype(np.int32)
    kq = rng.choice([1, 7, 50, 400], len(q)).astype(np.int32)
    ids, dis, off = oracle.search_batched(ix, q, wq, kq, nthreads=4)
    for i in range(len(q)):
        e_ids, e_dis = oracle.ivfpq_search(ix, q[i:i + 1], k=int(kq[i]), w=int(wq[i]), rerank=False,
                                           ties=oracle.TIES_KEYED)
        np.testing.assert_array_equal(ids[off[i]:off[i + 1]], e_ids[0])
        np.testing.assert_array_equal(dis[off[i]:off[i + 1]].view(np.uint32), e_dis[0].view(np.uint32))
    # some query asks for more candidates than its lists hold: padded
    assert (ids == -1).any() and np.isinf(dis[ids == -1]).all()
