"""The reference's file formats (TEXMEX vectors, the parallel2 index files)
and its R@r statistic, on the host."""
import os

import numpy as np
import pytest

from mestrado_gb300 import refio


def test_fvecs_ivecs_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.normal(size=(37, 12)).astype(np.float32)
    g = rng.integers(0, 1000, (37, 5)).astype(np.int32)
    refio.write_fvecs(tmp_path / "a.fvecs", a)
    refio.write_ivecs(tmp_path / "g.ivecs", g)
    np.testing.assert_array_equal(refio.read_fvecs(tmp_path / "a.fvecs"), a)
    np.testing.assert_array_equal(refio.read_fvecs(tmp_path / "a.fvecs", n=10), a[:10])
    np.testing.assert_array_equal(refio.read_ivecs(tmp_path / "g.ivecs"), g)
    np.testing.assert_array_equal(refio.ground_truth_first(g), g[:, 0])


def test_fvecs_byte_layout(tmp_path):
    """Each record: int32 d, then d values (vector.c:296-335)."""
    a = np.array([[1.5, -2.0, 3.25]], np.float32)
    refio.write_fvecs(tmp_path / "x.fvecs", a)
    raw = open(tmp_path / "x.fvecs", "rb").read()
    assert raw[:4] == np.int32(3).tobytes() and raw[4:] == a.tobytes()


def test_bvecs_widen_and_offset(tmp_path):
    """b2fvecs_read widens bytes to floats; my_bvecs_read's offset counts
    blocks of n vectors (pq_test_load_vectors.cpp:275-325)."""
    b = np.arange(6 * 4, dtype=np.uint8).reshape(6, 4) * 10
    refio.write_bvecs(tmp_path / "b.bvecs", b)
    np.testing.assert_array_equal(refio.read_bvecs(tmp_path / "b.bvecs"), b.astype(np.float32))
    np.testing.assert_array_equal(refio.read_bvecs(tmp_path / "b.bvecs", n=2, offset=1), b[2:4].astype(np.float32))
    np.testing.assert_array_equal(refio.read_bvecs(tmp_path / "b.bvecs", n=4, offset=1), b[4:6].astype(np.float32))


def test_bad_dimension_rejected(tmp_path):
    raw = np.concatenate([np.array([2], np.int32).view(np.uint8), np.zeros(8, np.uint8),
                          np.array([3], np.int32).view(np.uint8), np.zeros(8, np.uint8)])
    raw.tofile(tmp_path / "bad.fvecs")
    with pytest.raises(ValueError):
        refio.read_fvecs(tmp_path / "bad.fvecs")


def test_r_at_matches_reference_rule():
    """rank = the slot of the first ground-truth neighbour, k+1 if absent;
    R@r = % of queries with rank < r, for r <= k."""
    k = 10
    gnd = np.array([5, 7, 9, 11], np.int32)
    ids = np.full((4, k), -1, np.int32)
    ids[0, 0] = 5      # rank 0
    ids[1, 3] = 7      # rank 3
    ids[2, 9] = 9      # rank 9
    # query 3: absent
    r = refio.r_at(ids, gnd, k, layout="row0")
    assert r == {1: 25.0, 2: 25.0, 5: 50.0, 10: 75.0}
    # the same in pq_search's layout: k x nq column-major, 1-based ids
    col = np.where(ids >= 0, ids + 1, 0).T.copy()
    assert refio.r_at(col.ravel(), gnd, k, layout="col1") == r


def test_parallel2_index_round_trip_and_layout(tmp_path):
    from mestrado_gb300.ivfdata import IVFPQData

    rng = np.random.default_rng(3)
    C, d, m = 6, 16, 4
    sizes = np.array([3, 0, 5, 1, 0, 2], np.int64)
    off = np.concatenate([[0], np.cumsum(sizes)])
    n = int(off[-1])
    ix = IVFPQData(coa=rng.normal(size=(C, d)).astype(np.float32),
                   pq=rng.normal(size=(m, 256, d // m)).astype(np.float32), list_off=off,
                   ids=rng.permutation(100)[:n].astype(np.int32),
                   codes=rng.integers(0, 256, (n, m)).astype(np.uint8))
    refio.write_parallel2_index(ix, tmp_path / "train", tmp_path / "ivf")
    hdr = np.fromfile(tmp_path / "train" / "header", np.int32)
    assert hdr.tolist() == [m, 256, d // m, 256 * d // m, m, C, C, d]
    f2 = np.fromfile(tmp_path / "ivf" / "2", np.int32)
    assert f2[0] == C and f2[1] == 5 and f2[7] == 5 and f2[8] == m and f2.size == 2 + 5 + 2 + 5 * m
    back = refio.read_parallel2_index(tmp_path / "train", tmp_path / "ivf")
    for a in ("coa", "pq", "list_off", "ids", "codes"):
        np.testing.assert_array_equal(getattr(back, a), getattr(ix, a))


def test_parallel2_index_rejects_wide_codes(tmp_path):
    from mestrado_gb300.ivfdata import IVFPQData

    ix = IVFPQData(coa=np.zeros((1, 8), np.float32), pq=np.zeros((2, 256, 4), np.float32),
                   list_off=np.array([0, 1]), ids=np.zeros(1, np.int32), codes=np.zeros((1, 2), np.uint8))
    refio.write_parallel2_index(ix, tmp_path / "t", tmp_path / "i")
    a = np.fromfile(tmp_path / "i" / "0", np.int32)
    a[-1] = 300  # a code a ks = coarsek build could hold, not a byte
    a.tofile(tmp_path / "i" / "0")
    with pytest.raises(ValueError):
        refio.read_parallel2_index(tmp_path / "t", tmp_path / "i")


@pytest.mark.gpu
def test_imported_index_searches_like_the_reference(tmp_path):
    """The reference-built golden index, written in parallel2's layout and read
    back, searches on the GPU with the reference's own coarse lists and the
    oracle's results."""
    import oracle
    from mestrado_gb300.engine import GpuIndex
    from tests import golden_cases

    g = golden_cases.load("cfg1")
    refio.write_parallel2_index(g.ix, tmp_path / "train", tmp_path / "ivf")
    ix = refio.read_parallel2_index(tmp_path / "train", tmp_path / "ivf")
    gi = GpuIndex(ix, base=g.base)
    w = g.meta["w"]
    np.testing.assert_array_equal(gi.coarse_assign(g.queries, w)[0], g.z["ref_coaidx"])
    ids, dis = gi.search(g.queries, 100, w, kl=100, rerank=True)
    o_ids, o_dis = oracle.ivfpq_search(ix, g.queries, k=100, kl=100, w=w, base=g.base, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    gi.close()
