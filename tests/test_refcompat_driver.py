"""End to end through the reference-signature shim: a C++ program written
against the reference's sequential ivfpq_search signature
(tests/refcompat_driver.cpp), linked against libgbivf_refcompat_seq.so, run
as an executable.

The program refills ONE set of index and base buffers in place for each
index, the way the reference's ivfpq_assign hands back the same static
ivf_t array on every call (sequential/ivf_pq/ivf_assign.cpp:19): it searches
index A, then index B at the same addresses, then A again. Each call's ids
and distances must be the oracle's for the index the buffers held at the
time (bit for bit, ties ordered by (distance, id) on both sides).

The reference's own driver (sequential/ivf_test.cpp) is linked against the
shim in tests/test_refcompat.py where its sources exist; it cannot run on the
GPU host, which has no copy of the reference tree, so this program stands in
for it there."""
import os
import subprocess

import numpy as np
import pytest

from mestrado_gb300 import build as engine_build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_driver(out_dir):
    engine_build.build()
    exe = os.path.join(str(out_dir), "refcompat_driver")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "refcompat_driver.cpp"),
           "-o", exe, "-L", engine_build.LIBDIR, "-lgbivf_refcompat_seq", "-lgbivf",
           f"-Wl,-rpath,{engine_build.LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_builds_against_the_shim(tmp_path):
    exe = build_driver(tmp_path)
    nm = subprocess.run(["nm", exe], capture_output=True, text=True).stdout
    assert "U _Z12ivfpq_search5ivfpqP3ivf3matS2_iiiPiPf" in nm  # resolved by the shim at load time


def write_index(path, ix):
    sizes = np.diff(ix.list_off).astype(np.int32)
    with open(path, "wb") as f:
        np.array([ix.coarsek, ix.d, ix.m, ix.ks], np.int32).tofile(f)
        np.ascontiguousarray(ix.coa, np.float32).tofile(f)
        np.ascontiguousarray(ix.pq, np.float32).tofile(f)
        sizes.tofile(f)
        np.ascontiguousarray(ix.ids, np.int32).tofile(f)
        np.ascontiguousarray(ix.codes, np.int32).tofile(f)


def write_mat(path, x):
    with open(path, "wb") as f:
        np.array(x.shape, np.int32).tofile(f)
        np.ascontiguousarray(x, np.float32).tofile(f)


@pytest.mark.gpu
def test_driver_searches_each_index_it_is_given(tmp_path):
    import oracle
    from mestrado_gb300.synth import Mixture
    from mestrado_gb300.train import build_index
    from tests import golden_cases

    g = golden_cases.load("cfg1")
    # index B: another mixture, the same list count, sub-quantizers and base size
    mx = Mixture(d=128, ncomp=48, seed=11)
    means = mx.means()
    base_b = mx.base(len(g.base), means)
    ix_b = build_index(mx.train(4000, means), base_b, g.ix.coarsek, g.ix.m, niter=6, seed=5)
    write_index(tmp_path / "index_A.bin", g.ix)
    write_index(tmp_path / "index_B.bin", ix_b)
    write_mat(tmp_path / "base_A.bin", g.base)
    write_mat(tmp_path / "base_B.bin", base_b)
    write_mat(tmp_path / "queries.bin", g.queries)
    k, kl, w = 20, 60, 4
    exe = build_driver(tmp_path)
    r = subprocess.run([exe, str(tmp_path), str(k), str(kl), str(w)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nq = len(g.queries)
    expect = {}
    for name, ix, base in (("A", g.ix, g.base), ("B", ix_b, base_b)):
        expect[name] = oracle.ivfpq_search(ix, g.queries, k=k, kl=kl, w=w, base=base, ties=oracle.TIES_KEYED)
    for i, name in enumerate("ABA"):
        ids = np.fromfile(tmp_path / f"ids_{i}.bin", np.int32).reshape(nq, k)
        dis = np.fromfile(tmp_path / f"dis_{i}.bin", np.float32).reshape(nq, k)
        o_ids, o_dis = expect[name]
        np.testing.assert_array_equal(ids, o_ids, err_msg=f"call {i} (index {name})")
        np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32), err_msg=f"call {i} (index {name})")
    # the two indexes really give different answers, so a stale upload would have been caught
    assert not np.array_equal(expect["A"][0], expect["B"][0])
