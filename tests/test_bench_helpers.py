"""Host helpers of bench.py: the FP64 ADC-distance error report of the large configurations."""
import numpy as np


def _tiny_index(rng):
    from mestrado_gb300.ivfdata import IVFPQData

    C, d, m, n = 4, 16, 4, 50
    coa = rng.normal(size=(C, d)).astype(np.float32)
    pq = rng.normal(size=(m, 256, d // m)).astype(np.float32)
    off = np.array([0, 10, 25, 40, 50], np.int64)
    ids = rng.permutation(n).astype(np.int32)
    codes = rng.integers(0, 256, (n, m)).astype(np.uint8)
    return IVFPQData(coa=coa, pq=pq, list_off=off, ids=ids, codes=codes)


def _fp64_adc(ix, q, base_id):
    r = int(np.nonzero(ix.ids == base_id)[0][0])
    lst = int(np.searchsorted(ix.list_off, r, side="right") - 1)
    res = q.astype(np.float64) - ix.coa[lst].astype(np.float64)
    ds = ix.ds
    return sum(((res[s * ds:(s + 1) * ds] - ix.pq[s, ix.codes[r, s]].astype(np.float64)) ** 2).sum()
               for s in range(ix.m))


def test_adc_error_fp64_zero_for_rounded_exact_and_sees_perturbation():
    import bench

    rng = np.random.default_rng(0)
    ix = _tiny_index(rng)
    q = rng.normal(size=(2, ix.d)).astype(np.float32)
    sel = [ix.ids[[0, 12, 30]], ix.ids[[45, 5, 20]]]
    res_ids = np.concatenate(sel)
    res_dis = np.array([_fp64_adc(ix, q[i], b) for i in range(2) for b in sel[i]], np.float32)
    off, kq = np.array([0, 3, 6]), np.array([3, 3])
    err = bench.adc_error_fp64(ix, q, (res_ids, res_dis), off, kq, 2)
    assert err["pairs"] == 6 and err["max_rel"] < 1e-7
    bad = res_dis.copy()
    bad[4] *= 1.01
    err = bench.adc_error_fp64(ix, q, (res_ids, bad), off, kq, 2)
    assert 0.009 < err["max_rel"] < 0.011
    # padding ids (-1, fewer results than k) are skipped
    pad_ids = res_ids.copy()
    pad_ids[2] = -1
    assert bench.adc_error_fp64(ix, q, (pad_ids, res_dis), off, kq, 2)["pairs"] == 5


def test_parity_report_counts_rows_and_distance_bits():
    import bench

    g = np.array([[1, 2, 3], [4, 5, 6]], np.int32)
    gd = np.array([[1, 2, 3], [4, 5, 6]], np.float32)
    o = np.array([[1, 2, 3], [4, 6, 5]], np.int32)  # a tie order difference in row 1
    od = np.array([[1, 2, 3], [4, 6, 5]], np.float32)
    r = bench.parity_report(g, gd, o, od)
    assert r["identical_rows"] == 0.5 and r["distance_mismatches_on_shared_ids"] == 0
    od[0, 1] = np.nextafter(np.float32(2), np.float32(3))  # one ulp off for id 2
    assert bench.parity_report(g, gd, o, od)["distance_mismatches_on_shared_ids"] == 1


def test_parity_report_up_to_ties():
    import bench

    g = np.array([[1, 2, 3, 4], [5, 6, 7, 8]], np.int32)
    gd = np.array([[1, 2, 2, 3], [1, 2, 3, 3]], np.float32)
    o = np.array([[1, 3, 2, 4], [5, 6, 7, 9]], np.int32)  # tie order inside; a different boundary member
    od = gd.copy()
    r = bench.parity_report(g, gd, o, od)
    assert r["identical_rows"] == 0.0 and r["identical_rows_up_to_ties"] == 1.0
    o2 = np.array([[1, 9, 2, 4], [5, 6, 7, 8]], np.int32)  # a different id below the boundary
    assert bench.parity_report(g, gd, o2, od)["identical_rows_up_to_ties"] == 0.5
