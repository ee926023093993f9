"""The precision form's error bound, checked on the CPU.

The precision form keeps per sub-quantizer the approximate table entry
v_s = fma(-1/2, <r_s, c>, ||r_s||^2/4 + ||c||^2/4) in FP32 (the dot product
by fused multiply-adds), stored in FP16 with saturation, summed in FP32 and
scaled by 4. Its finalize re-scores only the candidates whose approximate
distance A is below (T0 + eps_q) / (1 - delta), relying on
E >= A (1 - delta) - eps_q for the exact distance E, with delta = 2^-9 and
eps_q = 2^-12 (max_probe ||r||^2 + sum_s max_c ||c_s||^2) + 2^-12.

Here the approximate distances are emulated in numpy for every (query, probe,
code row) of the golden m = 16 case (FP32 roundings as float32 operations, the
fused multiply-add as one rounding of the float64 product-sum, FP16 by
numpy's round-to-nearest-even conversion) and compared with the distance in
float64 to the same FP32 residual: the deviation must stay within a quarter
of delta and an eighth of eps_q, the margin the bound keeps for the FP32
rounding of the reference's own distance."""
import numpy as np

from tests import golden_cases

DELTA = 2.0 ** -9
EPS_REL = 2.0 ** -12
EPS_ABS = 2.0 ** -12


def _approx(r, pq, codes):
    """Approximate distances of code rows `codes` (n x m) for the FP32 residual r (d,)."""
    m, ks, ds = pq.shape
    f32 = np.float32
    acc = np.zeros(len(codes), np.float32)
    for s in range(m):
        rs = r[s * ds:(s + 1) * ds]
        f = f32(0.0)
        for t in range(ds):  # the reference's sequential float norm
            f = f32(f + f32(rs[t] * rs[t]))
        c = pq[s][codes[:, s]]  # n x ds
        cn = (c.astype(np.float64) ** 2).sum(axis=1).astype(np.float32)  # RN32 of the double norm
        dt = np.zeros(len(codes), np.float64)
        for t in range(ds):  # fused multiply-add chain: one rounding per step
            dt = (rs[t].astype(np.float64) * c[:, t].astype(np.float64) + dt).astype(np.float32).astype(np.float64)
        base = (f32(0.25) * f + (f32(0.25) * cn)).astype(np.float32)
        v = (-0.5 * dt + base.astype(np.float64)).astype(np.float32)
        h = np.clip(v, -65504.0, 65504.0).astype(np.float16)
        acc = (acc + h.astype(np.float32)).astype(np.float32)
    return acc * np.float32(4.0)


def test_bound_holds_with_margin_on_golden_m16():
    g = golden_cases.load("m16")
    ix, q = g.ix, g.queries
    pq = ix.pq
    cmax = sum(float((pq[s].astype(np.float64) ** 2).sum(axis=1).max()) for s in range(pq.shape[0]))
    worst_rel = 0.0
    for qi in range(0, len(q), 5):
        x = q[qi]
        d2 = ((ix.coa.astype(np.float64) - x) ** 2).sum(axis=1)
        probes = np.argsort(d2)[: g.meta["w"]]
        r2max = max(float(((x - ix.coa[l]).astype(np.float32).astype(np.float64) ** 2).sum()) for l in probes)
        eps = EPS_REL * (r2max + cmax) + EPS_ABS
        for l in probes:
            lo, hi = ix.list_off[l], ix.list_off[l + 1]
            if hi == lo:
                continue
            r = (x - ix.coa[l]).astype(np.float32)
            codes = ix.codes[lo:hi]
            a = _approx(r, pq, codes).astype(np.float64)
            rec = np.concatenate([pq[s][codes[:, s]] for s in range(pq.shape[0])], axis=1).astype(np.float64)
            exact = ((r.astype(np.float64) - rec) ** 2).sum(axis=1)
            # E >= A (1 - delta) - eps with the margins: A (1 - delta/4) - eps/8 <= E
            assert np.all(exact >= a * (1.0 - DELTA / 4) - eps / 8), (qi, int(l))
            worst_rel = max(worst_rel, float(np.max(np.abs(a - exact) / np.maximum(exact, 1.0))))
    print(f"largest relative deviation {worst_rel:.3e} (delta {DELTA:.3e})")
    assert worst_rel < DELTA / 2
