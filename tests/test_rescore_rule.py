"""The precision form's re-score rule, restated in numpy and checked on the CPU.

The GPU kernels (rs_first_kernel .. rs_order_kernel in scan_persistent.cu) keep the k_sel best
approximate keys of a query, re-score the kk best of them exactly (T0 = their largest exact
distance), then every other kept candidate whose approximate distance is below
tau = (T0 + eps) / (1 - delta), and call the query proven when the kept set held every candidate
below tau. The rule is sound when E >= A (1 - delta) - eps for every candidate (the error bound
that tests/test_mixed_bound.py checks against the FP16 tables): then a proven query's exact top-kk
over all its candidates is the top-kk of the re-scored set. Here candidates are drawn with
approximate distances inside that error model, including dense groups around the kk-th distance,
and the rule is run and checked query by query."""
import numpy as np

DELTA = 2.0 ** -9


def rescore(A, E, pos, ksel, kk, eps):
    """(re-scored indices, proven) for one query: A, E the approximate and exact distances, pos the
    (unique) positions that break ties, ksel the kept selection, kk the results wanted."""
    akey = np.lexsort((pos, A))  # ascending (A, position)
    kept = akey[:ksel]
    first = kept[:kk]
    t0 = max(0.0, float(E[first].max())) if len(first) else 0.0
    tau = (t0 + eps) / (1.0 - DELTA) * (1.0 + 2.0 ** -20)
    second = [i for i in kept[kk:] if A[i] < tau]
    proven = len(A) <= ksel or float(A[kept].max()) >= tau
    return np.concatenate([first, np.array(second, dtype=first.dtype)]), proven


def topk(E, pos, idx, kk):
    order = idx[np.lexsort((pos[idx], E[idx]))]
    return order[:kk]


def draw(rng, n, eps):
    """Exact distances with a dense group, approximate ones anywhere inside the error model."""
    E = rng.uniform(1e3, 5e4, n)
    E[: n // 8] = rng.normal(1.5e4, 30.0, n // 8)  # many candidates near one distance
    E = np.round(E, 1)  # ties in the exact distances
    lo = E * (1.0 - DELTA) - eps  # A may lie anywhere with A (1 - delta) - eps <= E
    hi = (E + eps) / (1.0 - DELTA)
    A = rng.uniform(np.minimum(lo, hi), hi)
    return A.astype(np.float64), E.astype(np.float64)


def test_proven_queries_return_the_exact_top_k():
    rng = np.random.default_rng(11)
    eps = 8.0
    proven_n = 0
    for trial in range(300):
        n = int(rng.integers(20, 4000))
        kk = int(rng.choice([1, 10, 100, 1000]))
        kk = min(kk, n)
        ksel = min(max(2 * kk, kk + 64), 4096)
        A, E = draw(rng, n, eps)
        pos = rng.permutation(n).astype(np.int64)
        idx, proven = rescore(A, E, pos, ksel, kk, eps)
        if proven:
            proven_n += 1
            want = topk(E, pos, np.arange(n), kk)
            got = topk(E, pos, idx, kk)
            np.testing.assert_array_equal(got, want, err_msg=f"trial {trial}: n={n} kk={kk}")
    assert proven_n > 250, proven_n  # the floor k + 64 and the 2k selection prove almost all


def test_a_short_selection_is_not_proven():
    """With the kept selection cut to kk (no margin) most queries cannot be proven, and a proven one
    is still exact."""
    rng = np.random.default_rng(12)
    eps = 8.0
    unproven = 0
    for trial in range(100):
        n, kk = 2000, 100
        A, E = draw(rng, n, eps)
        pos = rng.permutation(n).astype(np.int64)
        idx, proven = rescore(A, E, pos, kk, kk, eps)
        if proven:
            np.testing.assert_array_equal(topk(E, pos, idx, kk), topk(E, pos, np.arange(n), kk))
        else:
            unproven += 1
    assert unproven > 90, unproven
