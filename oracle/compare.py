"""TEST INFRASTRUCTURE ONLY -- tie-aware comparison of ranked id lists.

Two engines that compute the same distances can still return different ids
where distances tie: the reference orders ADC ties by whatever its qsort does
(sequential/yael_needs/sorting.c:34-37, 152-156) and heap ties by heap slot
(sorting.c:216-219). A difference is accepted only where it is explained by
a tie, and every such query is counted so that the tests can report it.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Report:
    nq: int = 0
    exact: int = 0
    tie: int = 0          # differs only inside groups of equal (within rtol) distances
    upstream_tie: int = 0  # differs because an earlier stage resolved a tie differently
    mismatch: list = dataclasses.field(default_factory=list)

    @property
    def ok(self) -> bool:
        return not self.mismatch

    def __str__(self) -> str:
        return (f"nq={self.nq} exact={self.exact} tie={self.tie} upstream_tie={self.upstream_tie} "
                f"mismatch={len(self.mismatch)} (first: {self.mismatch[:5]})")


def _close(a, b, rtol):
    same_inf = np.isinf(a) & np.isinf(b)
    return same_inf | (np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)))


def classify(a_ids, a_d, b_ids, b_d, rtol=0.0) -> str:
    """'exact' | 'tie' | 'mismatch' for one query's ascending lists."""
    a_ids = np.asarray(a_ids)
    b_ids = np.asarray(b_ids)
    a_d = np.asarray(a_d, np.float64)
    b_d = np.asarray(b_d, np.float64)
    if not np.array_equal(a_ids < 0, b_ids < 0):
        return "mismatch"
    valid = a_ids >= 0
    if rtol == 0.0:
        if not np.array_equal(a_d[valid], b_d[valid]):
            return "mismatch"
    elif not _close(a_d[valid], b_d[valid], rtol).all():
        return "mismatch"
    if np.array_equal(a_ids, b_ids):
        return "exact"
    if not valid.any():
        return "exact"
    last = max(a_d[valid][-1], b_d[valid][-1])
    for p in np.nonzero(a_ids != b_ids)[0]:
        v = a_d[p]
        tol = rtol * abs(v)
        lo, hi = v - tol, v + tol
        wa = valid & (a_d >= lo) & (a_d <= hi)
        wb = valid & (b_d >= lo) & (b_d <= hi)
        boundary = hi >= last - rtol * abs(last)
        if not boundary and set(a_ids[wa].tolist()) != set(b_ids[wb].tolist()):
            return "mismatch"
    return "tie"


def compare_ranked(a_ids, a_d, b_ids, b_d, rtol=0.0, upstream=None) -> Report:
    """Compare nq x k ranked lists. ``upstream`` (optional, length nq) marks
    queries whose input candidate sets already differed through a tie in an
    earlier stage; those count as ``upstream_tie`` when they differ."""
    r = Report(nq=len(a_ids))
    for q in range(len(a_ids)):
        c = classify(a_ids[q], a_d[q], b_ids[q], b_d[q], rtol)
        if c == "exact":
            r.exact += 1
        elif upstream is not None and upstream[q]:
            r.upstream_tie += 1
        elif c == "tie":
            r.tie += 1
        else:
            r.mismatch.append(q)
    return r


def set_differs(a_ids, b_ids):
    """Per query: do the two candidate lists hold different id sets?"""
    return np.array([set(x.tolist()) != set(y.tolist()) for x, y in zip(np.asarray(a_ids), np.asarray(b_ids))])
