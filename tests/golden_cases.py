"""Load the golden fixtures written by tests/golden/make_golden.py.

Vectors are regenerated from the seeded mixture and checked against the
sha256 stored with the fixture, so that a change in the generator cannot
silently change the inputs the reference outputs belong to."""
from __future__ import annotations

import json
import os
from types import SimpleNamespace

import numpy as np

from mestrado_gb300.ivfdata import IVFPQData
from mestrado_gb300.synth import Mixture, digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["cfg1", "small", "m16"]
_cache: dict = {}


def load(name: str) -> SimpleNamespace:
    if name in _cache:
        return _cache[name]
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(z["meta"]))
    mx = Mixture(d=meta["d"], ncomp=meta["ncomp"], seed=meta["seed"])
    means = mx.means()
    base = mx.base(meta["nbase"], means)
    queries = mx.queries(meta["nq"], means)
    assert digest(base) == meta["sha_base"], "synthetic base drifted from the fixture"
    assert digest(queries) == meta["sha_queries"], "synthetic queries drifted from the fixture"
    ix = IVFPQData(coa=z["coa"], pq=z["pq"], list_off=z["list_off"].astype(np.int64),
                   ids=z["ids"], codes=z["codes"])
    ix.validate()
    out = SimpleNamespace(name=name, meta=meta, ix=ix, base=base, queries=queries,
                          z={k: z[k] for k in z.files if k != "meta"})
    _cache[name] = out
    return out
