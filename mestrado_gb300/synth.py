"""Seeded synthetic inputs with the shape of the reference's SIFT-style runs.

The reference measures on TEXMEX/BIGANN files (SIFT1M/1B), loaded by
``sequential/pq-utils/pq_test_load_vectors.cpp:46-140``; those sets are not
available, so a Gaussian mixture with the same dimensionality and byte range
stands in for them:

* ``ncomp`` component means drawn uniformly in ``[0, 120]^d``;
* each vector picks a component (uniformly, or with Zipf-distributed
  weights) and adds N(0, sigma^2) noise per dimension (sigma = 20);
* values are clipped to ``[0, 255]`` and rounded to integers, stored as
  float32 -- like the byte-valued SIFT descriptors.

Streams (means, base, train, queries) come from independent children of
one ``numpy.random.SeedSequence`` so that each set is reproducible on its
own and in chunks.
"""
from __future__ import annotations

import dataclasses

import numpy as np

STREAM_MEANS, STREAM_BASE, STREAM_TRAIN, STREAM_QUERY, STREAM_LABEL = range(5)


@dataclasses.dataclass(frozen=True)
class Mixture:
    d: int = 128
    ncomp: int = 64
    seed: int = 0
    sigma: float = 20.0
    mean_hi: float = 120.0
    zipf: float | None = None  # exponent of the component weights (None = uniform)

    def _rng(self, stream: int, chunk: int = 0) -> np.random.Generator:
        ss = np.random.SeedSequence([self.seed, stream, chunk])
        return np.random.Generator(np.random.PCG64(ss))

    def means(self) -> np.ndarray:
        return self._rng(STREAM_MEANS).uniform(0.0, self.mean_hi, (self.ncomp, self.d)).astype(np.float32)

    def weights(self) -> np.ndarray | None:
        if self.zipf is None:
            return None
        w = 1.0 / np.arange(1, self.ncomp + 1, dtype=np.float64) ** self.zipf
        return w / w.sum()

    def sample(self, stream: int, n: int, chunk: int = 0, means: np.ndarray | None = None) -> np.ndarray:
        """n vectors of one stream (chunk selects an independent sub-stream)."""
        if means is None:
            means = self.means()
        rng = self._rng(stream, chunk)
        w = self.weights()
        if w is None:
            lab = rng.integers(0, self.ncomp, n)
        else:
            lab = rng.choice(self.ncomp, size=n, p=w)
        out = means[lab]
        out += np.float32(self.sigma) * rng.standard_normal((n, self.d), dtype=np.float32)
        np.clip(out, 0.0, 255.0, out=out)
        np.rint(out, out=out)
        return out.astype(np.float32, copy=False)

    def base(self, n: int, means: np.ndarray | None = None, chunk_rows: int = 1 << 20) -> np.ndarray:
        """Base vectors, generated in independent chunks of ``chunk_rows``."""
        if means is None:
            means = self.means()
        out = np.empty((n, self.d), np.float32)
        for c, s in enumerate(range(0, n, chunk_rows)):
            e = min(n, s + chunk_rows)
            out[s:e] = self.sample(STREAM_BASE, e - s, chunk=c, means=means)
        return out

    def train(self, n: int, means: np.ndarray | None = None) -> np.ndarray:
        return self.sample(STREAM_TRAIN, n, means=means)

    def queries(self, n: int, means: np.ndarray | None = None) -> np.ndarray:
        return self.sample(STREAM_QUERY, n, means=means)


def digest(a: np.ndarray) -> str:
    """sha256 of an array's bytes (pins generated inputs in the fixtures)."""
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
