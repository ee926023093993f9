"""Host-side IVF-PQ index data, in the layout the GPU engine uploads.

The reference keeps one ``ivf_t`` per inverted list (``ids``, ``idstam``,
``codes`` as an int32 ``matI`` of n x nsq; sequential/ivf_pq/myIVF.h:15-27)
plus an ``ivfpq_t`` with the coarse centroids and a ``pqtipo`` holding
``nsq`` arrays of ``ks x ds`` sub-quantizer centroids
(sequential/pq-utils/pq_new.h:26-33). Here the same content is flattened:

* ``coa``      C x d float32 coarse centroids (``ivfpq.coa_centroids``)
* ``pq``       m x ks x ds float32 (``pq.centroids[s]`` stacked)
* ``list_off`` C+1 int64 offsets; list l is rows ``list_off[l]:list_off[l+1]``
* ``ids``      n int32 base ids, list-contiguous (``ivf[l].ids``)
* ``codes``    n x m uint8 (``ivf[l].codes``; exact when ks <= 256)
* ``pq2``, ``codes2`` (optional) refinement quantizer of the residual error
  x - y_list - c1(codes): m2 x 256 x d/m2 float32 and n x m2 uint8 codes in
  the row order of ``codes`` (no counterpart in the reference)
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class IVFPQData:
    coa: np.ndarray
    pq: np.ndarray
    list_off: np.ndarray
    ids: np.ndarray
    codes: np.ndarray
    pq2: np.ndarray | None = None
    codes2: np.ndarray | None = None

    @property
    def d(self) -> int:
        return int(self.coa.shape[1])

    @property
    def coarsek(self) -> int:
        return int(self.coa.shape[0])

    @property
    def m(self) -> int:
        return int(self.pq.shape[0])

    @property
    def ks(self) -> int:
        return int(self.pq.shape[1])

    @property
    def ds(self) -> int:
        return int(self.pq.shape[2])

    @property
    def n(self) -> int:
        return int(self.ids.shape[0])

    def list_sizes(self) -> np.ndarray:
        return np.diff(self.list_off).astype(np.int32)

    def validate(self) -> None:
        C, d = self.coa.shape
        m, ks, ds = self.pq.shape
        if m * ds != d:
            raise ValueError(f"pq shape {self.pq.shape} does not split d={d}")
        if not 0 < ks <= 256:
            raise ValueError(f"ks={ks} needs uint8 codes (ks <= 256)")
        if self.list_off.shape != (C + 1,) or self.list_off[0] != 0 or np.any(np.diff(self.list_off) < 0):
            raise ValueError("list_off must be C+1 non-decreasing offsets from 0")
        n = int(self.list_off[-1])
        if self.ids.shape != (n,) or self.codes.shape != (n, m):
            raise ValueError("ids / codes do not match list_off")
        if n and int(self.codes.max()) >= ks:
            raise ValueError("code value >= ks")
        if (self.pq2 is None) != (self.codes2 is None):
            raise ValueError("pq2 and codes2 go together")
        if self.pq2 is not None:
            m2 = self.pq2.shape[0]
            if self.pq2.shape != (m2, 256, d // m2) or m2 * (d // m2) != d:
                raise ValueError(f"pq2 shape {self.pq2.shape}")
            if self.codes2.shape != (n, m2):
                raise ValueError("codes2 does not match the codes")

    @staticmethod
    def from_reference_lists(coa, pq, list_sizes, ids, codes_i32) -> "IVFPQData":
        """Build from the reference's per-list content: int32 codes n x nsq
        concatenated in list order, as ``ivfpq_assign`` produces them
        (sequential/ivf_pq/ivf_assign.cpp:24-42)."""
        sizes = np.asarray(list_sizes, np.int64)
        off = np.zeros(len(sizes) + 1, np.int64)
        np.cumsum(sizes, out=off[1:])
        codes = np.asarray(codes_i32)
        if codes.size and (codes.min() < 0 or codes.max() > 255):
            raise ValueError("reference codes outside 0..255 cannot be held as uint8 (ks > 256)")
        out = IVFPQData(
            coa=np.ascontiguousarray(coa, np.float32),
            pq=np.ascontiguousarray(pq, np.float32),
            list_off=off,
            ids=np.ascontiguousarray(ids, np.int32),
            codes=np.ascontiguousarray(codes, np.uint8),
        )
        out.validate()
        return out

    def save(self, path: str) -> None:
        extra = {} if self.pq2 is None else dict(pq2=self.pq2, codes2=self.codes2)
        np.savez_compressed(path, coa=self.coa, pq=self.pq, list_off=self.list_off, ids=self.ids, codes=self.codes,
                            **extra)

    def save_dir(self, path: str) -> None:
        """Uncompressed arrays, one .npy file each, under directory `path` (fast for GB-sized
        indexes; written to a temporary name first and renamed, so a reader never sees half)."""
        import os

        tmp = f"{path}.tmp{os.getpid()}"
        os.makedirs(tmp, exist_ok=True)
        arrays = dict(coa=self.coa, pq=self.pq, list_off=self.list_off, ids=self.ids, codes=self.codes)
        if self.pq2 is not None:
            arrays.update(pq2=self.pq2, codes2=self.codes2)
        for k, v in arrays.items():
            np.save(os.path.join(tmp, f"{k}.npy"), v)
        os.replace(tmp, path)

    @staticmethod
    def load_dir(path: str) -> "IVFPQData":
        import os

        def get(k):
            f = os.path.join(path, f"{k}.npy")
            return np.load(f) if os.path.exists(f) else None

        out = IVFPQData(coa=get("coa"), pq=get("pq"), list_off=get("list_off").astype(np.int64), ids=get("ids"),
                        codes=get("codes"), pq2=get("pq2"), codes2=get("codes2"))
        out.validate()
        return out

    @staticmethod
    def load(path: str) -> "IVFPQData":
        z = np.load(path)
        out = IVFPQData(coa=z["coa"], pq=z["pq"], list_off=z["list_off"].astype(np.int64),
                        ids=z["ids"].astype(np.int32), codes=z["codes"].astype(np.uint8),
                        pq2=z["pq2"] if "pq2" in z else None,
                        codes2=z["codes2"].astype(np.uint8) if "codes2" in z else None)
        out.validate()
        return out
