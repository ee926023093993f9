"""TEST INFRASTRUCTURE ONLY -- build recipe for the CPU oracle.

Two shared libraries come out of this recipe:

* ``oracle/liboracle.so`` -- the plain-C restatement of the search path
  (``ivfpq_oracle.c``); built on every machine (x86 here, Arm on the GPU
  host).
* ``oracle/_ref/libref_seq.so`` -- the reference's own sequential IVF-PQ
  code compiled from its sources where they lie, plus ``ref_harness.cpp``
  (C entry points) and ``ref_blas.c`` (a netlib-order sgemm/sgemv, since the
  reference ships no BLAS). Built only where the reference tree exists.

Both compile with ``-ffp-contract=off`` so that no multiply-add is fused and
the float rounding is the same on x86 and Arm.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference tree lies: MESTRADO_REFERENCE, else the mount of the build container. This recipe
# is the one file that names it; on a machine without the tree (the GPU host) nothing is built from it.
REF_ROOT = os.environ.get("MESTRADO_REFERENCE", "/root/reference")
REF_SEQ = os.path.join(REF_ROOT, "sequential")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libref_seq.so")

FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC"]

# the reference files on the search path and what they need to link
REF_C = ["vector.c", "matrix.c", "nn.c", "kmeans.c", "sorting.c", "binheap.c", "machinedeps.c"]
REF_CXX = [
    "pq-utils/pq_new.cpp",
    "pq-utils/pq_assign.cpp",
    "pq-utils/pq_search.cpp",
    "pq-utils/pq_test_load_vectors.cpp",
    "ivf_pq/ivf_new.cpp",
    "ivf_pq/ivf_assign.cpp",
    "ivf_pq/ivf_search.cpp",
]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "ivfpq_oracle.c")
    hdr = os.path.join(HERE, "ivfpq_oracle.h")
    if force or _stale(LIB, [src, hdr, __file__]):
        tmp = LIB + f".tmp{os.getpid()}"
        _run(["gcc", "-std=c11", *FP_FLAGS, "-fopenmp", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def reference_available() -> bool:
    return os.path.isdir(REF_SEQ)


def build_reference(force: bool = False) -> str | None:
    """Compile the reference's sequential search into oracle/_ref (or None)."""
    if not reference_available():
        return None
    ours = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_blas.c"), __file__]
    if not force and not _stale(REF_LIB, ours) and os.path.exists(REF_LIB):
        return REF_LIB
    os.makedirs(REF_DIR, exist_ok=True)
    objs = []
    cflags = [*FP_FLAGS, "-DFINTEGER=int", "-w"]
    for f in REF_C:
        o = os.path.join(REF_DIR, f.replace("/", "_") + ".o")
        _run(["gcc", *cflags, "-c", os.path.join(REF_SEQ, "yael_needs", f), "-o", o])
        objs.append(o)
    for f in REF_CXX:
        o = os.path.join(REF_DIR, f.replace("/", "_") + ".o")
        _run(["g++", "-std=gnu++11", *cflags, "-I", REF_SEQ, "-c", os.path.join(REF_SEQ, f), "-o", o])
        objs.append(o)
    o = os.path.join(REF_DIR, "ref_harness.o")
    _run(["g++", "-std=gnu++11", *cflags, "-I", REF_SEQ, "-c", os.path.join(HERE, "ref_harness.cpp"), "-o", o])
    objs.append(o)
    o = os.path.join(REF_DIR, "ref_blas.o")
    _run(["gcc", *cflags, "-c", os.path.join(HERE, "ref_blas.c"), "-o", o])
    objs.append(o)
    tmp = REF_LIB + f".tmp{os.getpid()}"
    _run(["g++", "-shared", "-o", tmp, *objs, "-lm", "-lpthread", "-Wl,--no-undefined"])
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
