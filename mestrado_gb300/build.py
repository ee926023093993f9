"""Build the engine's shared library, in-tree, for sm_103a.

    python -m mestrado_gb300.build            # -> mestrado_gb300/lib/libgbivf.so

Translation units compile in parallel with one -gencode (sm_103a only) and
link with nvcc into one shared library exporting the C ABI of
include/gbivf.h. Host code compiles with -ffp-contract=off so that the
index-constant norms round exactly like the reference's.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libgbivf.so")
# C++ shims with the reference's own signatures, linked against libgbivf.so
SHIMS = {"libgbivf_refcompat_seq.so": "refcompat_seq.cpp", "libgbivf_refcompat_par2.so": "refcompat_par2.cpp"}
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["kernels.cu", "scan_persistent.cu", "scan_lists.cu", "coarse_mma.cu", "coarse_filter.cu", "coarse_gemm.cu", "build_gpu.cu", "api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I", INCLUDE,
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    out.append(os.path.abspath(__file__))
    return out


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    outs = [LIB] + [os.path.join(LIBDIR, n) for n in SHIMS]
    if not force and all(os.path.exists(o) for o in outs):
        t = min(os.path.getmtime(o) for o in outs)
        if all(os.path.getmtime(p) <= t for p in _deps()):
            return LIB
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    objs = [os.path.join(LIBDIR, s.replace(".cu", ".o")) for s in SOURCES]
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], extra), zip(SOURCES, objs)))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for name, src in SHIMS.items():
        out = os.path.join(LIBDIR, name)
        tmp = out + f".tmp{os.getpid()}"
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", INCLUDE, "-o", tmp, os.path.join(CSRC, src),
               "-L", LIBDIR, "-lgbivf", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"shim build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
