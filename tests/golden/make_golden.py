"""Write the golden fixtures of the IVF-PQ search path from the reference itself.

Runs only where the reference sources exist (it links them through
``oracle/_ref/libref_seq.so``). For each case it:

1. generates base / train / query vectors with ``mestrado_gb300.synth``
   (their sha256 is stored, the vectors are not);
2. trains and fills the index with the reference's ``ivfpq_new`` +
   ``ivfpq_assign`` (sequential/ivf_test.cpp:52-59);
3. records the reference's coarse k-min and ADC k-min
   (sequential/ivf_pq/ivf_search.cpp:37-107), its final ``ivfpq_search``
   ids for each (k, kl), and the exact re-rank distance of every returned id;
4. for the flat case, trains a PQ with ``pq_new``/``pq_assign`` and records
   ``pq_search`` (sequential/pq_test.cpp:45-67).

Each case runs in a fresh process: ``ivfpq_assign`` keeps its list array in
a static (sequential/ivf_pq/ivf_assign.cpp:19).

    python tests/golden/make_golden.py            # all cases
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    # the reference's CPU-runnable configuration: 10k base, 5k train, 100
    # queries, 64-component mixture, 16 lists, m=8 x 256, w=4, k=100
    "cfg1": dict(d=128, ncomp=64, seed=0, nbase=10000, ntrain=5000, nq=100, C=16, m=8, w=4,
                 searches=[(100, 100), (10, 100), (1, 50)], flat=dict(k=100)),
    # many small and empty lists, short candidate lists (L < kl), d=32, m=4
    "small": dict(d=32, ncomp=8, seed=1, nbase=600, ntrain=600, nq=20, C=64, m=4, w=3,
                  searches=[(5, 40), (3, 3)]),
    # m=16 sub-quantizers (ds=8), uneven lists
    "m16": dict(d=128, ncomp=40, seed=2, nbase=8000, ntrain=4000, nq=50, C=32, m=16, w=8,
                searches=[(50, 100)]),
}


def run_case(name: str) -> None:
    import oracle
    from mestrado_gb300.ivfdata import IVFPQData
    from mestrado_gb300.synth import Mixture, digest

    c = CASES[name]
    mx = Mixture(d=c["d"], ncomp=c["ncomp"], seed=c["seed"])
    means = mx.means()
    base = mx.base(c["nbase"], means)
    train = mx.train(c["ntrain"], means)
    q = mx.queries(c["nq"], means)
    coa, pq, sizes, ids, codes = oracle.ref_build_index(train, base, c["C"], c["m"])
    ix = IVFPQData.from_reference_lists(coa, pq, sizes, ids, codes)
    klmax = max(kl for _, kl in c["searches"])
    co, cd, ai, ad = oracle.ref_adc_stage(ix, q, klmax, c["w"])
    out = dict(
        meta=np.array(json.dumps(dict(c, name=name, sha_base=digest(base), sha_train=digest(train),
                                      sha_queries=digest(q)))),
        coa=ix.coa, pq=ix.pq, list_off=ix.list_off, ids=ix.ids, codes=ix.codes,
        ref_coaidx=co, ref_coadis=cd, ref_adc_ids=ai, ref_adc_dis=ad,
    )
    for k, kl in c["searches"]:
        r = oracle.ref_ivfpq_search(ix, q, base, k, kl, c["w"])
        rd = np.array([[oracle.ref_l2(base[i], q[j]) if i >= 0 else np.inf for i in r[j]]
                       for j in range(len(q))], np.float32)
        out[f"ref_ids_k{k}_kl{kl}"] = r
        out[f"ref_dis_k{k}_kl{kl}"] = rd
    if "flat" in c:
        fpq, fcodes = oracle.ref_build_pq(train, base, c["m"])
        fd, fi = oracle.ref_pq_search(c["d"], c["m"], fpq, fcodes, q, c["flat"]["k"])
        out.update(flat_pq=fpq, flat_codes=fcodes.astype(np.uint8), ref_flat_dis=fd, ref_flat_ids=fi)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: lists {sizes.min()}..{sizes.max()} ({(sizes == 0).sum()} empty)")


def main() -> None:
    if len(sys.argv) > 1 and sys.argv[1] == "--case":
        run_case(sys.argv[2])
        return
    for name in (sys.argv[1:] or CASES):
        subprocess.run([sys.executable, __file__, "--case", name], check=True)


if __name__ == "__main__":
    main()
