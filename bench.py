#!/usr/bin/env python
"""Benchmark of the IVF-PQ search path (the reference's ivfpq_search and its
batched GPU replacement) on GB300.

Headline (default, ``--config cfg4``): the workload the metric is quoted on --
batched search of 32,768 queries over a 100M-vector index (d = 128,
Zipf(1.1)-sized mixture components, C = 262,144 lists, m = 16 x 256 codes),
each query with its own nprobe (log-uniform in 1..256) and k (from
{1, 10, 100, 1000}), in two forms:

* plain: FP32 throughout, the reference's arithmetic (the drop-in);
* mixed: BF16 tensor-core coarse stage with an FP32 re-check of every
  centroid within the error margin (the same probe lists), FP16 PQ tables
  summed in FP32, the candidates within the tables' error bound re-scored
  exactly (the same ids on every query the engine proves; the count of the
  others is reported as ``unproven_queries``).

A step is one search of the whole batch, replayed as a CUDA graph.

* ``value``: mixed-form QPS with queries, index and outputs resident in HBM,
  CUDA events around each replay on the launching stream, L2 flushed (a 256 MB
  write) between steps outside the timed events; ``forms`` holds both forms,
  their ratio and recall@100 (equal by construction: identical ids).
* ``e2e``: the same batch through the host C ABI (gbivf_search_batched):
  queries, nprobe and k copied from pinned host memory, ids and distances
  copied back, per step.
* ``roofline``: the dominant kernel of the mixed step (the list-centric ADC
  scan): algorithmic bytes (sum over queries of the codes of the probes it
  scans, n_l * m) over its CUDA-event time, against the measured HBM copy
  bandwidth; ``traffic`` from the committed ncu summary.
* ``cpu_baseline``: the CPU oracle (the plain-C restatement of the
  reference's search) on all host cores, on a sample of the same queries.
* ``parity``: the plain form against the oracle on a sample of queries (ids
  and distance bits), the mixed form against the plain form on all queries.
* ``sub``: the 1M drop-in workload (``ivfpq_search`` with re-rank, all
  10,000 queries checked against the oracle, the reference's OpenMP
  ``core_cpu`` timed), the 10M workload (C = 65,536, w = 32, k = 100) and
  the 1B workload (refinement re-rank).

``--impl reference`` times the oracle alone on the headline workload, in
steps of a bounded sample of its queries, with every host thread. The index
it searches is built by the engine's GPU index builder (input preparation;
nothing of the engine runs in its timed region).

The synthetic mixture stands in for the reference's SIFT/BIGANN runs.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import re
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "QPS at equal recall@100, batched mixed-prec vs plain FP32 GPU; ADC scan GB/s"
HEADLINE = "cfg4"

# Host-built indexes: the drop-in workloads of the reference's own CPU runs.
CONFIGS = {
    "cfg2": dict(d=128, ncomp=1024, seed=0, nbase=1_000_000, ntrain=100_000, nq=10_000, C=1024, m=8,
                 w=16, k=100, kl=100, rerank=True, train_iters=10),
    "cfg1": dict(d=128, ncomp=64, seed=0, nbase=10_000, ntrain=5_000, nq=100, C=16, m=8,
                 w=4, k=100, kl=100, rerank=True, train_iters=10),
}

# Larger workloads, generated and indexed on the GPU (gbivf_generate_mixture,
# gbivf_kmeans, gbivf_pq_encode): the precision form against the plain one.
LARGE = {
    # billion scale with re-rank by refinement codes; the base is generated, assigned and encoded in
    # chunks and never held (1B x 128 floats is 512 GB)
    "cfg5": dict(d=128, ncomp=16384, seed=0, zipf=None, nbase=1_000_000_000, ntrain=2_621_440, nq=10_000,
                 C=262144, m=8, m2=8, w=64, k=100, kl=1000, uneven=False, train_iters=6, recall_q=100,
                 stream=True),
    # the 100M workload's shape at 1/5 scale (20M base, 65,536 Zipf lists, m = 16, uneven nprobe / k)
    "cfg4s": dict(d=128, ncomp=65536, seed=0, zipf=1.1, nbase=20_000_000, ntrain=655_360, nq=8192,
                  C=65536, m=16, w=256, k=1000, uneven=True, train_iters=4, recall_q=256),
    # 10M base, 4,096-component mixture, 65,536 lists, m = 8, 10k queries, w = 32, k = 100
    "cfg3": dict(d=128, ncomp=4096, seed=0, zipf=None, nbase=10_000_000, ntrain=1_000_000, nq=10_000,
                 C=65536, m=8, w=32, k=100, uneven=False, train_iters=8, recall_q=1000),
    # 100M base, Zipf(1.1) cluster sizes over 262,144 lists, m = 16, 32,768 queries with
    # nprobe log-uniform in [1, 256] and k from {1, 10, 100, 1000}
    "cfg4": dict(d=128, ncomp=262144, seed=0, zipf=1.1, nbase=100_000_000, ntrain=2_621_440, nq=32768,
                 C=262144, m=16, w=256, k=1000, uneven=True, train_iters=6, recall_q=256),
}

CACHE = os.environ.get("MESTRADO_GB300_CACHE", "/tmp/mestrado_gb300_cache")
L2_FLUSH_BYTES = 256 << 20


def workload_name(c):
    return (f"ivfpq_search plain fp32: base {c['nbase']:,} x d={c['d']} ({c['ncomp']}-component mixture), "
            f"C={c['C']} lists, m={c['m']}x256, {c['nq']:,} queries/step, w={c['w']}, k={c['k']}, "
            f"rerank kl={c['kl']}")


def large_workload(name, c):
    return (f"{name}: base {c['nbase']:,} x d=128 ({c['ncomp']}-component mixture"
            f"{', Zipf ' + str(c['zipf']) + ' component sizes' if c['zipf'] else ''}), C={c['C']:,} lists, "
            f"m={c['m']}x256, {c['nq']:,} queries/step, "
            + (f"nprobe log-uniform 1..{c['w']}, k in {{1,10,100,1000}}" if c["uneven"] else f"w={c['w']}, k={c['k']}"))


def large_config(name, c):
    """The config dict of a large workload: the same in the engine's arm and the reference arm."""
    return {"workload": large_workload(name, c), "queries_per_step": c["nq"],
            "l2": "flushed between steps (256 MB write)",
            "index": "built on the GPU by the engine's index builder (k-means with FP64 centroid sums, PQ "
                     "training and encoding); input preparation, outside every timed region"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def ncpu():
    return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------

def make_inputs(c, rank=0):
    """(index data, base, queries): host-built, cached on local disk by config."""
    from mestrado_gb300.ivfdata import IVFPQData
    from mestrado_gb300.synth import STREAM_QUERY, Mixture
    from mestrado_gb300.train import build_index

    key = hashlib.sha1(json.dumps({k: c[k] for k in sorted(c)}, sort_keys=True).encode()).hexdigest()[:12]
    os.makedirs(CACHE, exist_ok=True)
    ipath = os.path.join(CACHE, f"index_{key}.npz")
    mx = Mixture(d=c["d"], ncomp=c["ncomp"], seed=c["seed"])
    means = mx.means()
    base = mx.base(c["nbase"], means)
    # each rank searches its own query batch (weak scaling)
    queries = mx.sample(STREAM_QUERY, c["nq"], chunk=rank, means=means)
    if os.path.exists(ipath):
        ix = IVFPQData.load(ipath)
    else:
        t = time.time()
        train = mx.train(c["ntrain"], means)
        ix = build_index(train, base, c["C"], c["m"], niter=c["train_iters"], seed=c["seed"])
        tmp = ipath + f".{os.getpid()}.npz"
        ix.save(tmp)
        os.replace(tmp, ipath)
        log(f"index built in {time.time() - t:.1f}s")
    return ix, base, queries, key


def large_inputs(name, c, dev, rank=0, dist=None):
    """(GPU mixture, host index, device queries, build seconds or None): the index is built on the
    GPU once per machine and cached on local disk (rank 0 builds, the other ranks wait and load)."""
    import torch

    from mestrado_gb300.gpu_build import GpuMixture, build_index_gpu
    from mestrado_gb300.ivfdata import IVFPQData
    from mestrado_gb300.synth import Mixture

    gm = GpuMixture(Mixture(d=c["d"], ncomp=c["ncomp"], seed=c["seed"], zipf=c["zipf"]), device=dev)
    key = hashlib.sha1(json.dumps({k: c[k] for k in sorted(c)}, sort_keys=True).encode()).hexdigest()[:12]
    path = os.path.join(CACHE, f"{name}_{key}")
    t_build, ix = None, None
    if rank == 0 and not os.path.isdir(path):
        t0 = time.time()
        base = gm.generate(c["nbase"], stream_id=1)
        train = gm.generate(c["ntrain"], stream_id=2)
        ix = build_index_gpu(base, train, c["C"], c["m"], niter=c["train_iters"], seed=c["seed"])
        del base, train
        torch.cuda.empty_cache()
        t_build = time.time() - t0
        os.makedirs(CACHE, exist_ok=True)
        ix.save_dir(path)
        sizes = ix.list_sizes()
        log(f"{name}: index built in {t_build:.1f}s; lists {sizes.min()}..{sizes.max()}")
    if dist is not None:
        dist.barrier()
    if ix is None:
        ix = IVFPQData.load_dir(path)
    queries = gm.generate(c["nq"], stream_id=3, row0=rank * c["nq"])
    return gm, ix, queries, t_build


def batch_shape(c, nq):
    """Per-query nprobe and k of a large workload (seeded; uniform where the workload is)."""
    rng = np.random.default_rng(c["seed"] + 17)
    if c["uneven"]:
        wq = np.clip(np.floor(np.exp(rng.uniform(0.0, np.log(c["w"] + 1), nq))), 1, c["w"]).astype(np.int32)
        kq = rng.choice([1, 10, 100, 1000], nq).astype(np.int32)
    else:
        wq = np.full(nq, c["w"], np.int32)
        kq = np.full(nq, c["k"], np.int32)
    return wq, kq


def ground_truth(base, queries, k, key, device):
    """Exact FP64 brute-force top-k on the GPU (evaluation only)."""
    import torch

    path = os.path.join(CACHE, f"gt_{key}_{hashlib.sha1(queries.tobytes()).hexdigest()[:8]}_{k}.npy")
    if os.path.exists(path):
        return np.load(path)
    b = torch.from_numpy(base).to(device, torch.float64)
    bn = (b * b).sum(1)
    out = np.empty((len(queries), k), np.int64)
    for s in range(0, len(queries), 1024):
        q = torch.from_numpy(queries[s:s + 1024]).to(device, torch.float64)
        dist = (q * q).sum(1, keepdim=True) + bn[None, :] - 2.0 * (q @ b.T)
        out[s:s + len(q)] = torch.topk(dist, k, dim=1, largest=False).indices.cpu().numpy()
    del b
    np.save(path, out)
    return out


def stage_split(gi):
    """Stage times of the index's last profiled search: coarse, scan (scan kernel + finalize) and the
    two parts of the scan."""
    cm, sk, fm = gi.last_stages_ms()
    return {"coarse": cm, "scan": sk + fm, "scan_kernel": sk, "finalize": fm}


def recall_report(ids, gt, k):
    hits = np.array([len(set(a[a >= 0].tolist()) & set(b[:k].tolist())) for a, b in zip(ids, gt)])
    # R@r as the reference prints it: share of queries whose true 1-NN is in the top r
    # (sequential/pq-utils/pq_test_compute_stats.cpp:76-149)
    r_at = {f"R@{r}": float(np.mean([(gt[i, 0] in ids[i, :r]) for i in range(len(ids))])) for r in (1, 10, 100)
            if r <= ids.shape[1]}
    return {f"recall@{k}": float(hits.mean() / k), **r_at}


def packed_recall(ids, off, kq, gt, nsample):
    """recall@k_q per query (k_q its own k) and recall@100 over the queries with k_q >= 100 (their
    first 100 results against the 100 exact nearest), on the first nsample queries."""
    at_k, at_100 = [], []
    for i in range(nsample):
        row = ids[off[i]:off[i] + kq[i]]
        at_k.append(len(set(row[row >= 0].tolist()) & set(gt[i, :kq[i]].tolist())) / kq[i])
        if kq[i] >= 100:
            r = row[:100]
            at_100.append(len(set(r[r >= 0].tolist()) & set(gt[i, :100].tolist())) / 100)
    return {"recall@k": float(np.mean(at_k)) if at_k else None,
            "recall@100": float(np.mean(at_100)) if at_100 else None, "recall@100_queries": len(at_100)}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.p = None

    def start(self):
        """Start polling (every 50 ms) and return once the first sample has arrived, so that the
        timed region that follows is covered from its start."""
        import threading

        self.lines = []
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
            return
        first = threading.Event()

        def reader():
            for line in self.p.stdout:
                self.lines.append(line)
                first.set()
            first.set()

        self.t = threading.Thread(target=reader, daemon=True)
        self.t.start()
        first.wait(timeout=10)
        self.skip = len(self.lines)  # samples taken before the timed region

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=10)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=10)
        lines = self.lines[self.skip:] or self.lines[-1:]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary
    profiles/<name>.txt, scaled there to a full launch of the workload (None if absent)."""
    path = os.path.join(ROOT, "profiles", f"{name}.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch"):
                return float(line.split("=")[1])
    except (OSError, ValueError):
        pass
    return None


# ---------------------------------------------------------------------------
# CPU baselines (the oracle: the plain-C restatement of the reference)
# ---------------------------------------------------------------------------

def cpu_search(ix, base, queries, c, nthreads, results=False):
    import oracle

    t = time.perf_counter()
    ids, dis = oracle.ivfpq_search(ix, queries, k=c["k"], kl=c["kl"], w=c["w"], base=base, rerank=c["rerank"],
                                   nthreads=nthreads)
    t = time.perf_counter() - t
    return (t, ids, dis) if results else t


def cpu_batched(ix, q, wq, kq, nthreads):
    """(seconds, (ids, dis, off)) of the oracle's uneven batch."""
    import oracle

    t = time.perf_counter()
    r = oracle.search_batched(ix, q, wq, kq, ties=oracle.TIES_KEYED, nthreads=nthreads)
    return time.perf_counter() - t, r


def sample_size(seconds_per_query, target_s, lo, hi):
    return int(max(lo, min(hi, target_s / max(seconds_per_query, 1e-9))))


def mixed_alpha():
    """The precision form's approximate selection, max(alpha * k, k + extra): (alpha, extra) from the
    header's GBIVF_MIXED_SCAN_ALPHA and GBIVF_MIXED_SCAN_EXTRA, alpha overridden by the
    GBIVF_MIXED_SCAN_SEL variable the engine reads."""
    hdr = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "include", "gbivf.h")).read()
    alpha = int(re.search(r"#define GBIVF_MIXED_SCAN_ALPHA (\d+)", hdr).group(1))
    extra = int(re.search(r"#define GBIVF_MIXED_SCAN_EXTRA (\d+)", hdr).group(1))
    if os.environ.get("GBIVF_MIXED_SCAN_SEL"):
        alpha = min(16, max(1, int(os.environ["GBIVF_MIXED_SCAN_SEL"])))
    return alpha, extra


def core_cpu_baseline(ix, queries, c):
    """The reference's OpenMP CPU path, parallel2 core_cpu (parallel2/ivf_pq/ivf_search.cpp:61-117),
    restated by the oracle: residuals and probe lists from the reference's coarse stage (knn_full then
    bsxfunMINUS, timed separately on one thread), then core_cpu with its hard-coded team of 8 threads
    (:62), and ceil(cores / 8) such calls at once on disjoint query slices."""
    import concurrent.futures as cf

    import oracle

    w, k = c["w"], c["k"]
    t0 = time.perf_counter()
    coaidx, _ = oracle.knn_full(ix.coa, queries, w)
    t_coarse = time.perf_counter() - t0
    d = queries.shape[1]
    res = np.ascontiguousarray((queries[:, None, :] - ix.coa[coaidx]).reshape(-1, d), np.float32)
    rid = np.ascontiguousarray(coaidx.reshape(-1), np.int32)
    cnt = np.minimum(ix.list_sizes()[coaidx].astype(np.int64).sum(1), k)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
    nout = int(cnt.sum())
    nq = len(queries)
    oracle.core_cpu(ix, res[:w * 8], rid[:w * 8], start[:8], nout, k, w, nthreads=8)  # warm-up
    t0 = time.perf_counter()
    oracle.core_cpu(ix, res, rid, start, nout, k, w, nthreads=8)
    t8 = time.perf_counter() - t0
    ncalls = max(1, math.ceil(ncpu() / 8))
    bounds = np.linspace(0, nq, ncalls + 1).astype(int)

    def part(i):
        a, b = bounds[i], bounds[i + 1]
        st = start[a:b] - start[a] if b > a else start[a:b]
        n = int(cnt[a:b].sum())
        oracle.core_cpu(ix, res[a * w:b * w], rid[a * w:b * w], np.ascontiguousarray(st, np.int32), max(n, 1), k, w,
                        nthreads=8)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(ncalls) as ex:
        list(ex.map(part, range(ncalls)))
    tn = time.perf_counter() - t0
    return {"value": nq / t8, "unit": "queries/s", "cores": 8, "kind": "port",
            "sample": f"{nq} queries: core_cpu with 8 OpenMP threads ({t8:.2f}s) on residuals from the "
                      f"coarse stage",
            "concurrent": {"value": nq / tn, "unit": "queries/s", "cores": 8 * ncalls, "calls": ncalls,
                           "sample": f"{ncalls} concurrent core_cpu calls of 8 threads on disjoint slices "
                                     f"({tn:.2f}s)"},
            "coarse_stage": {"value": nq / t_coarse, "unit": "queries/s", "cores": 1,
                             "sample": f"knn_full of {nq} queries over {ix.coarsek} centroids, one thread "
                                       f"({t_coarse:.2f}s)"}}


def parity_report(g_ids, g_dis, o_ids, o_dis):
    """The engine's results against the oracle's on the same queries: identical rows, and every id
    both return carrying the same distance bits (the oracle keeps the reference's heap tie order,
    the engine orders ties by (distance, id), so rows can differ only at ties)."""
    n = len(o_ids)
    same = float(np.mean([np.array_equal(g_ids[i], o_ids[i]) for i in range(n)]))

    def up_to_ties(i):
        # the same distance bits in the same positions, and the same ids at every distance but the
        # last (a tie across the k-th position can keep different members)
        gd, od = g_dis[i].view(np.uint32), o_dis[i].view(np.uint32)
        if not np.array_equal(gd, od):
            return False
        last = gd[-1]
        return set(g_ids[i][gd != last].tolist()) == set(o_ids[i][od != last].tolist())

    ties_ok = float(np.mean([up_to_ties(i) for i in range(n)]))
    mism = 0
    for i in range(n):
        o = dict(zip(o_ids[i].tolist(), o_dis[i].view(np.uint32).tolist()))
        mism += sum(int(x in o and o[x] != y) for x, y in zip(g_ids[i].tolist(), g_dis[i].view(np.uint32).tolist()))
    return {"queries": n, "identical_rows": same, "identical_rows_up_to_ties": ties_ok,
            "distance_mismatches_on_shared_ids": mism,
            "ties": "oracle in the reference's heap tie order; engine ties ordered by (distance, id)"}


def packed_parity(a_ids, a_dis, b_ids, b_dis, off, nq):
    """Two packed result sets (query q at off[q]:off[q+1]) compared row by row: identical rows (ids
    and distance bits), distance bits that differ for an id both return, and the share of real (not
    padding) ids the rows have in common."""
    same, mism, shared, real = 0, 0, 0, 0
    for i in range(nq):
        a, b = a_ids[off[i]:off[i + 1]], b_ids[off[i]:off[i + 1]]
        ad, bd = a_dis[off[i]:off[i + 1]].view(np.uint32), b_dis[off[i]:off[i + 1]].view(np.uint32)
        same += int(np.array_equal(a, b) and np.array_equal(ad, bd))
        bm = dict(zip(b.tolist(), bd.tolist()))
        mism += sum(int(x in bm and bm[x] != y) for x, y in zip(a.tolist(), ad.tolist()) if x >= 0)
        ra, rb = set(a[a >= 0].tolist()), set(b[b >= 0].tolist())
        shared += len(ra & rb)
        real += max(len(ra), len(rb))
    return {"queries": nq, "identical_rows_fraction": same / max(nq, 1), "distance_mismatches_on_shared_ids": mism,
            "shared_real_ids_fraction": shared / max(real, 1),
            "padding": "ids -1 (fewer candidates than k) are excluded from the id overlap"}


# ---------------------------------------------------------------------------
# multi-rank helpers
# ---------------------------------------------------------------------------

def max_over_ranks(x, dist, device):
    """The slowest rank's time: every rank takes part in the reduction (None: one process)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(nq_per_rank, steps, world, seconds):
    """Queries per second of the whole job: every rank searches its own nq_per_rank queries per
    step (weak scaling), timed by the slowest rank."""
    return nq_per_rank * steps * world / seconds


# ---------------------------------------------------------------------------
# the drop-in workload (host-built 1M index, ivfpq_search with re-rank)
# ---------------------------------------------------------------------------

def drop_in_record(args, c, rank, world, dist, dev, local_rank, with_cpu=True):
    """QPS (device buffers), e2e (host buffers), roofline of the scan kernel, parity against the
    oracle on every query, recall, and the CPU baselines of the drop-in workload."""
    import torch

    from mestrado_gb300.engine import GpuIndex

    ix_data, base, queries, key = make_inputs(c, rank)
    nq, k, kl, w, m = c["nq"], c["k"], c["kl"], c["w"], c["m"]
    cpu = cpu_1core = core = None
    if with_cpu:
        nthreads = ncpu()
        sample = min(nq, args.ref_sample)
        cpu_search(ix_data, base, queries[: max(1, sample // 10)], c, nthreads)
        t, cpu_ids, cpu_dis = cpu_search(ix_data, base, queries[:sample], c, nthreads, results=True)
        cpu = {"value": sample / t, "unit": "queries/s", "cores": nthreads, "kind": "port",
               "sample": f"{sample} queries of this workload, OpenMP over queries ({t:.2f}s)"}
        # the reference's own search is single-threaded (sequential/ivf_pq/ivf_search.cpp): one core too
        s1 = max(1, sample // 10)
        t1 = cpu_search(ix_data, base, queries[:s1], c, 1)
        cpu_1core = {"value": s1 / t1, "unit": "queries/s", "cores": 1, "kind": "port",
                     "sample": f"{s1} queries of this workload, one thread ({t1:.2f}s)"}
        core = core_cpu_baseline(ix_data, queries, c)

    gi = GpuIndex(ix_data, device=local_rank, base=base)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    d_q = torch.from_numpy(queries).to(dev)
    d_ids = torch.empty((nq, k), dtype=torch.int32, device=dev)
    d_dis = torch.empty((nq, k), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    def step(profile):
        gi.search_device(d_q.data_ptr(), nq, k, w, d_ids.data_ptr(), d_dis.data_ptr(), kl=kl,
                         rerank=c["rerank"], stream_ptr=sp, profile=profile)

    coaidx, _ = gi.coarse_assign(queries, w)
    sizes = ix_data.list_sizes().astype(np.int64)
    scan_bytes = int(sizes[coaidx].sum()) * m
    unique_bytes = int(sizes[np.unique(coaidx[coaidx >= 0])].sum()) * m  # each probed list once

    for i in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xff)
        step(True)
    stream.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    clocks.start()
    barrier()
    step_ms, coarse_ms, scank_ms, fin_ms = [], [], [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_((i + 1) & 0xff)  # L2 flush, outside the timed events
            ev0.record(stream)
        step(True)
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
        cm, sk, fm = gi.last_stages_ms()
        coarse_ms.append(cm)
        scank_ms.append(sk)
        fin_ms.append(fm)
    barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(step_ms), dist, dev)
    value = whole_job_rate(nq, args.steps, world, total_ms / 1000.0)

    # end to end through the host C ABI: pinned host queries in, ids/dis out
    h_q = torch.from_numpy(queries).pin_memory().numpy()
    h_ids = torch.empty((nq, k), dtype=torch.int32).pin_memory().numpy()
    h_dis = torch.empty((nq, k), dtype=torch.float32).pin_memory().numpy()
    for _ in range(2):
        gi.search(h_q, k, w, kl=kl, rerank=c["rerank"], out=(h_ids, h_dis))
    e2e_s = 0.0
    for i in range(args.steps):
        flush.fill_((i + 7) & 0xff)
        torch.cuda.synchronize()
        t = time.perf_counter()
        gi.search(h_q, k, w, kl=kl, rerank=c["rerank"], out=(h_ids, h_dis))
        e2e_s += time.perf_counter() - t
    e2e_s = max_over_ranks(e2e_s, dist, dev)
    e2e = whole_job_rate(nq, args.steps, world, e2e_s)

    quality = {}
    if cpu is not None:
        quality["parity_vs_oracle"] = parity_report(h_ids[:len(cpu_ids)], h_dis[:len(cpu_ids)], cpu_ids, cpu_dis)
    if rank == 0 and not args.no_recall:
        gt = ground_truth(base, queries, k, key, dev)
        quality.update(recall_report(h_ids, gt, k))

    peak, peak_kind = measured_peak_hbm()
    mean_scan_s = statistics.mean(scank_ms) / 1000.0
    achieved = scan_bytes / mean_scan_s / 1e9
    gi.close()
    return {
        "metric": "QPS", "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(c), "queries_per_step": nq, "parallelism": f"replica x{world}",
                   "l2": "flushed between steps (256 MB write)"},
        "quality": quality,
        "stage_ms": {"coarse": statistics.mean(coarse_ms), "scan_kernel": statistics.mean(scank_ms),
                     "finalize": statistics.mean(fin_ms)},
        "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": int(queries.nbytes),
                "d2h_bytes_per_step": int(nq * k * 8)},
        "roofline": {"bound": "hbm", "kernel": "ivf_scan_persistent_kernel", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "bytes_per_launch": scan_bytes, "bytes_unique_per_launch": unique_bytes,
                     "traffic": profiled_traffic("ivf_scan_cfg2")},
        "cpu_baseline": cpu, "cpu_baseline_1core": cpu_1core, "cpu_baseline_core_cpu": core,
        # norm_d, coarse_dist, coarse_select, ivf_scan_persistent, finalize per search
        "gpu_launches": 5 * args.steps,
        "clocks": clk,
    }


# ---------------------------------------------------------------------------
# the large workloads (GPU-built indexes, both forms as CUDA-graph replays)
# ---------------------------------------------------------------------------

FORMS = (("plain", dict(mixed_coarse=False, mixed_scan=False)), ("mixed", dict(mixed_coarse=True, mixed_scan=True)))


def adc_error_fp64(ix, queries, res, off, kq, nsample):
    """Relative error of the returned ADC distances against the same distance in FP64
    (sum over sub-quantizers of ||(x - y_l)_s - c_s(code)||^2 in double), over the first
    nsample queries' results: {"max_rel": ..., "mean_rel": ..., "pairs": ...}."""
    if not nsample:
        return None
    ids, dis_all = res
    row_of = np.empty(ix.n, np.int64)
    row_of[ix.ids] = np.arange(ix.n, dtype=np.int64)
    rels = []
    coa = ix.coa.astype(np.float64)
    pq = ix.pq.astype(np.float64)
    m, ds = ix.m, ix.ds
    for i in range(nsample):
        got = ids[off[i]:off[i] + kq[i]]
        dis = dis_all[off[i]:off[i] + kq[i]]
        keep = got >= 0
        got, dis = got[keep], dis[keep].astype(np.float64)
        if got.size == 0:
            continue
        rows = row_of[got]
        lists = np.searchsorted(ix.list_off, rows, side="right") - 1
        r = queries[i].astype(np.float64)[None, :] - coa[lists]             # residuals, n x d
        cw = pq[np.arange(m)[None, :], ix.codes[rows].astype(np.int64)]    # n x m x ds
        exact = ((r.reshape(-1, m, ds) - cw) ** 2).sum(axis=(1, 2))
        rels.append(np.abs(dis - exact) / np.maximum(exact, 1e-30))
    if not rels:
        return None
    rel = np.concatenate(rels)
    return {"max_rel": float(rel.max()), "mean_rel": float(rel.mean()), "pairs": int(rel.size)}


def large_record(args, name, c, dev, rank, world, dist, local_rank, headline):
    """Both forms of a large workload timed as CUDA-graph replays, with stage split, recall against
    an exact ground truth, FP64 distance error, oracle parity on a sample of queries and, for the
    headline, e2e through the host C ABI and the CPU baseline."""
    import torch

    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import exact_topk_streaming

    gm, ix, queries, t_build = large_inputs(name, c, dev, rank, dist)
    gi = GpuIndex(ix, device=local_rank)
    nq, m = c["nq"], c["m"]
    wq, kq = batch_shape(c, nq)
    off = np.concatenate([[0], np.cumsum(kq)]).astype(np.int64)
    max_w, max_k = int(wq.max()), int(kq.max())
    d_w = torch.from_numpy(wq).to(dev)
    d_k = torch.from_numpy(kq).to(dev)
    d_off = torch.from_numpy(off[:-1].copy()).to(dev)
    d_ids = torch.empty(int(off[-1]), dtype=torch.int32, device=dev)
    d_dis = torch.empty(int(off[-1]), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    q_host = queries.cpu().numpy()
    # algorithmic bytes of the ADC scan: sum over queries of their probed lists' codes
    sizes = ix.list_sizes().astype(np.int64)
    coa_idx, _ = gi.coarse_assign(q_host, max_w)
    probed = np.where(np.arange(max_w)[None, :] < wq[:, None], coa_idx, -1)
    scan_bytes = int(np.where(probed >= 0, sizes[np.maximum(probed, 0)], 0).sum()) * m
    uniq = np.unique(probed[probed >= 0])
    unique_bytes = int(sizes[uniq].sum()) * m
    sample = 0 if args.no_recall else min(nq, c["recall_q"])
    gt = exact_topk_streaming(gm, c["nbase"], queries[:sample], max_k) if sample else None

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    forms = {}
    for form, fl in FORMS:
        graph = gi.capture_graph(queries.data_ptr(), nq, max_k, max_w, d_ids.data_ptr(), d_dis.data_ptr(),
                                 d_w_ptr=d_w.data_ptr(), d_k_ptr=d_k.data_ptr(), d_off_ptr=d_off.data_ptr(),
                                 stream_ptr=sp, **fl)
        kernels = graph.kernel_count()
        for i in range(args.warmup):
            graph.launch(sp)
        stream.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        clocks = ClockSampler(local_rank)
        clocks.start()
        barrier()
        window = args.profile_steps and form == "mixed"
        if window:  # the range an external profiler started with --profile-from-start off captures
            torch.cuda.profiler.start()
        total = 0.0
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xff)
                ev0.record(stream)
            graph.launch(sp)
            with torch.cuda.stream(stream):
                ev1.record(stream)
            ev1.synchronize()
            total += ev0.elapsed_time(ev1)
        if window:
            torch.cuda.profiler.stop()
        barrier()
        clk = clocks.stop()
        graph.close()
        total = max_over_ranks(total, dist, dev)
        ids = d_ids.cpu().numpy()
        dis = d_dis.cpu().numpy()
        # stage split: the mean of three profiled (non-graph) searches
        st, parts_l = [], []
        for _ in range(3):
            flush.fill_(1)
            gi.search_batched_device(queries.data_ptr(), nq, d_w.data_ptr(), d_k.data_ptr(), d_off.data_ptr(),
                                     max_w, max_k, d_ids.data_ptr(), d_dis.data_ptr(), stream_ptr=sp, profile=True,
                                     **fl)
            st.append(stage_split(gi))
            parts_l.append(gi.last_scan_parts())
        unproven = gi.last_unproven()  # precision form: queries not proven equal to the exact form
        stages = {k_: statistics.mean(s[k_] for s in st) for k_ in st[0]}
        scan_parts = {k_: statistics.mean(p_[0][k_] for p_ in parts_l) for k_ in parts_l[0][0]}
        scan_counters = parts_l[-1][1]
        rec = packed_recall(ids, off, kq, gt, sample) if sample else {}
        forms[form] = dict(qps=whole_job_rate(nq, args.steps, world, total / 1000.0), ms_per_step=total / args.steps,
                           stages=stages, scan_parts_ms=scan_parts, scan_counters=scan_counters,
                           unproven_queries=unproven, gpu_launches_per_step=kernels, clocks=clk, ids=ids, dis=dis, **rec,
                           adc_distance_error_vs_fp64=adc_error_fp64(ix, q_host, (ids, dis), off, kq,
                                                                     min(sample or 100, 100)))
    pl, mx = forms["plain"], forms["mixed"]
    plain_vs_mixed = packed_parity(mx["ids"], mx["dis"], pl["ids"], pl["dis"], off, nq)

    # the plain form (the drop-in) against the oracle on a sample of queries, over the same index
    par = None
    if rank == 0 and args.parity_sample > 0:
        ns = min(nq, args.parity_sample)
        t_or, (o_ids, o_dis, o_off) = cpu_batched(ix, q_host[:ns], wq[:ns], kq[:ns], ncpu())
        par = packed_parity(pl["ids"][:off[ns]], pl["dis"][:off[ns]], o_ids, o_dis, o_off, ns)
        par["ties"] = "both keyed by (distance, position in the probe order)"
        par["oracle_seconds"] = t_or
        par["largest_k_in_sample"] = int(kq[:ns].max())
        par["largest_nprobe_in_sample"] = int(wq[:ns].max())

    peak, peak_kind = measured_peak_hbm()
    # The dominant kernel of the mixed step. Scanned list by list, it is the list-centric kernel, whose
    # algorithmic bytes are the codes of the probes the first pass left to it (the engine's rule: each
    # query's leading probes up to beta * k_sel rows go to the first pass); else the per-query scan kernel.
    if mx["scan_counters"]["list_scan"]:
        alpha, extra = mixed_alpha()
        kq64 = kq.astype(np.int64)
        sel = np.minimum(np.maximum(kq64 * alpha, kq64 + extra), 4096)  # the precision form's k_sel
        rows = np.where(probed >= 0, sizes[np.maximum(probed, 0)], 0)
        csum = np.cumsum(rows, axis=1)
        lead = (csum < sel[:, None]).sum(1) + 1  # leading probes holding beta * k_sel rows (beta = 1)
        lead = np.minimum(lead, wq)
        lc_bytes = int(np.where(np.arange(max_w)[None, :] >= lead[:, None], rows, 0).sum()) * m
        kern_name, kern_ms, kern_bytes = "lc_scan_kernel (mixed form)", mx["scan_parts_ms"]["list_scan"], lc_bytes
    else:
        kern_name, kern_ms, kern_bytes = "ivf_scan_persistent_kernel (mixed form)", mx["stages"]["scan_kernel"], scan_bytes
    achieved = kern_bytes / (kern_ms / 1000.0) / 1e9
    stage_ms = mx["stages"]["scan_kernel"]  # the whole scan stage before finalize (all its kernels)
    rec = {
        "workload": large_workload(name, c),
        "forms": {f: {k_: v for k_, v in forms[f].items() if k_ not in ("ids", "dis", "clocks")} for f in forms},
        "mixed_over_plain_qps": mx["qps"] / pl["qps"],
        "recall@100_delta": (None if mx.get("recall@100") is None else mx["recall@100"] - pl["recall@100"]),
        "recall_sample_queries": sample,
        "mixed_vs_plain": plain_vs_mixed,
        "parity_plain_vs_oracle": par,
        "roofline": {"bound": "hbm", "kernel": kern_name, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / peak, "bytes_per_launch": kern_bytes, "kernel_ms": kern_ms,
                     "traffic": profiled_traffic(f"lc_scan_{name}"),
                     "scan_stage": {"bytes_per_step": scan_bytes, "bytes_unique_per_step": unique_bytes,
                                    "ms": stage_ms, "gbs": scan_bytes / (stage_ms / 1000.0) / 1e9,
                                    "frac": scan_bytes / (stage_ms / 1000.0) / 1e9 / peak,
                                    "what": "every kernel between the coarse stage and finalize (first pass, "
                                            "grouping, list-centric scan, selection, overflow pass) on all "
                                            "probed codes"}},
        "index_build_s": t_build,
        "clocks": mx["clocks"], "clocks_plain": pl["clocks"],
    }

    if headline:
        # end to end through the host C ABI: pinned queries, nprobe and k in, packed ids / dis out
        h_q = torch.from_numpy(q_host).pin_memory().numpy()
        h_w = torch.from_numpy(wq).pin_memory().numpy()
        h_k = torch.from_numpy(kq).pin_memory().numpy()
        h_ids = torch.empty(int(off[-1]), dtype=torch.int32).pin_memory().numpy()
        h_dis = torch.empty(int(off[-1]), dtype=torch.float32).pin_memory().numpy()
        mixed_fl = dict(FORMS)["mixed"]
        for _ in range(2):
            gi.search_batched(h_q, h_w, h_k, out=(h_ids, h_dis), **mixed_fl)
        e2e_s = 0.0
        for i in range(args.steps):
            flush.fill_((i + 7) & 0xff)
            torch.cuda.synchronize()
            t = time.perf_counter()
            gi.search_batched(h_q, h_w, h_k, out=(h_ids, h_dis), **mixed_fl)
            e2e_s += time.perf_counter() - t
        e2e_s = max_over_ranks(e2e_s, dist, dev)
        same = bool(np.array_equal(h_ids, mx["ids"]))
        rec["e2e"] = {"value": whole_job_rate(nq, args.steps, world, e2e_s), "unit": "queries/s",
                      "h2d_bytes_per_step": int(h_q.nbytes + h_w.nbytes + h_k.nbytes),
                      "d2h_bytes_per_step": int(h_ids.nbytes + h_dis.nbytes),
                      "api": "gbivf_search_batched (host buffers, mixed form)", "ids_equal_device_run": same}
        # the oracle on all host cores, on a sample of the same queries sized to ~10 s
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            t32, _ = cpu_batched(ix, q_host[:32], wq[:32], kq[:32], ncpu())
            ns = sample_size(t32 / 32, 10.0, 64, nq)
            t, _ = cpu_batched(ix, q_host[:ns], wq[:ns], kq[:ns], ncpu())
            rec["cpu_baseline"] = {"value": ns / t, "unit": "queries/s", "cores": ncpu(), "kind": "port",
                                   "sample": f"the first {ns} of the {nq} queries (their own nprobe and k), "
                                             f"OpenMP over queries ({t:.2f}s)"}
    gi.close()
    return rec


def run_headline(args, rank, world, local_rank):
    import torch

    name, c = HEADLINE, LARGE[HEADLINE]
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    rec = large_record(args, name, c, dev, rank, world, dist, local_rank, headline=True)
    sub = {}
    if world == 1 and not args.no_sub:
        for sub_name, fn in (("drop_in_cfg2", lambda: drop_in_record(args, CONFIGS["cfg2"], rank, world, None, dev,
                                                                     local_rank)),
                             ("cfg3", lambda: large_record(args, "cfg3", LARGE["cfg3"], dev, rank, world, None,
                                                           local_rank, headline=False)),
                             ("cfg5_1B", lambda: stream_record(argparse.Namespace(**{**vars(args), "steps": 3}),
                                                               LARGE["cfg5"], "cfg5", local_rank))):
            try:
                sub[sub_name] = fn()
            except Exception as e:  # a failed sub-record must not lose the headline
                sub[sub_name] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()
    if rank == 0:
        mx, pl = rec["forms"]["mixed"], rec["forms"]["plain"]
        line = {
            "metric": METRIC, "value": mx["qps"], "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "mixed: bf16 tensor-core coarse + f32 re-check, f16 tables with f32 accumulation and f32 "
                     "re-score (plain form: f32)",
            "data": "synthetic",
            "config": large_config(name, c),
            "forms": {"mixed_qps": mx["qps"], "plain_qps": pl["qps"], "mixed_over_plain": rec["mixed_over_plain_qps"],
                      "recall@100_mixed": mx.get("recall@100"), "recall@100_plain": pl.get("recall@100"),
                      "recall@100_delta": rec["recall@100_delta"], "adc_scan_gbs": rec["roofline"]["achieved"],
                      "detail": rec["forms"], "mixed_vs_plain": rec["mixed_vs_plain"]},
            "parity": rec["parity_plain_vs_oracle"],
            "e2e": rec.get("e2e"),
            "roofline": rec["roofline"],
            "cpu_baseline": rec.get("cpu_baseline"),
            "gpu_launches": mx["gpu_launches_per_step"] * args.steps,
            "clocks": rec["clocks"],
            "index_build_s": rec["index_build_s"],
            "sub": sub,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference_headline(args, rank, world):
    """The oracle alone on the headline workload: each step searches a bounded sample of the batch
    (rotating through it), every host thread."""
    if rank != 0:
        return
    import torch

    name, c = HEADLINE, LARGE[HEADLINE]
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _, ix, queries, _ = large_inputs(name, c, dev)
    q_host = queries.cpu().numpy()
    del queries
    torch.cuda.empty_cache()
    nq = c["nq"]
    wq, kq = batch_shape(c, nq)
    t32, _ = cpu_batched(ix, q_host[:32], wq[:32], kq[:32], ncpu())
    # about 1.5 s of CPU work per step
    ns = sample_size(t32 / 32, 1.5, 32, nq)

    def step(i):
        s = (i * ns) % nq
        sl = slice(s, min(nq, s + ns))
        return cpu_batched(ix, q_host[sl], wq[sl], kq[sl], ncpu())[0], sl.stop - sl.start

    for i in range(args.warmup):
        step(i)
    ts = [step(args.warmup + i) for i in range(args.steps)]
    total = sum(t for t, _ in ts)
    done = sum(n for _, n in ts)
    qps = done / total
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": large_config(name, c),
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": ncpu(), "kind": "port",
                         "sample": f"{ns} of the {nq} queries per step (consecutive slices), OpenMP over queries"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, c, rank, world):
    """The oracle alone on a drop-in workload (cfg1 / cfg2)."""
    if rank != 0:
        return
    ix, base, queries, _ = make_inputs(c, 0)
    nthreads = ncpu()
    sample = min(len(queries), args.ref_sample)
    qs = queries[:sample]
    for _ in range(args.warmup):
        cpu_search(ix, base, qs[: max(1, sample // 10)], c, nthreads)
    ts = [cpu_search(ix, base, qs, c, nthreads) for _ in range(args.steps)]
    total = sum(ts)
    qps = sample * args.steps / total
    line = {
        "impl": "reference", "metric": "QPS", "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": workload_name(c), "queries_per_step": c["nq"],
                                        "parallelism": f"replica x{world}",
                                        "l2": "flushed between steps (256 MB write)"},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": nthreads, "kind": "port",
                         "sample": f"{sample} of the {c['nq']} queries per step"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_drop_in(args, c, rank, world, local_rank):
    import torch

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    line = drop_in_record(args, c, rank, world, dist, dev, local_rank,
                          with_cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_large_line(args, name, local_rank):
    import torch

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    rec = large_record(args, name, LARGE[name], dev, 0, 1, None, local_rank, headline=False)
    mx = rec["forms"]["mixed"]
    line = {"metric": METRIC, "value": mx["qps"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "data": "synthetic", "config": large_config(name, LARGE[name]), **rec}
    print(json.dumps(line), flush=True)


def run_stream(args, c, name, local_rank):
    print(json.dumps(stream_record(args, c, name, local_rank)), flush=True)


def stream_record(args, c, name, local_rank):
    """Billion-scale configuration: streaming GPU build with refinement codes, both forms (plain
    FP32; tensor-core coarse + precision-form scan) timed as CUDA-graph replays of one batch with
    the refinement re-rank of the kl best ADC candidates; recall@1/10/100 against a brute-force
    ground truth computed over the regenerated base."""
    import torch

    from mestrado_gb300.gpu_build import GpuMixture, build_index_streaming, exact_topk_streaming
    from mestrado_gb300.synth import Mixture

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    gm = GpuMixture(Mixture(d=c["d"], ncomp=c["ncomp"], seed=c["seed"], zipf=c["zipf"]))
    t0 = time.time()
    train = gm.generate(c["ntrain"], stream_id=2)
    gi, off = build_index_streaming(gm, c["nbase"], train, c["C"], c["m"], m2=c["m2"], niter=c["train_iters"],
                                    seed=c["seed"], log=log)
    del train
    torch.cuda.empty_cache()
    t_build = time.time() - t0
    nq, k, kl, w = c["nq"], c["k"], c["kl"], c["w"]
    queries = gm.generate(nq, stream_id=3)
    sample = 0 if args.no_recall else min(nq, c["recall_q"])
    t0 = time.time()
    gt = exact_topk_streaming(gm, c["nbase"], queries[:sample], k) if sample else None
    t_gt = time.time() - t0
    d_ids = torch.empty((nq, k), dtype=torch.int32, device=dev)
    d_dis = torch.empty((nq, k), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    forms = {}
    # the precision-form scan pays on short lists; at this list length (~3,800 codes) the exact tables
    # are amortised, so the tensor-core coarse stage with the exact scan is timed as well
    for form, mixed, mscan in (("plain", False, False), ("mixed_coarse", True, False), ("mixed", True, True)):
        graph = gi.capture_graph(queries.data_ptr(), nq, k, w, d_ids.data_ptr(), d_dis.data_ptr(), kl=kl,
                                 refine=True, mixed_coarse=mixed, mixed_scan=mscan, stream_ptr=sp)
        for i in range(args.warmup):
            graph.launch(sp)
        stream.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks = ClockSampler(local_rank)
        clocks.start()
        total = 0.0
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xff)
                ev0.record(stream)
            graph.launch(sp)
            with torch.cuda.stream(stream):
                ev1.record(stream)
            ev1.synchronize()
            total += ev0.elapsed_time(ev1)
        clk = clocks.stop()
        graph.close()
        ids = d_ids.cpu().numpy()
        gi.search_device(queries.data_ptr(), nq, k, w, d_ids.data_ptr(), d_dis.data_ptr(), kl=kl, refine=True,
                         stream_ptr=sp, profile=True, mixed_coarse=mixed, mixed_scan=mscan)
        stages = stage_split(gi)
        rec = {}
        if sample:
            for r in (1, 10, 100):
                rec[f"recall@{r}"] = float(np.mean([len(set(ids[i, :r].tolist()) & set(gt[i, :r].tolist())) / r
                                                    for i in range(sample)]))
        forms[form] = dict(qps=nq * args.steps / (total / 1000.0), ms_per_step=total / args.steps, stages=stages,
                           recall=rec, clocks=clk, ids=ids)
    same_rows = {f: float(np.mean([np.array_equal(a, b) for a, b in zip(forms["plain"]["ids"], forms[f]["ids"])]))
                 for f in ("mixed_coarse", "mixed")}
    best = max(("mixed_coarse", "mixed"), key=lambda f: forms[f]["qps"])
    mx = forms[best]
    wl = (f"{name}: base {c['nbase']:,} x d=128 ({c['ncomp']}-component mixture, generated and encoded on the GPU "
          f"in chunks), C={c['C']:,} lists, m={c['m']}x256 + m2={c['m2']}x256 refinement codes, {nq:,} queries/step, "
          f"w={w}, k={k}, re-rank of the {kl} best ADC candidates by refinement codes")
    line = {
        "metric": "QPS", "value": mx["qps"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 tensor-core coarse + fp32 re-check; fp16 tables, fp32 re-score",
        "data": "synthetic",
        "config": {"workload": wl,
                   "form": ("tensor-core coarse stage, exact scan" if best == "mixed_coarse" else
                            "tensor-core coarse stage, fp16-table scan") + ", CUDA-graph replay (the faster of the two)",
                   "plain_qps": forms["plain"]["qps"], "mixed_coarse_qps": forms["mixed_coarse"]["qps"],
                   "mixed_both_qps": forms["mixed"]["qps"],
                   "speedup_vs_plain": mx["qps"] / forms["plain"]["qps"], "identical_rows_fraction": same_rows,
                   "recall_sample_queries": sample, "recall_mixed": mx["recall"],
                   "recall_plain": forms["plain"]["recall"],
                   "stage_ms_mixed": mx["stages"], "stage_ms_plain": forms["plain"]["stages"],
                   "stage_ms_mixed_both": forms["mixed"]["stages"],
                   "index_build_s": t_build, "ground_truth_s": t_gt, "l2": "flushed between steps (256 MB write)"},
        "clocks": mx["clocks"],
    }
    gi.close()
    del gi, flush, d_ids, d_dis, queries
    torch.cuda.empty_cache()
    return line


def run_coarse(args, c, name, local_rank):
    """The coarse stage alone at a large configuration's shape (knn_full over C
    centroids, w nearest per query): plain FP32 and tensor-core forms, timed
    with CUDA events on device buffers. Centroids are mixture points plus
    Gaussian noise (no k-means: the stage's cost does not depend on training)."""
    import ctypes

    import torch

    from mestrado_gb300.engine import GpuIndex
    from mestrado_gb300.gpu_build import GpuMixture
    from mestrado_gb300.ivfdata import IVFPQData
    from mestrado_gb300.synth import Mixture

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    gm = GpuMixture(Mixture(d=c["d"], ncomp=c["ncomp"], seed=c["seed"], zipf=c["zipf"]))
    coa = gm.generate(c["C"], stream_id=5)
    coa += torch.randn(coa.shape, device=dev, generator=torch.Generator(device=dev).manual_seed(1)) * 2.0
    q = gm.generate(c["nq"], stream_id=3)
    m = c["m"]
    rng = np.random.default_rng(0)
    ix = IVFPQData(coa=coa.cpu().numpy(), pq=rng.normal(0, 10, (m, 256, c["d"] // m)).astype(np.float32),
                   list_off=np.zeros(c["C"] + 1, np.int64), ids=np.zeros(0, np.int32),
                   codes=np.zeros((0, m), np.uint8))
    gi = GpuIndex(ix, device=local_rank)
    nq, w = c["nq"], c["w"]
    out_i = torch.empty((nq, w), dtype=torch.int32, device=dev)
    out_d = torch.empty((nq, w), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    forms = {}
    for form, flags in (("plain", 0), ("mixed", 0x4)):
        ts = []
        for i in range(args.warmup + args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xff)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            check_rc(gi.lib.gbivf_coarse_assign_device(gi.h, ctypes.c_void_p(q.data_ptr()), nq, w, flags,
                                                       ctypes.c_void_p(out_i.data_ptr()),
                                                       ctypes.c_void_p(out_d.data_ptr()),
                                                       ctypes.c_void_p(stream.cuda_stream)), gi)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            if i >= args.warmup:
                ts.append(e0.elapsed_time(e1))
        forms[form] = dict(ms=float(np.median(ts)), ids=out_i.cpu().numpy())
    same = bool(np.array_equal(forms["plain"]["ids"], forms["mixed"]["ids"]))
    flops = 2.0 * nq * c["C"] * c["d"]
    line = {"metric": "coarse-stage time", "unit": "ms", "higher_is_better": False, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
            "config": {"workload": f"{name} coarse stage: {nq:,} queries x C={c['C']:,} centroids (d=128), w={w}",
                       "l2": "flushed between steps (256 MB write)"},
            "plain_ms": forms["plain"]["ms"], "mixed_ms": forms["mixed"]["ms"],
            "speedup": forms["plain"]["ms"] / forms["mixed"]["ms"], "identical_lists": same,
            "coarse_tflops_mixed": flops / (forms["mixed"]["ms"] / 1000.0) / 1e12}
    print(json.dumps(line), flush=True)
    gi.close()


def check_rc(rc, gi):
    if rc != 0:
        raise RuntimeError(f"gbivf error {rc}: {gi.lib.gbivf_last_error().decode()}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbivf", choices=["gbivf", "reference"])
    ap.add_argument("--config", default=HEADLINE, choices=sorted(CONFIGS) + sorted(LARGE))
    ap.add_argument("--ref-sample", type=int, default=10_000, help="drop-in workloads: queries per CPU step")
    ap.add_argument("--parity-sample", type=int, default=128,
                    help="large workloads: queries checked against the oracle")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-recall", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="headline: skip the drop-in, 10M and 1B sub-records")
    ap.add_argument("--profile-steps", action="store_true",
                    help="large workloads: mark the mixed form's timed steps for a profiler started with "
                         "--profile-from-start off (numbers printed under a profiler are not measurements)")
    ap.add_argument("--stage", default="search", choices=["search", "coarse"],
                    help="large configurations: time the whole search, or the coarse stage alone")
    ap.add_argument("--nbase", type=int, default=None,
                    help="large configurations: override the base size (trial runs of a smaller base)")
    args = ap.parse_args()
    if args.warmup < 3:
        log(f"--warmup {args.warmup} raised to 3 (at least 3 untimed warm-up steps)")
        args.warmup = 3
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.config in LARGE and args.nbase:
        LARGE[args.config] = dict(LARGE[args.config], nbase=args.nbase)
    if args.config == HEADLINE and args.stage == "search":
        if args.impl == "reference":
            run_reference_headline(args, rank, world)
        else:
            run_headline(args, rank, world, local_rank)
        return
    if args.config in LARGE:
        if args.impl == "reference" or world > 1:
            if rank == 0:
                print(json.dumps({"impl": args.impl, "unavailable": "this workload runs the GPU engine alone, on "
                                  "one GPU; the headline workload (the default) has the reference arm"}))
            return
        c = LARGE[args.config]
        if args.stage == "coarse":
            run_coarse(args, c, args.config, local_rank)
        elif c.get("stream"):
            run_stream(args, c, args.config, local_rank)
        else:
            run_large_line(args, args.config, local_rank)
        return
    c = CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, c, rank, world)
    else:
        run_drop_in(args, c, rank, world, local_rank)


if __name__ == "__main__":
    main()
