#!/usr/bin/env python3
"""Benchmark of the residual-correlation kNN hot path on one GB300 (or N, sharded).

Metric: residual kNN queries/s (and p99 step latency), BF16-screened form vs the
plain FP32 form, same neighbours.  Default workload = the precision-form shape:
N=262144, D=8, m=512, k=50, predecessor_mode=True, Q = all N queries, RBF l=2 over
a seeded mixture of 16 Gaussians (synthetic; no dataset exists for it).

One step = one ct_knn_residual call over the whole query set with V, coords and
queries resident in HBM.  `e2e` repeats the step through the host-facing call:
query ids copied from pinned host memory, results copied back to pinned host
memory, all inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) each rank holds a replica of the metric and takes an
interleaved slice of the queries (no data-path collective); the max over ranks
of the timed region gives the time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "residual kNN queries/s & p99 ms, BF16-screened vs plain FP32 GPU, same neighbours"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["precision", "readme", "plain_small"], default="precision")
    ap.add_argument("--plain-steps", type=int, default=1, help="timed steps of the plain FP32 form (0 = skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=2048, help="queries per CPU baseline sample")
    ap.add_argument("--n", type=int, default=None, help="override N of the workload (profiling on a smaller case)")
    ap.add_argument("--no-batching", action="store_true", help="skip the 64-tree batching-form measurement")
    ap.add_argument("--batch-trees", type=int, default=64, help="trees of the batching form (fewer for profiling)")
    ap.add_argument("--no-headline", action="store_true",
                    help="skip the precision-form workload (profiling the batching form alone)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-form measurement")
    ap.add_argument("--no-euclidean", action="store_true", help="skip the Euclidean k=10 measurement")
    ap.add_argument("--no-tree", action="store_true", help="skip the cover-tree form measurement")
    ap.add_argument("--tree-queries", type=int, default=4096, help="sampled queries of the tree-form measurement")
    ap.add_argument("--serving-rates", default="100,500,1000", help="request rates (req/s) of the serving sweep")
    ap.add_argument("--serving-seconds", type=float, default=2.0, help="arrival window per serving rate")
    ap.add_argument("--new-points-request", default=None, metavar="N,LS,Q",
                    help="profiling aid: one screened request of Q new points against a serving-shaped tree of N "
                         "points (D=3, Matern 5/2 lengthscale LS, m=256), timed alone; no bench line")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def shard_queries(nq: int, world: int, rank: int) -> np.ndarray:
    """Interleaved slice: balances the triangular cost of predecessor mode across ranks."""
    return np.arange(rank, nq, world, dtype=np.int64)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


# ------------------------------------------------------------------ CPU (oracle) legs
def oracle_queries_per_s(wl, sample: int, threads: int, parity: bool, seed: int = 4, tree=None):
    """Time the restated rust-hilbert engine (oracle/ct_oracle.c) on `sample` random queries."""
    from oracle import oracle as O

    if tree is None:
        t0 = time.perf_counter()
        tree = O.OracleResidualTree(wl.v, wl.p, wl.coords, wl.variance, [wl.lengthscale] * wl.d,
                                    kernel_type=wl.kernel_type, chunk=512, order="hilbert", parity=parity)
        tree.build_seconds = time.perf_counter() - t0
    q = np.random.default_rng(seed).choice(wl.n, min(sample, wl.n), replace=False)
    t0 = time.perf_counter()
    tree.knn(q, wl.k, predecessor=wl.predecessor, parity=parity, threads=threads)
    dt = time.perf_counter() - t0
    return q.size / dt, tree


def run_reference(args, wl):
    """--impl reference: the reference's own CPU algorithm (restated rust-hilbert, default
    budget mode) on this machine's host cores; each step is a bounded query sample."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    qps, tree = oracle_queries_per_s(wl, 64, threads, parity=False)
    build_s = tree.build_seconds
    for w in range(args.warmup):
        oracle_queries_per_s(wl, args.cpu_sample, threads, parity=False, seed=100 + w, tree=tree)
    times = []
    for s in range(args.steps):
        q = np.random.default_rng(200 + s).choice(wl.n, min(args.cpu_sample, wl.n), replace=False)
        t1 = time.perf_counter()
        tree.knn(q, wl.k, predecessor=wl.predecessor, parity=False, threads=threads)
        times.append(time.perf_counter() - t1)
    ms = float(np.mean(times) * 1e3)
    value = args.cpu_sample / (ms / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "p99_ms": float(np.percentile(np.array(times) * 1e3, 99)), "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.describe(), "engine": "rust-hilbert restated in C (oracle/ct_oracle.c), default budget mode"},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{args.cpu_sample} random query ids per step; tree build {build_s:.2f} s excluded"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "build_seconds": build_s,
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ FP64 check of the timed output
def fp64_check(wl, dev, rows, got_idx, got_dist, near_tie=1e-6, block=256):
    """Check the neighbour rows of query ids `rows` (int64 numpy) produced by the timed
    run against an FP64 brute force evaluated here with torch on the GPU (independent
    of the engine's kernels): x/l, the RBF or Matern 5/2 kernel, rho = (K - v_q.v_c) /
    sqrt(max(p_q p_c, 1e-18)) clamped to [-1, 1], d = sqrt(1 - |rho|), d(q, q) = 0;
    order (d, idx).  A row whose set differs is a near-tie row when every swapped pair
    of candidates is closer than `near_tie` in FP64 distance, else a mismatch."""
    import torch

    f64 = torch.float64
    inv_ls = 1.0 / torch.tensor([wl.lengthscale] * wl.d, dtype=f64, device=dev)
    X = torch.as_tensor(wl.coords, device=dev).to(f64) * inv_ls
    V = torch.as_tensor(wl.v, device=dev).to(f64)
    P = torch.as_tensor(wl.p, device=dev).to(f64)
    k = wl.k
    rows = np.asarray(rows, dtype=np.int64)
    order = np.argsort(rows, kind="stable")
    stats = {"queries": int(rows.size), "rows_identical": 0, "near_tie_rows": 0, "mismatches_beyond_near_tie": 0,
             "count_mismatches": 0, "max_abs_err": 0.0, "predecessor_violations": 0, "near_tie": near_tie,
             "oracle": "FP64 brute force (torch, GPU) over the stored f32 V, p and coordinates"}
    for s in range(0, rows.size, block):
        sel = order[s:s + block]
        q = torch.as_tensor(rows[sel], device=dev)
        hi = int(rows[sel].max()) if wl.predecessor else wl.n
        if hi <= 0:
            continue
        xc = X[:hi]
        d2 = torch.zeros((q.numel(), hi), dtype=f64, device=dev)
        for a in range(wl.d):
            d2 += (X[q, a][:, None] - xc[:, a][None, :]) ** 2
        if wl.kernel_type == 1:
            t = np.sqrt(5.0) * torch.sqrt(d2)
            K = wl.variance * (1.0 + t + t * t / 3.0) * torch.exp(-t)
        else:
            K = wl.variance * torch.exp(-0.5 * d2)
        K -= V[q] @ V[:hi].T
        K /= torch.sqrt(torch.clamp(P[q][:, None] * P[:hi][None, :], min=1e-18))
        D = torch.sqrt(torch.clamp(1.0 - torch.abs(torch.clamp(K, -1.0, 1.0)), min=0.0))
        cols = torch.arange(hi, device=dev)
        D[q[:, None] == cols[None, :]] = 0.0
        if wl.predecessor:
            D[cols[None, :] >= q[:, None]] = float("inf")
        dv, di = torch.sort(D, dim=1, stable=True)
        dv, di = dv[:, :k].cpu().numpy(), di[:, :k].cpu().numpy()
        Dh = None
        for r_local, r in enumerate(sel):
            fin = np.isfinite(dv[r_local])
            ref = set(int(x) for x in di[r_local][fin])
            gi = got_idx[r]
            got = set(int(x) for x in gi if x >= 0)
            if (gi >= 0).sum() != fin.sum():
                stats["count_mismatches"] += 1
            if wl.predecessor and np.any(gi[gi >= 0] >= rows[r]):
                stats["predecessor_violations"] += 1
            nv = int(min((gi >= 0).sum(), fin.sum()))
            if nv:
                err = float(np.abs(got_dist[r][:nv].astype(np.float64) - dv[r_local][:nv]).max())
                stats["max_abs_err"] = max(stats["max_abs_err"], err)
            if got == ref:
                stats["rows_identical"] += 1
                continue
            if Dh is None:
                Dh = D.cpu().numpy()
            eg, ef = sorted(got - ref), sorted(ref - got)
            gap = np.inf if len(eg) != len(ef) or max(eg + ef) >= hi else float(
                np.max(np.abs(np.sort(Dh[r_local, eg]) - np.sort(Dh[r_local, ef]))))
            if gap < near_tie:
                stats["near_tie_rows"] += 1
            else:
                stats["mismatches_beyond_near_tie"] += 1
        del d2, K, D
    return stats


# ------------------------------------------------------------------ Euclidean and tree forms
def bench_euclidean(dev, steps: int = 3, warmup: int = 3, cpu: bool = True):
    """README-shape Euclidean run: N=32768 N(0,1) coordinates in D=3 (seed 1), k=10,
    queries = the coordinates, exact GPU kNN (ct_knn_euclidean); beside it the
    restated reference Euclidean cover tree (oracle) on a query sample, host cores."""
    import torch

    from covertreex_gb300 import synthetic
    from covertreex_gb300.euclidean import EuclideanTree

    X = synthetic.gaussian_coords(32768, 3, 1)
    tree = EuclideanTree(X, device=dev)
    q = torch.as_tensor(X, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        tree.knn_device(q, 10)
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        tree.knn_device(q, 10)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    step_ms = float(np.mean(ms))
    out = {"workload": "Euclidean kNN, N=32768, D=3, N(0,1) seed 1, k=10, queries = coordinates (exact)",
           "queries_per_s": 32768 / (step_ms / 1e3), "ms_per_step": step_ms, "steps": steps,
           "gpu_launches_per_step": 1}
    if cpu:
        from oracle import oracle as O

        threads = os.cpu_count() or 1
        ot = O.OracleEuclideanTree(X)
        sample = X[np.random.default_rng(4).choice(32768, 4096, replace=False)]
        t0 = time.perf_counter()
        ot.knn(sample, 10)
        dt = time.perf_counter() - t0
        out["cpu_reference"] = {"value": sample.shape[0] / dt, "unit": "queries/s", "cores": threads,
                                "kind": "port", "sample": "4096 random coordinates as queries (restated "
                                "rust Euclidean cover tree, best-first, approximate as the reference)"}
    return out


def bench_tree(wl, dev, nsample: int):
    """Cover-tree form on the same workload: device build seconds (prefix-doubling groups,
    conflict graph, MIS, certified radii) and the exact traversal on `nsample` sampled
    queries, with the distance evaluations per query (the reference's E_q) beside the
    dense form's."""
    import torch

    from covertreex_gb300 import _lib
    from covertreex_gb300.device import CudaResidualIndex

    L = _lib.load()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    idx = CudaResidualIndex(wl.v, wl.p, wl.coords, variance=wl.variance, lengthscale=[wl.lengthscale] * wl.d,
                            kernel_type=wl.kernel_type, build_tree=True, device=dev)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    info = idx.build_info()
    q = np.sort(np.random.default_rng(4).choice(wl.n, min(nsample, wl.n), replace=False))
    L.ct_set_timing(1)
    ti, td = idx.knn(q, wl.k, predecessor=wl.predecessor, form="tree")
    st = dict(idx.last_stats)
    di, dd = idx.knn(q, wl.k, predecessor=wl.predecessor, form="dense")
    same = bool(np.array_equal(ti, di) and np.array_equal(td.view(np.uint32), dd.view(np.uint32)))
    dense_pairs = float(np.sum(q)) if wl.predecessor else float(q.size) * wl.n
    idx.free()
    return {"workload": wl.describe() + f" (tree form, {q.size} sampled queries)",
            "build_s": info["build_ms"] / 1e3, "build_wall_s": wall, "build": info,
            "queries_per_s": q.size / (st["device_ms"] / 1e3) if st["device_ms"] else None,
            "ms": st["device_ms"], "distance_evals_per_query": st["distance_evals"] / q.size,
            "dense_pairs_per_query": dense_pairs / q.size, "identical_to_dense": same}


# ------------------------------------------------------------------ batching form
def fp32_core_peak(sm_mhz):
    """Separately rounded FP32 multiply + add throughput of the CUDA cores (the plain
    form's arithmetic): SMs x 128 lanes x clock, in T ops/s.  Computed, not measured."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_mhz or 2070.0
    return sms * 128 * mhz * 1e6 / 1e12


def bench_batching(dev, steps: int = 3, warmup: int = 1, count: int = 64):
    """64 independent trees (N log-uniform [2048, 65536], D in {2,3,5}, Matern/RBF
    alternating, m = 128, k in {10,30,50}, predecessor alternating), every point of
    every tree queried: one persistent launch per step (CUDA-graph replay, autotuned
    shape) against one dense launch per tree."""
    import torch

    from covertreex_gb300 import synthetic
    from covertreex_gb300.device import CudaBatch, CudaResidualIndex, CudaVFactor
    from covertreex_gb300.residual import inducing_indices

    specs = synthetic.batch_trees(count=count)
    trees = []
    t0 = time.perf_counter()
    for sp in specs:
        X = synthetic.tree_coords(sp)
        ind = inducing_indices(sp.n, sp.m, sp.inducing_seed)
        f = CudaVFactor(X[ind].astype(np.float64), kernel_type=sp.kernel_type, variance=1.0,
                        lengthscale=sp.lengthscale, device=dev)
        V, p = f.embed_device(torch.as_tensor(X, device=dev))
        index = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=sp.lengthscale, kernel_type=sp.kernel_type,
                                  build_tree=False, device=dev)
        f.free()
        del V, p
        trees.append((sp, index, torch.arange(sp.n, dtype=torch.int64, device=dev)))
    torch.cuda.synchronize(dev)
    build_s = time.perf_counter() - t0
    b = CudaBatch(dev)
    outs = [b.add_ids(index, q, sp.k, predecessor=sp.predecessor) for sp, index, q in trees]
    t1 = time.perf_counter()
    shape = b.autotune(reps=1)
    tune_s = time.perf_counter() - t1
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        b.run(use_graph=True)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    ms = []
    for _ in range(steps):
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        b.run(use_graph=True)
        e.record(stream)
        e.synchronize()
        ms.append(a.elapsed_time(e))
    clocks = sampler.stop()
    got = [(i.clone(), d.clone()) for i, d in outs]
    # per-tree form: one ct_knn_residual (dense) launch per tree, back to back
    per = []
    for _ in range(max(1, steps - 1)):
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for (sp, index, q), (i, d) in zip(trees, outs):
            index.knn_device(q, sp.k, predecessor=sp.predecessor, form="dense", out=(i, d))
        e.record(stream)
        e.synchronize()
        per.append(a.elapsed_time(e))
    same = all(torch.equal(g[0], o[0]) and torch.equal(g[1], o[1]) for g, o in zip(got, outs))
    nq = sum(sp.n for sp in specs)
    pairs = sum(sp.n * sp.n * (0.5 if sp.predecessor else 1.0) for sp in specs)
    macs = sum(sp.n * sp.n * (0.5 if sp.predecessor else 1.0) * sp.m for sp in specs)
    step_ms = float(np.mean(ms))
    peak = fp32_core_peak(clocks.get("sm_mhz"))
    ops = 2.0 * macs / (step_ms / 1e3) / 1e12
    for sp, index, q in trees:
        index.free()
    b.free()
    return {
        "workload": f"{len(specs)} trees: N log-uniform [2048, 65536], D in {{2,3,5}}, Matern 5/2 / RBF alternating, "
                    "lengthscale U[0.5,2], m=128, k in {10,30,50}, predecessor alternating; all N ids queried",
        "trees": len(specs), "queries": nq, "pairs": pairs,
        "ms_per_step": step_ms, "queries_per_s": nq / (step_ms / 1e3),
        "per_tree_launches": {"ms_per_step": float(np.mean(per)), "queries_per_s": nq / (np.mean(per) / 1e3),
                              "launches_per_step": len(specs)},
        "speedup_vs_per_tree": float(np.mean(per)) / step_ms,
        "gpu_launches_per_step": 1, "cuda_graph": True, "shape": shape, "autotune_s": tune_s,
        "identical_to_per_tree": bool(same), "setup_s": build_s, "dtype": "f32",
        "roofline": {"bound": "fp32 cores (separately rounded multiply + add)", "achieved": ops, "peak": peak,
                     "unit": "Tops/s", "frac": ops / peak,
                     "peak_kind": "computed: SMs x 128 lanes x median SM clock (no measured FP32 peak)"},
        "clocks": clocks,
    }


# ------------------------------------------------------------------ serving form
def bench_serving(dev, rates, seconds: float):
    """Poisson request streams (10% builds of N log-uniform [1k, 128k], D=3, Matern
    5/2, m=256; 90% queries of 1..4096 new points, k in {30,50,60}) served with
    continuous batching against a 120 GB HBM budget, beside the plain per-request form."""
    from covertreex_gb300 import _lib, synthetic
    from covertreex_gb300.serving import QueryRequest, ServingEngine, latency_by_size, latency_summary

    # Library phase timing off on this thread (it is per thread): with it on, every dense
    # step's ct_batch_run waits for its kernel to read the elapsed time, which serialises the
    # serving loop's steps.
    _lib.load().ct_set_timing(0)
    out = []
    for rate in rates:
        pre, stream = synthetic.serving_stream(rate, seconds, seed=6, preload=8)
        warm = [QueryRequest(rid=10**7 + j, arrival=0.0, tree=pre[j % len(pre)].rid,
                             points=np.random.default_rng(j).standard_normal((1 + 137 * j, 3)).astype(np.float32),
                             k=(30, 50, 60)[j % 3]) for j in range(30)]
        eng = ServingEngine(hbm_budget_bytes=120e9)
        try:
            eng.preload(pre)
            eng.serve(warm, realtime=False)
            l0 = eng.launches
            t0 = time.perf_counter()
            recs = eng.serve(stream, realtime=True, time_limit=4 * seconds + 2)
            wall = time.perf_counter() - t0
            row = {"rate_req_s": rate, "requests": len(stream), "wall_s": wall,
                   "query": latency_summary(recs, "query"), "build": latency_summary(recs, "build"),
                   "query_by_points": latency_by_size(recs, "query"),
                   "peak_hbm_GB": eng.peak_bytes / 1e9, "evicted": len(eng.evicted),
                   "gpu_launches": eng.launches - l0}
        finally:
            eng.close()
        if rate <= 500:
            eng = ServingEngine(hbm_budget_bytes=120e9)
            try:
                eng.preload(pre)
                eng.serve_per_request(warm, realtime=False)
                base = eng.serve_per_request(stream, realtime=True, time_limit=4 * seconds + 2)
                row["per_request"] = latency_summary(base, "query")
                row["per_request"]["unfinished"] = len(stream) - len(base)
            finally:
                eng.close()
        out.append(row)
    return {"workload": "seeded Poisson stream (seed 6): 10% builds N log-uniform [1k,128k], D=3, Matern 5/2, "
                        "lengthscale U[0.5,2], m=256; 90% queries of 1..4096 N(0,1) points (log-uniform), "
                        "k in {30,50,60}; 8 trees preloaded",
            "hbm_budget_GB": 120, "seconds_per_rate": seconds, "rates": out,
            "p99_target_ms": 5.0}


# ------------------------------------------------------------------ one serving-shaped request
def bench_new_points_request(dev, n: int, ls: float, q: int, reps: int = 3):
    """Profiling aid: a serving-shaped tree (N(0,1) coordinates in D=3, seed 7; Matern 5/2,
    lengthscale ls, m=256 inducing points, seed 11; V and p by the GPU FP64 factor) and one
    screened request of q new N(0,1) points (seed q), k=60, timed alone."""
    import torch
    from covertreex_gb300 import _lib
    from covertreex_gb300.device import CudaResidualIndex, CudaVFactor
    from covertreex_gb300.residual import inducing_indices

    _lib.load().ct_set_timing(1)
    X = np.random.default_rng(7).standard_normal((n, 3)).astype(np.float32)
    ind = inducing_indices(n, 256, 11)
    f = CudaVFactor(X[ind].astype(np.float64), kernel_type=1, variance=1.0, lengthscale=ls, device=dev)
    V, p = f.embed_device(torch.as_tensor(X, device=dev))
    idx = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=[ls] * 3, kernel_type=1, build_tree=False,
                            query_slab=True, device=dev)
    idx.prepare_screened()
    Q = torch.as_tensor(np.random.default_rng(q).standard_normal((q, 3)).astype(np.float32), device=dev)
    qv, qp = f.embed_device(Q)
    runs = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        idx.knn_points_device(qv, qp, Q, 60, form="screened")
        torch.cuda.synchronize()
        st = dict(idx.last_stats)
        runs.append({"ms": (time.perf_counter() - t0) * 1e3,
                     **{key: st[key] for key in ("threshold_ms", "screen_ms", "rescore_ms", "overflow_queries",
                                                 "pairs_exhaustive", "pairs_rescored", "kernel_launches")}})
    _lib.load().ct_set_timing(0)
    idx.free()
    f.free()
    return {"request": {"n": n, "lengthscale": ls, "points": q, "k": 60, "m": 256, "d": 3}, "runs": runs}


# ------------------------------------------------------------------ GPU leg
def main():
    args = parse_args()
    world, rank, local = dist_env()
    from covertreex_gb300 import synthetic

    if args.impl == "reference":
        if rank == 0:
            import subprocess as sp

            sp.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
            wl = synthetic.make(args.workload, n=args.n)
            run_reference(args, wl)
        return

    import torch

    torch.cuda.set_device(local)
    dist = dist_init(world, "nccl")
    from covertreex_gb300 import _build, _lib
    from covertreex_gb300.device import CudaResidualIndex

    _build.build_library()
    L = _lib.load()
    if args.new_points_request:
        if rank == 0:
            n_s, ls_s, q_s = args.new_points_request.split(",")
            print(json.dumps(bench_new_points_request(torch.device("cuda", local), int(n_s), float(ls_s), int(q_s),
                                                      reps=max(1, args.steps))))
        return
    if args.no_headline:
        # profiling aid: the batching / serving forms alone (not the bench line)
        dev = torch.device("cuda", local)
        out = {"batching": None if args.no_batching else bench_batching(dev, count=args.batch_trees),
               "serving": None if args.no_serving else bench_serving(
                   dev, [float(x) for x in args.serving_rates.split(",") if x], args.serving_seconds)}
        if rank == 0:
            print(json.dumps(out))
        return
    wl = synthetic.make(args.workload, n=args.n)
    dev = torch.device("cuda", local)
    # The serving stream runs first, before the full-size legs allocate anything and before
    # the headline switches the library's phase timing on (served after them, with timing on,
    # its p99 at 100 / 500 / 1000 req/s was 5.6 / 11.0 / 44 ms in one run, against 4.3-4.4 /
    # 6.6-7.2 / 18.1-18.5 ms in two runs of the serving leg alone).
    serving = None
    if rank == 0 and world == 1 and not args.no_serving:
        try:
            serving = bench_serving(dev, [float(x) for x in args.serving_rates.split(",") if x],
                                    args.serving_seconds)
        except Exception as exc:
            serving = {"unavailable": repr(exc)}
    index = CudaResidualIndex(wl.v, wl.p, wl.coords, variance=wl.variance, lengthscale=[wl.lengthscale] * wl.d,
                              kernel_type=wl.kernel_type, build_tree=False, device=dev)
    q_host = shard_queries(wl.n, world, rank)
    q_dev = torch.as_tensor(q_host, device=dev)
    nq = int(q_dev.numel())
    idx_out = torch.empty((nq, wl.k), dtype=torch.int64, device=dev)
    dist_out = torch.empty((nq, wl.k), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(form):
        index.knn_device(q_dev, wl.k, predecessor=wl.predecessor, form=form, out=(idx_out, dist_out))
        return index.last_stats

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- warm-up (screened form builds its operands lazily on first use)
    L.ct_set_timing(1)
    for _ in range(max(args.warmup, 3)):
        step("screened")
    # ---- timed region (screened)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    t_wall0 = time.perf_counter()
    for s in range(args.steps):
        ev[s][0].record(stream)
        stats.append(dict(step("screened")))
        ev[s][1].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(float(np.sum(step_ms)))
    ms_per_step = total_ms / args.steps
    q_total = wl.n  # all ranks together process every query once per step
    value = q_total / (ms_per_step / 1e3)
    screened_idx = idx_out.clone()
    screened_dist = dist_out.clone()
    # FP64 check of the last timed step's output on 4096 sampled queries
    fp64 = None
    if world == 1:
        sample = np.random.default_rng(4).choice(wl.n, min(4096, wl.n), replace=False)
        fp64 = fp64_check(wl, dev, sample, screened_idx[sample].cpu().numpy(), screened_dist[sample].cpu().numpy())
        fp64["sample"] = "default_rng(4).choice(N, 4096, replace=False) rows of the last timed step"
        torch.cuda.empty_cache()

    # ---- e2e through the host-facing call (pinned host buffers, copies timed)
    q_pin = torch.as_tensor(q_host).pin_memory()
    idx_pin = torch.empty((nq, wl.k), dtype=torch.int64).pin_memory()
    dist_pin = torch.empty((nq, wl.k), dtype=torch.float32).pin_memory()
    barrier()
    e2e_ms = []
    for s in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        qd = q_pin.to(dev, non_blocking=True)
        i_d, d_d = index.knn_device(qd, wl.k, predecessor=wl.predecessor, form="screened")
        idx_pin.copy_(i_d, non_blocking=True)
        dist_pin.copy_(d_d, non_blocking=True)
        b.record(stream)
        b.synchronize()
        e2e_ms.append(a.elapsed_time(b))
    e2e_total = max_over_ranks(float(np.sum(e2e_ms)))
    e2e_value = q_total / (e2e_total / args.steps / 1e3)

    # ---- plain FP32 form (dense sweep, bit-exact reference f32 distances)
    plain = None
    agree = None
    if args.plain_steps > 0:
        step("dense")
        barrier()
        pm = []
        for _ in range(args.plain_steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step("dense")
            b.record(stream)
            b.synchronize()
            pm.append(a.elapsed_time(b))
        p_ms = max_over_ranks(float(np.mean(pm)))
        plain = {"value": q_total / (p_ms / 1e3), "unit": "queries/s", "ms_per_step": p_ms, "steps": args.plain_steps,
                 "dtype": "f32"}
        si = screened_idx.cpu().numpy()
        di = idx_out.cpu().numpy()
        same = np.all(np.sort(si, axis=1) == np.sort(di, axis=1), axis=1)
        pv = torch.as_tensor(wl.p)[torch.as_tensor(q_host)].numpy()
        well = pv >= 0.05
        agree = {"all_rows": float(same.mean()), "rows_p_ge_0.05": float(same[well].mean()) if well.any() else None}

    # ---- roofline of the dominant kernel (Pass B tensor-core screening)
    hbm, bf16_burst, bf16_sus, peak_kind = measured_peaks()
    st = stats[-1]
    pairs_main = st["screen_pairs_main"]
    screen_ms = float(np.mean([s["screen_ms"] for s in stats]))
    # algorithmic unit: one query x eligible-candidate pair, 2m flops; N(N-1)/2 pairs in
    # predecessor mode (candidates j < i), N(N-1) otherwise.  The sweep also re-screens
    # its heap-only warm-up tiles, so it screens more pairs than that (pairs_screened).
    n_all = float(wl.n)
    alg_pairs = n_all * (n_all - 1.0) / 2.0 if wl.predecessor else n_all * (n_all - 1.0)
    alg_pairs /= world  # this rank's interleaved share of the queries
    alg_flops = 2.0 * wl.m * alg_pairs
    issued_flops = 3.0 * 2.0 * wl.m * pairs_main    # hi.hi + hi.lo + lo.hi per screened pair
    achieved = alg_flops / (screen_ms / 1e3) / 1e12
    # DRAM bytes per screened pair of the sweep, from a one-pass ncu capture of a full-size
    # launch of this workload, scaled to this launch's pairs
    sweep_dram_bytes_per_pair = 11.39
    roofline = {
        "bound": "tensor", "kernel": "screen_sweep_kernel (main sweep)", "achieved": achieved,
        "peak": bf16_sus, "unit": "TFLOP/s", "frac": achieved / bf16_sus,
        "traffic": sweep_dram_bytes_per_pair * pairs_main,
        "traffic_note": "bytes per launch: 11.39 B per screened pair x pairs of this launch (ncu "
                        "dram__bytes_read.sum + dram__bytes_write.sum of one full-size sweep launch, one pass: "
                        "423.4 GB for 3.718e10 pairs)",
        "peak_kind": f"bf16_tflops_sustained ({peak_kind})",
        "tensor_issued_tflops": issued_flops / (screen_ms / 1e3) / 1e12,
        "kernel_ms": screen_ms, "algorithmic_pairs": alg_pairs, "pairs_screened": pairs_main,
        "phase_ms": {"threshold": float(np.mean([s["threshold_ms"] for s in stats])), "screen": screen_ms,
                     "rescore": float(np.mean([s["rescore_ms"] for s in stats])),
                     "call": float(np.mean([s["device_ms"] for s in stats]))},
    }

    batching = None
    euclid = None
    tree = None
    if rank == 0 and world == 1 and not args.no_batching:
        try:
            batching = bench_batching(dev, count=args.batch_trees)
        except Exception as exc:
            batching = {"unavailable": repr(exc)}

    # ---- Euclidean and tree forms (after serving: the Euclidean CPU reference starts an OpenMP pool)
    if rank == 0 and world == 1 and not args.no_euclidean:
        try:
            euclid = bench_euclidean(dev, cpu=not args.no_cpu_baseline)
        except Exception as exc:
            euclid = {"unavailable": repr(exc)}
    if rank == 0 and world == 1 and not args.no_tree:
        try:
            tree = bench_tree(wl, dev, args.tree_queries)
        except Exception as exc:
            tree = {"unavailable": repr(exc)}
    # ---- CPU baseline (rank 0, N=1 only): restated rust-hilbert on host cores, last,
    # so that its OpenMP thread pool does not share the host with the serving loop
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
            threads = os.cpu_count() or 1
            qps, otree = oracle_queries_per_s(wl, args.cpu_sample, threads, parity=False)
            cpu = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                   "sample": f"{min(args.cpu_sample, wl.n)} random query ids of the same workload, default budget "
                             f"mode; tree build {otree.build_seconds:.2f} s excluded"}
            del otree
            # the reference's parity mode (COVERTREEX_RESIDUAL_PARITY=1: no budget ladder,
            # exhaustive up to the cover-radius prune), reported separately
            pq = max(16, args.cpu_sample // 32)
            qps_p, tree_p = oracle_queries_per_s(wl, pq, threads, parity=True)
            cpu["parity_mode"] = {"value": qps_p, "unit": "queries/s", "cores": threads,
                                  "sample": f"{min(pq, wl.n)} random query ids, parity mode; tree build "
                                            f"{tree_p.build_seconds:.2f} s excluded"}
            del tree_p
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"unavailable: {exc}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step,
            "p99_ms": float(np.percentile(step_ms, 99)), "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded; no public dataset for this shape)",
            "config": {"workload": wl.describe(), "form": "screened", "N": wl.n, "D": wl.d, "m": wl.m, "k": wl.k,
                       "predecessor": wl.predecessor, "queries": wl.n, "parallelism": f"query-shard x{world}",
                       "l2": "inputs larger than L2 (V f32 512 MiB + bf16 hi/lo blocks 1 GiB)"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(q_pin.numel() * 8),
                    "d2h_bytes_per_step": int(nq * wl.k * 12)},
            "clocks": clocks,
            "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
            "plain_fp32": plain,
            "speedup_vs_plain_fp32": (value / plain["value"]) if plain else None,
            "neighbour_agreement_vs_plain": agree,
            "fp64_check": fp64,
            "wall_s_timed": t_wall,
            "batching": batching,
            "serving": serving,
            "euclidean": euclid,
            "tree": tree,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
