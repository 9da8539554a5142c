"""Serving form: a request loop that keeps built trees and their V factors on the
GPU, admits build and query requests of differing sizes against an HBM budget, and
batches query requests as they arrive (continuous batching).

No counterpart in the reference (covertreex answers one ``tree.knn`` call at a
time on the host, api/pcct.py:215-279); the device work it schedules is this
package's own:

* a build request becomes a resident tree: the FP64 factor of
  host_backend.py:202-212 (``CudaVFactor``), V and p for the N points, the
  device metric (``CudaResidualIndex``) and the screened form's BF16 operands;
* a query request of new points is embedded with the tree's factor
  (v = L^-1 k(Z, x), p = var - |v|^2) and searched with the dense form (plain
  FP32, bit-exact to the f32 oracle) when its pair count is small, or with the
  screened form (BF16 tcgen05 screening + FP64-grade rescoring) when it is large.
  The choice depends on the request's own size only, so a result is the same
  whether the request runs alone or in a mix.

Continuous batching: the loop keeps up to ``slots`` dense steps in flight on as
many CUDA streams.  Requests that arrive while steps run wait in the queue and are
admitted into the next free slot; one step embeds its requests (one call per
tree) and launches all their dense query sets in a single persistent kernel
(``CudaBatch``, replayed as a CUDA graph).  Large query sets go to a worker thread
that runs the screened form on its own stream, so they overlap the dense steps on
the device instead of holding up the loop.
Builds run on a worker thread with their own stream, admitted when the HBM
budget (resident trees + the build's estimate) allows; idle trees are evicted
least-recently-used first.
"""
from __future__ import annotations

import contextlib
import gc
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .residual import inducing_indices


@dataclass
class BuildRequest:
    rid: int
    arrival: float
    coords: np.ndarray          # [N, D] float32
    kernel_type: int = 1        # Matern 5/2
    lengthscale: float = 1.0
    inducing_count: int = 256
    seed: int = 0
    variance: float = 1.0


@dataclass
class QueryRequest:
    rid: int
    arrival: float
    tree: int                   # rid of the build request whose tree is searched
    points: np.ndarray          # [Q, D] float32
    k: int = 50


@dataclass
class RequestRecord:
    rid: int
    kind: str                   # "build" | "query"
    arrival: float
    size: int                   # N of a build, Q of a query
    start: float = float("nan")
    done: float = float("nan")
    form: str = ""
    status: str = "pending"     # "ok" | "evicted" | "rejected"
    result: Optional[tuple] = None

    @property
    def latency_ms(self) -> float:
        return (self.done - self.arrival) * 1e3


@dataclass
class ResidentTree:
    rid: int
    index: object
    factor: object
    n: int
    d: int
    m: int
    nbytes: int
    build_s: float
    last_used: float = 0.0
    inflight: int = 0


@dataclass
class _Step:
    slot: int
    event: object
    items: list = field(default_factory=list)   # (record, idx_host, dist_host, _, _)
    trees: list = field(default_factory=list)
    buffers: tuple = ()


@contextlib.contextmanager
def _gc_paused():
    enabled = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if enabled:
            gc.enable()


def estimate_tree_bytes(n: int, d: int, m: int) -> int:
    """Device bytes a resident tree will hold (metric arrays, screened operands,
    factor), plus the transient V/p of its build."""
    rows_pad = -(-n // 128) * 128
    lvl_rows = 2 * rows_pad + 128 * 8
    metric = n * m * 8 + n * d * 16 + n * 16
    screened = (rows_pad + lvl_rows) * m * 4 + (rows_pad + lvl_rows) * 16 + n * 32
    factor = 8 * (m * d + 2 * m * m)
    transient = n * m * 4 + n * d * 8 + 2 * 8 * m * min(n, 32768)
    return int(metric + screened + factor + transient)


class ServingEngine:
    def __init__(self, *, hbm_budget_bytes: float = 120e9, slots: int = 3, max_step_points: int = 16384,
                 max_step_work: float = 2.0e10, dense_pair_limit: float = 1.0e10, device=None,
                 reserve=(256, 3, 64), build_workers: int = 1, build_ctas: int = 0):
        import torch

        from .device import CudaBatch

        if not torch.cuda.is_available():
            raise RuntimeError("ServingEngine requires a CUDA device")
        self.torch = torch
        self.device = torch.device(device if device is not None else "cuda")
        self.budget = float(hbm_budget_bytes)
        self.max_step_points = int(max_step_points)
        self.max_step_work = float(max_step_work)         # sum of Q * N * m per dense step
        self.dense_pair_limit = float(dense_pair_limit)   # Q * N * m at or below which a query runs dense
        self.build_ctas = int(build_ctas)                 # grid cap of a build's FP64 embed (0 = none)
        self.trees: Dict[int, ResidentTree] = {}
        self.used_bytes = 0
        self.reserved_bytes = 0
        self.peak_bytes = 0
        self.rejected: set = set()
        self.evicted: set = set()
        # Three stream priorities: dense steps (short, latency-bound) highest, screened
        # requests next, builds lowest, so the block scheduler hands freed SMs to queued
        # step kernels first and to build kernels last (p99 at 500 req/s 6.7-8.3 -> 6.1-6.4
        # ms against one query priority).
        self.streams = [torch.cuda.Stream(self.device, priority=-3) for _ in range(slots)]
        self.batches = [CudaBatch(self.device) for _ in range(slots)]
        for b in self.batches:
            b.reserve(*reserve)
        # Builds are chains of small kernels with host synchronisations between them;
        # with build_workers > 1 several run at once, each on its own thread and stream
        # (more build throughput near saturation, a higher query p99 below it).
        self.build_streams = [torch.cuda.Stream(self.device, priority=0) for _ in range(max(1, build_workers))]
        self._build_in: "queue.Queue" = queue.Queue()
        self._build_out: "queue.Queue" = queue.Queue()
        self._workers = [threading.Thread(target=self._build_worker, args=(st,), daemon=True)
                         for st in self.build_streams]
        for w in self._workers:
            w.start()
        self.screen_stream = torch.cuda.Stream(self.device, priority=-2)
        self._screen_in: "queue.Queue" = queue.Queue()
        self._screen_out: "queue.Queue" = queue.Queue()
        self._screener = threading.Thread(target=self._screened_worker, daemon=True)
        self._screener.start()
        self.launches = 0

    # ------------------------------------------------------------------ builds
    def _build_tree(self, req: BuildRequest, st=None) -> ResidentTree:
        torch = self.torch
        from .device import CudaResidualIndex, CudaVFactor

        t0 = time.perf_counter()
        X = np.ascontiguousarray(req.coords, dtype=np.float32)
        n, d = X.shape
        idx = inducing_indices(n, req.inducing_count, req.seed)
        st = self.build_streams[0] if st is None else st
        with torch.cuda.device(self.device), torch.cuda.stream(st):
            xd = torch.as_tensor(X, device=self.device)
            f = CudaVFactor(X[idx].astype(np.float64), kernel_type=req.kernel_type, variance=req.variance,
                            lengthscale=req.lengthscale, device=self.device, stream=st)
            V, p = f.embed_device(xd, stream=st)
            index = CudaResidualIndex(V, p, xd, variance=req.variance, lengthscale=req.lengthscale,
                                      kernel_type=req.kernel_type, build_tree=False, query_slab=True,
                                      device=self.device, stream=st)
            if index.m % 32 == 0 and index.d <= 8:
                index.prepare_screened(stream=st)
            del V, p, xd
            st.synchronize()
        nbytes = index.device_bytes() + f.device_bytes()
        return ResidentTree(req.rid, index, f, n, d, index.m, nbytes, time.perf_counter() - t0)

    def _build_worker(self, st):
        from . import _lib

        # optionally the FP64 embed of a build runs on a capped grid, so that most SMs stay
        # free of build blocks (measured: a cap of 48 blocks slows builds enough that queries
        # wait for their trees at 500 req/s, so the default is no cap)
        _lib.check(_lib.load().ct_set_cta_budget(int(self.build_ctas)))
        while True:
            item = self._build_in.get()
            if item is None:
                return
            req, rec, est = item
            try:
                tree = self._build_tree(req, st)
                self._build_out.put((req, rec, est, tree, None))
            except Exception as exc:  # reported through the record
                self._build_out.put((req, rec, est, None, exc))

    def preload(self, builds: List[BuildRequest]):
        """Build trees synchronously before serving (the state a running server starts from)."""
        for req in builds:
            tree = self._build_tree(req)
            self._install(tree)

    def _install(self, tree: ResidentTree):
        tree.last_used = time.perf_counter()
        self.trees[tree.rid] = tree
        self.used_bytes += tree.nbytes
        self.peak_bytes = max(self.peak_bytes, self.used_bytes + self.reserved_bytes)

    def _evict_for(self, need: int, protect: set) -> bool:
        while self.used_bytes + self.reserved_bytes + need > self.budget:
            idle = [t for t in self.trees.values() if t.inflight == 0 and t.rid not in protect]
            if not idle:
                return False
            victim = min(idle, key=lambda t: t.last_used)
            self._drop(victim)
        return True

    def _drop(self, tree: ResidentTree):
        self.trees.pop(tree.rid, None)
        self.evicted.add(tree.rid)
        self.used_bytes -= tree.nbytes
        tree.index.free()
        tree.factor.free()

    # ------------------------------------------------------------------ queries
    def use_dense(self, q: int, tree: ResidentTree, k: int) -> bool:
        screened_ok = tree.m % 32 == 0 and tree.d <= 8 and k <= 64
        return (not screened_ok) or q * tree.n * tree.m <= self.dense_pair_limit

    def _embed_group(self, tree: ResidentTree, reqs: List[QueryRequest], st):
        """Device copies of the requests' points and their V rows / p values, embedded
        with one call for all requests on the same tree.  Returns per-request
        (x, qv, qp) views."""
        torch = self.torch
        host = np.concatenate([np.ascontiguousarray(r.points, dtype=np.float32) for r in reqs], axis=0)
        x = torch.from_numpy(host).pin_memory().to(self.device, non_blocking=True)
        qv, qp = tree.factor.embed_device(x, stream=st)
        self.launches += 3  # kernel matrix, GEMM, finalise
        out, a = [], 0
        for r in reqs:
            q = r.points.shape[0]
            out.append((x[a:a + q], qv[a:a + q], qp[a:a + q]))
            a += q
        return out

    def _launch_step(self, slot: int, items: List[tuple]) -> _Step:
        """One continuous-batching step: every dense query set of `items` in one
        persistent launch (graph replay) on the slot's stream, results copied back
        asynchronously; completion is the step's event."""
        torch = self.torch
        st = self.streams[slot]
        b = self.batches[slot]
        b.clear()
        step = _Step(slot, torch.cuda.Event())
        with torch.cuda.device(self.device), torch.cuda.stream(st):
            groups: Dict[int, list] = {}
            for rec, req, tree in items:
                tree.inflight += 1
                tree.last_used = time.perf_counter()
                step.trees.append(tree)
                groups.setdefault(tree.rid, []).append((rec, req, tree))
            # one device and one pinned host buffer for every result row of the step
            total = sum(int(req.points.shape[0]) * int(req.k) for _, req, _ in items)
            d_idx = torch.empty(total, dtype=torch.int64, device=self.device)
            d_dist = torch.empty(total, dtype=torch.float32, device=self.device)
            h_idx = torch.empty(total, dtype=torch.int64, pin_memory=True)
            h_dist = torch.empty(total, dtype=torch.float32, pin_memory=True)
            off = 0
            for members in groups.values():
                tree = members[0][2]
                views = self._embed_group(tree, [m[1] for m in members], st)
                for (rec, req, _), (x, qv, qp) in zip(members, views):
                    rec.form = "dense"
                    q, k = int(req.points.shape[0]), int(req.k)
                    sl = slice(off, off + q * k)
                    b.add_points(tree.index, qv, qp, x, k, out=(d_idx[sl].view(q, k), d_dist[sl].view(q, k)))
                    step.items.append((rec, h_idx[sl].view(q, k), h_dist[sl].view(q, k), None, None))
                    off += q * k
            b.run(use_graph=True, stream=st)
            self.launches += 1
            h_idx.copy_(d_idx, non_blocking=True)
            h_dist.copy_(d_dist, non_blocking=True)
            step.buffers = (d_idx, d_dist, h_idx, h_dist)
            step.event.record(st)
        return step

    def _finish_step(self, step: _Step, now: float):
        for rec, hi, hd, _, _ in step.items:
            rec.done = now
            rec.status = "ok"
            rec.result = (hi.numpy().copy(), hd.numpy().copy())
        for t in step.trees:
            t.inflight -= 1
        step.items = []

    def _screened_worker(self):
        """Large query sets: the screened form on its own stream, one request at a
        time, overlapping the dense steps of the main loop on the device."""
        torch = self.torch
        st = self.screen_stream
        while True:
            item = self._screen_in.get()
            if item is None:
                return
            rec, req, tree = item
            try:
                with torch.cuda.device(self.device), torch.cuda.stream(st):
                    (x, qv, qp), = self._embed_group(tree, [req], st)
                    idx, dist = tree.index.knn_points_device(qv, qp, x, req.k, form="screened", stream=st)
                    self.launches += int(tree.index.last_stats.get("kernel_launches", 0))
                    res = (idx.cpu().numpy(), dist.cpu().numpy())
                self._screen_out.put((rec, tree, res, None))
            except Exception as exc:
                self._screen_out.put((rec, tree, None, exc))

    # ------------------------------------------------------------------ loop
    def serve(self, requests: List[object], *, realtime: bool = True, time_limit: Optional[float] = None
              ) -> List[RequestRecord]:
        """Serve `requests` (arrival times in seconds from the start) and return one
        record per request.  realtime=False admits everything at t=0.  Python's cyclic
        garbage collector is suspended for the length of the loop: a full collection in
        a process holding many objects stalls the loop for tens of milliseconds."""
        with _gc_paused():
            return self._serve(requests, realtime=realtime, time_limit=time_limit)

    def _serve(self, requests: List[object], *, realtime: bool, time_limit: Optional[float]) -> List[RequestRecord]:
        reqs = sorted(requests, key=lambda r: r.arrival)
        recs = {r.rid: RequestRecord(r.rid, "build" if isinstance(r, BuildRequest) else "query", r.arrival,
                                     (r.coords.shape[0] if isinstance(r, BuildRequest) else r.points.shape[0]))
                for r in reqs}
        pending_builds: List[BuildRequest] = []
        pending_queries: List[QueryRequest] = []
        inflight: List[_Step] = []
        free_slots = list(range(len(self.streams)))
        builds_inflight = 0
        screened_inflight = 0
        t0 = time.perf_counter()
        i = 0
        left = len(reqs)
        while left > 0:
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                break
            while i < len(reqs) and (not realtime or reqs[i].arrival <= now):
                r = reqs[i]
                (pending_builds if isinstance(r, BuildRequest) else pending_queries).append(r)
                i += 1
            progressed = False
            # finished builds
            while True:
                try:
                    req, rec, est, tree, exc = self._build_out.get_nowait()
                except queue.Empty:
                    break
                builds_inflight -= 1
                progressed = True
                self.reserved_bytes -= est
                rec.done = time.perf_counter() - t0
                if exc is not None or tree is None:
                    rec.status = "rejected"
                    self.rejected.add(req.rid)
                else:
                    self._install(tree)
                    rec.status = "ok"
                left -= 1
            # finished screened requests
            while True:
                try:
                    rec, tree, res, exc = self._screen_out.get_nowait()
                except queue.Empty:
                    break
                progressed = True
                screened_inflight -= 1
                tree.inflight -= 1
                rec.done = time.perf_counter() - t0
                rec.status = "ok" if exc is None else "rejected"
                rec.result = res
                left -= 1
            # finished dense steps
            for step in list(inflight):
                if step.event.query():
                    left -= len(step.items)
                    self._finish_step(step, time.perf_counter() - t0)
                    inflight.remove(step)
                    free_slots.append(step.slot)
                    progressed = True
            # admit a build
            if builds_inflight < len(self._workers) and pending_builds:
                req = pending_builds[0]
                n, d = req.coords.shape
                est = estimate_tree_bytes(n, d, min(req.inducing_count, n))
                protect = {q.tree for q in pending_queries}
                if est > self.budget:
                    pending_builds.pop(0)
                    rec = recs[req.rid]
                    rec.status, rec.done = "rejected", now
                    self.rejected.add(req.rid)
                    left -= 1
                    progressed = True
                elif self._evict_for(est, protect):
                    pending_builds.pop(0)
                    rec = recs[req.rid]
                    rec.start = now
                    self.reserved_bytes += est
                    self.peak_bytes = max(self.peak_bytes, self.used_bytes + self.reserved_bytes)
                    builds_inflight += 1
                    self._build_in.put((req, rec, est))
                    progressed = True
            # admit queries: large ones to the screened worker, the rest into a free step slot
            if pending_queries:
                take, keep, rows, work = [], [], 0, 0.0
                slot_free = bool(free_slots)
                for q in pending_queries:
                    rec = recs[q.rid]
                    if q.tree in self.rejected or (q.tree in self.evicted and q.tree not in self.trees):
                        rec.status, rec.done = "evicted", now
                        left -= 1
                        continue
                    tree = self.trees.get(q.tree)
                    if tree is None:
                        keep.append(q)
                        continue
                    if not self.use_dense(q.points.shape[0], tree, q.k):
                        rec.start, rec.form = now, "screened"
                        tree.inflight += 1
                        tree.last_used = time.perf_counter()
                        screened_inflight += 1
                        self._screen_in.put((rec, q, tree))
                        continue
                    w = float(q.points.shape[0]) * tree.n * tree.m
                    if not slot_free or (rows > 0 and (rows + q.points.shape[0] > self.max_step_points
                                                       or work + w > self.max_step_work)):
                        keep.append(q)
                        continue
                    rows += q.points.shape[0]
                    work += w
                    rec.start = now
                    take.append((rec, q, tree))
                pending_queries = keep
                if take:
                    slot = free_slots.pop(0)
                    inflight.append(self._launch_step(slot, take))
                    progressed = True
            if not progressed:
                nxt = reqs[i].arrival - now if (realtime and i < len(reqs)) else 5e-5
                time.sleep(max(0.0, min(nxt, 5e-5)))
        for step in inflight:
            step.event.synchronize()
            self._finish_step(step, time.perf_counter() - t0)
        while screened_inflight > 0:
            rec, tree, res, exc = self._screen_out.get()
            screened_inflight -= 1
            tree.inflight -= 1
            rec.done = time.perf_counter() - t0
            rec.status = "ok" if exc is None else "rejected"
            rec.result = res
        return [recs[r.rid] for r in reqs]

    def serve_per_request(self, requests: List[object], *, realtime: bool = True,
                          time_limit: Optional[float] = None) -> List[RequestRecord]:
        """Baseline: the plain per-request form.  One request at a time in arrival
        order, each query embedded and searched alone with the dense form, each
        build done inline; nothing is batched or overlapped (garbage collection
        suspended as in serve())."""
        with _gc_paused():
            return self._serve_per_request(requests, realtime=realtime, time_limit=time_limit)

    def _serve_per_request(self, requests: List[object], *, realtime: bool,
                           time_limit: Optional[float]) -> List[RequestRecord]:
        torch = self.torch
        reqs = sorted(requests, key=lambda r: r.arrival)
        out = []
        t0 = time.perf_counter()
        st = self.streams[0]
        for r in reqs:
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                break
            if realtime and r.arrival > now:
                time.sleep(r.arrival - now)
            if isinstance(r, BuildRequest):
                rec = RequestRecord(r.rid, "build", r.arrival, r.coords.shape[0], start=time.perf_counter() - t0)
                n, d = r.coords.shape
                if not self._evict_for(estimate_tree_bytes(n, d, min(r.inducing_count, n)), set()):
                    rec.status = "rejected"
                else:
                    self._install(self._build_tree(r))
                    rec.status = "ok"
                rec.done = time.perf_counter() - t0
                out.append(rec)
                continue
            rec = RequestRecord(r.rid, "query", r.arrival, r.points.shape[0], start=time.perf_counter() - t0)
            tree = self.trees.get(r.tree)
            if tree is None:
                rec.status, rec.done = "evicted", time.perf_counter() - t0
                out.append(rec)
                continue
            tree.last_used = time.perf_counter()
            with torch.cuda.device(self.device), torch.cuda.stream(st):
                x = torch.as_tensor(np.ascontiguousarray(r.points, dtype=np.float32), device=self.device)
                qv, qp = tree.factor.embed_device(x, stream=st)
                idx, dist = tree.index.knn_points_device(qv, qp, x, r.k, form="dense", stream=st)
                res = (idx.cpu().numpy(), dist.cpu().numpy())
            rec.form, rec.status, rec.result = "dense", "ok", res
            rec.done = time.perf_counter() - t0
            out.append(rec)
        return out

    def close(self):
        for _ in self._workers:
            self._build_in.put(None)
        self._screen_in.put(None)
        for w in self._workers:
            w.join(timeout=30)
        self._screener.join(timeout=30)
        for t in list(self.trees.values()):
            t.index.free()
            t.factor.free()
        self.trees.clear()
        for b in self.batches:
            b.free()


def latency_summary(records: List[RequestRecord], kind: str = "query") -> dict:
    ok = [r for r in records if r.kind == kind and r.status == "ok"]
    lat = np.array([r.latency_ms for r in ok]) if ok else np.array([np.nan])
    span = (max(r.done for r in ok) - min(r.arrival for r in ok)) if ok else float("nan")
    pts = sum(r.size for r in ok)
    return {"count": len(ok), "dropped": sum(1 for r in records if r.kind == kind and r.status != "ok"),
            "p50_ms": float(np.nanpercentile(lat, 50)), "p99_ms": float(np.nanpercentile(lat, 99)),
            "mean_ms": float(np.nanmean(lat)), "requests_per_s": len(ok) / span if span > 0 else float("nan"),
            "points_per_s": pts / span if span > 0 else float("nan"),
            "forms": {f: sum(1 for r in ok if r.form == f) for f in ("dense", "screened")}}


def latency_by_size(records: List[RequestRecord], kind: str = "query",
                    edges=(1, 16, 256, 1024, 4097)) -> List[dict]:
    """p50 / p99 / max latency of the finished requests of one kind per size bucket
    [edges[i], edges[i+1]) (query points, or build rows); empty buckets are left out."""
    out = []
    ok = [r for r in records if r.kind == kind and r.status == "ok"]
    for lo, hi in zip(edges[:-1], edges[1:]):
        lat = np.array([r.latency_ms for r in ok if lo <= r.size < hi])
        if lat.size == 0:
            continue
        out.append({"size": f"{lo}-{hi - 1}", "count": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
                    "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max())})
    return out


__all__ = ["BuildRequest", "QueryRequest", "RequestRecord", "ServingEngine", "estimate_tree_bytes",
           "latency_by_size", "latency_summary"]
