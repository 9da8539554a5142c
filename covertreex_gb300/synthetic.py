"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is read: every array is generated from explicit seeds.  The V
matrix is built with :func:`covertreex_gb300.residual.build_residual_backend`
(FP64 Cholesky / triangular solve, as covertreex/metrics/residual/host_backend.py).

  plain_small   N=8192,   D=3, m=64,  Matern 5/2 l=1, N(0,1) coords (seed 0), inducing seed 42
  readme        N=32768,  D=3, m=256, Matern 5/2 l=1, N(0,1) coords (seed 1)
  precision     N=262144, D=8, m=512, RBF l=2, mixture of 16 Gaussians: centres U[-5,5]^8
                (seed 2), sigma 0.5, equal weights, points seed 3
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .residual import build_residual_backend


@dataclass
class Workload:
    name: str
    coords: np.ndarray
    v: np.ndarray
    p: np.ndarray
    variance: float
    lengthscale: float
    kernel_type: int
    k: int
    predecessor: bool

    @property
    def n(self) -> int:
        return int(self.coords.shape[0])

    @property
    def d(self) -> int:
        return int(self.coords.shape[1])

    @property
    def m(self) -> int:
        return int(self.v.shape[1])

    def describe(self) -> str:
        kern = "RBF" if self.kernel_type == 0 else "Matern52"
        return (f"residual-kNN N={self.n} D={self.d} m={self.m} k={self.k} "
                f"{'predecessor' if self.predecessor else 'plain'} Q=N {kern} l={self.lengthscale:g}")


def gaussian_coords(n: int, d: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)


def mixture_coords(n: int, d: int, centre_seed: int = 2, point_seed: int = 3, n_centres: int = 16,
                   sigma: float = 0.5) -> np.ndarray:
    centres = np.random.default_rng(centre_seed).uniform(-5.0, 5.0, (n_centres, d))
    r = np.random.default_rng(point_seed)
    labels = r.integers(0, n_centres, n)
    return (centres[labels] + sigma * r.standard_normal((n, d))).astype(np.float32)


def make(name: str, *, n: int | None = None) -> Workload:
    if name == "plain_small":
        n = n or 8192
        X = gaussian_coords(n, 3, 0)
        kt, ls, m, k, pred = 1, 1.0, 64, 50, True
    elif name == "readme":
        n = n or 32768
        X = gaussian_coords(n, 3, 1)
        kt, ls, m, k, pred = 1, 1.0, 256, 50, True
    elif name == "precision":
        n = n or 262144
        X = mixture_coords(n, 8)
        kt, ls, m, k, pred = 0, 2.0, 512, 50, True
    else:
        raise ValueError(f"unknown workload {name!r}")
    hb = build_residual_backend(X, seed=42, inducing_count=m, variance=1.0, lengthscale=ls, kernel_type=kt)
    return Workload(name=name, coords=X, v=hb.v_matrix, p=hb.p_diag, variance=1.0, lengthscale=ls, kernel_type=kt,
                    k=k, predecessor=pred)


# ---------------------------------------------------------------------------
# Batching workload: 64 independent trees of uneven N, D and k
# ---------------------------------------------------------------------------
@dataclass
class TreeSpec:
    n: int
    d: int
    kernel_type: int
    lengthscale: float
    m: int
    k: int
    predecessor: bool
    coord_seed: int
    inducing_seed: int


def batch_trees(count: int = 64, seed: int = 5, n_min: int = 2048, n_max: int = 65536, m: int = 128):
    """64 trees: N log-uniform in [2048, 65536], D in {2, 3, 5}, kernels alternating
    Matern 5/2 / RBF, lengthscale U[0.5, 2], m = 128, k in {10, 30, 50}, predecessor
    mode alternating.  Coordinates are N(0,1) float32 drawn per tree."""
    r = np.random.default_rng(seed)
    out = []
    for t in range(count):
        n = int(np.floor(np.exp(r.uniform(np.log(n_min), np.log(n_max)))))
        d = int(r.choice([2, 3, 5]))
        ls = float(r.uniform(0.5, 2.0))
        k = int(r.choice([10, 30, 50]))
        out.append(TreeSpec(n=n, d=d, kernel_type=1 if t % 2 == 0 else 0, lengthscale=ls, m=m, k=k,
                            predecessor=(t % 2 == 1), coord_seed=seed * 1000 + t, inducing_seed=seed * 1000 + 500 + t))
    return out


def tree_coords(spec: TreeSpec) -> np.ndarray:
    return np.random.default_rng(spec.coord_seed).standard_normal((spec.n, spec.d)).astype(np.float32)


# ---------------------------------------------------------------------------
# Serving workload: a seeded Poisson stream of build and query requests
# ---------------------------------------------------------------------------
def serving_stream(rate: float, duration: float, *, seed: int = 6, preload: int = 8, build_frac: float = 0.1,
                   n_min: int = 1024, n_max: int = 131072, m: int = 256, q_max: int = 4096,
                   ks=(30, 50, 60), working_set: int = 32, lag: float = 0.5):
    """Returns (preload_builds, stream).  Arrivals are Poisson at `rate` requests/s
    over `duration` seconds.  Builds (fraction `build_frac`): N log-uniform in
    [1k, 128k], D = 3, N(0,1) coordinates, Matern 5/2 with lengthscale U[0.5, 2],
    m = 256.  Queries: 1..4096 new N(0,1) points (log-uniform count), k drawn from
    {30, 50, 60}, against a tree drawn from the most recent `working_set` trees among
    the preloaded ones and the builds that arrived at least `lag` seconds earlier (a
    client queries a tree once it has had time to be built)."""
    from .serving import BuildRequest, QueryRequest

    r = np.random.default_rng(seed)
    rid = 0
    builds = []

    def make_build(arrival):
        nonlocal rid
        n = int(np.floor(np.exp(r.uniform(np.log(n_min), np.log(n_max)))))
        cs = int(r.integers(0, 2**31 - 1))
        X = np.random.default_rng(cs).standard_normal((n, 3)).astype(np.float32)
        b = BuildRequest(rid=rid, arrival=arrival, coords=X, kernel_type=1, lengthscale=float(r.uniform(0.5, 2.0)),
                         inducing_count=m, seed=cs % 100000)
        rid += 1
        return b

    pre = [make_build(0.0) for _ in range(preload)]
    ready = [(-1.0, b.rid) for b in pre]   # (arrival, rid) of trees a query may target
    stream = []
    t = 0.0
    while True:
        t += float(r.exponential(1.0 / rate))
        if t > duration:
            break
        if r.random() < build_frac:
            b = make_build(t)
            stream.append(b)
            ready.append((t, b.rid))
        else:
            q = int(np.clip(np.floor(np.exp(r.uniform(0.0, np.log(q_max)))), 1, q_max))
            pts = r.standard_normal((q, 3)).astype(np.float32)
            pool = [rid_ for (a, rid_) in ready if a <= t - lag][-working_set:]
            stream.append(QueryRequest(rid=rid, arrival=t, tree=int(r.choice(pool)), points=pts,
                                       k=int(r.choice(ks))))
            rid += 1
    return pre, stream
