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
