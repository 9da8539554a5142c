"""Seeded synthetic inputs with the shapes of the benchmark configurations.

Every case is generated from explicit seeds (no datasets are read): coordinates
are i.i.d. N(0,1) float32 unless stated, V/p come from the numpy restatement of
build_residual_backend in the oracle.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def gaussian_case(n, d, m, kernel_type, lengthscale, seed, inducing_seed=42, variance=1.0):
    X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
    V, p, idx, L = O.build_residual_backend_np(X, seed=inducing_seed, inducing_count=m, variance=variance,
                                               lengthscale=lengthscale, kernel_type=kernel_type)
    return dict(X=X, V=V, p=p, var=variance, ls=np.full(d, lengthscale, np.float32), kt=kernel_type,
                inducing=idx, L=L)


def mixture_case(n, d, m, lengthscale, centre_seed=2, point_seed=3, n_centres=16, sigma=0.5, inducing_seed=42,
                 kernel_type=0):
    C = np.random.default_rng(centre_seed).uniform(-5, 5, (n_centres, d))
    r = np.random.default_rng(point_seed)
    lab = r.integers(0, n_centres, n)
    X = (C[lab] + sigma * r.standard_normal((n, d))).astype(np.float32)
    V, p, idx, L = O.build_residual_backend_np(X, seed=inducing_seed, inducing_count=m, variance=1.0,
                                               lengthscale=lengthscale, kernel_type=kernel_type)
    return dict(X=X, V=V, p=p, var=1.0, ls=np.full(d, lengthscale, np.float32), kt=kernel_type, inducing=idx, L=L)
