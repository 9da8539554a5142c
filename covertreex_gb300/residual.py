"""Residual-correlation host data and the V-matrix construction.

``ResidualCorrHostData`` mirrors covertreex/metrics/residual/core.py:45-155 (the
fields the hot path reads: f32 ``v_matrix``, ``p_diag``, ``kernel_diag``,
``kernel_points_f32`` plus ``rbf_variance`` / ``rbf_lengthscale``).

``build_residual_backend`` follows covertreex/metrics/residual/host_backend.py:165-246:
inducing rows Z = sorted ``default_rng(seed).choice(N, m, replace=False)``,
L = chol(K(Z,Z) + 1e-6 var I) in FP64, V = (L^-1 K(X,Z)^T)^T,
p = max(var - ||v_i||^2, 1e-9), all cast to f32.  With ``device="cuda"`` the
kernel matrices, the Cholesky and the triangular solve run on the GPU in FP64
through libcovertree_cuda (``ct_vmatrix``); ``device="host"`` keeps the
reference's numpy formulation.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np


@dataclass
class ResidualCorrHostData:
    v_matrix: np.ndarray
    p_diag: np.ndarray
    kernel_diag: np.ndarray
    kernel_points_f32: Optional[np.ndarray] = None
    rbf_variance: float = 1.0
    rbf_lengthscale: Optional[np.ndarray] = None
    kernel_type: int = 0
    chunk_size: int = 512
    inducing_idx: Optional[np.ndarray] = None
    chol_l: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        self.v_matrix = np.ascontiguousarray(self.v_matrix, dtype=np.float32)
        self.p_diag = np.ascontiguousarray(self.p_diag, dtype=np.float32).reshape(-1)
        self.kernel_diag = np.ascontiguousarray(self.kernel_diag, dtype=np.float32).reshape(-1)
        n = self.v_matrix.shape[0]
        if self.p_diag.shape[0] != n or self.kernel_diag.shape[0] != n:
            raise ValueError("p_diag and kernel_diag must have one entry per row of v_matrix")
        if self.kernel_points_f32 is not None:
            self.kernel_points_f32 = np.ascontiguousarray(self.kernel_points_f32, dtype=np.float32)
            if self.kernel_points_f32.shape[0] != n:
                raise ValueError("kernel_points_f32 must have one row per row of v_matrix")
        if self.rbf_lengthscale is not None:
            self.rbf_lengthscale = np.atleast_1d(np.asarray(self.rbf_lengthscale, dtype=np.float32))

    @property
    def num_points(self) -> int:
        return int(self.v_matrix.shape[0])

    @property
    def rank(self) -> int:
        return int(self.v_matrix.shape[1])


def _kernel_f64(x: np.ndarray, y: np.ndarray, kernel_type: int, variance: float, lengthscale: float) -> np.ndarray:
    """host_backend.py:14-43 (pairwise differences, FP64)."""
    diff = x[:, None, :] - y[None, :, :]
    sq = np.sum(diff * diff, axis=2, dtype=np.float64)
    denom = max(float(lengthscale), 1e-12)
    if kernel_type == 1:
        a = np.sqrt(5.0) * (np.sqrt(sq) / denom)
        return float(variance) * (1.0 + a + (a * a) / 3.0) * np.exp(-a)
    return float(variance) * np.exp(-0.5 * sq / (denom * denom))


def inducing_indices(n_points: int, inducing_count: int, seed: int) -> np.ndarray:
    """host_backend.py:193-200."""
    m = min(int(inducing_count), n_points)
    if m <= 0:
        m = min(32, n_points)
    if m < n_points:
        return np.sort(np.random.default_rng(seed).choice(n_points, size=m, replace=False))
    return np.arange(n_points)


def build_residual_backend(points: np.ndarray, *, seed: int, inducing_count: int, variance: float,
                           lengthscale: float, chunk_size: int = 512, kernel_type: int = 0,
                           device: str = "host") -> ResidualCorrHostData:
    pts = np.asarray(points, dtype=np.float64)
    if pts.size == 0:
        raise ValueError("Residual metric requires at least one point to configure caches.")
    n = pts.shape[0]
    idx = inducing_indices(n, inducing_count, seed)
    if device == "cuda":
        from .device import build_vmatrix_cuda

        V, p, L = build_vmatrix_cuda(pts, idx, kernel_type=int(kernel_type), variance=float(variance),
                                     lengthscale=float(lengthscale))
    else:
        Z = pts[idx]
        kmm = _kernel_f64(Z, Z, kernel_type, variance, lengthscale) + np.eye(idx.size) * (1e-6 * variance)
        L = np.linalg.cholesky(kmm)
        V = np.empty((n, idx.size), dtype=np.float64)
        for s in range(0, n, 4096):
            kxm = _kernel_f64(pts[s:s + 4096], Z, kernel_type, variance, lengthscale)
            V[s:s + 4096] = np.linalg.solve(L, kxm.T).T
        p = np.maximum(variance - np.sum(V * V, axis=1), 1e-9)
        V = V.astype(np.float32)
        p = p.astype(np.float32)
    d = pts.shape[1]
    return ResidualCorrHostData(
        v_matrix=V, p_diag=p, kernel_diag=np.full(n, variance, dtype=np.float32),
        kernel_points_f32=pts.astype(np.float32), rbf_variance=float(variance),
        rbf_lengthscale=np.full(d, lengthscale, dtype=np.float32), kernel_type=int(kernel_type),
        chunk_size=int(chunk_size), inducing_idx=idx, chol_l=np.asarray(L),
    )


__all__ = ["ResidualCorrHostData", "build_residual_backend", "inducing_indices"]
