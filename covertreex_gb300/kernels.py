"""GP kernels accepted by :func:`covertreex_gb300.cover_tree`.

Mirror of covertreex/kernels.py:59-132: ``RBF`` (kernel_type 0) and
``Matern52`` (kernel_type 1), each with ``lengthscale`` and ``variance``.
Calling a kernel evaluates it in FP64 on the host (for small matrices and
tests); the engine evaluates kernels on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


class Kernel:
    lengthscale: float = 1.0
    variance: float = 1.0

    @property
    def kernel_type(self) -> int:
        return 0

    def __call__(self, X1: np.ndarray, X2: np.ndarray) -> np.ndarray:  # pragma: no cover - abstract
        raise NotImplementedError


def _sq_dist(X1: np.ndarray, X2: np.ndarray) -> np.ndarray:
    X1 = np.asarray(X1, dtype=np.float64)
    X2 = np.asarray(X2, dtype=np.float64)
    diff = X1[:, None, :] - X2[None, :, :]
    return np.sum(diff * diff, axis=2)


@dataclass(frozen=True)
class RBF(Kernel):
    """K(x, y) = variance * exp(-0.5 * ||x - y||^2 / lengthscale^2)."""

    lengthscale: float = 1.0
    variance: float = 1.0

    def __call__(self, X1, X2):
        denom = max(self.lengthscale, 1e-12)
        return float(self.variance) * np.exp(-0.5 * _sq_dist(X1, X2) / (denom * denom))

    @property
    def kernel_type(self) -> int:
        return 0


@dataclass(frozen=True)
class Matern52(Kernel):
    """K(x, y) = variance * (1 + a + a^2/3) * exp(-a), a = sqrt(5) ||x - y|| / lengthscale."""

    lengthscale: float = 1.0
    variance: float = 1.0

    def __call__(self, X1, X2):
        denom = max(self.lengthscale, 1e-12)
        a = np.sqrt(5.0) * np.sqrt(_sq_dist(X1, X2)) / denom
        return float(self.variance) * (1.0 + a + a * a / 3.0) * np.exp(-a)

    @property
    def kernel_type(self) -> int:
        return 1


__all__ = ["Kernel", "RBF", "Matern52"]
