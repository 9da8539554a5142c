"""``cover_tree`` factory and ``BuiltCoverTree`` (covertreex/api/factory.py:40-348).

Same signature as the reference's factory.  ``engine`` defaults to ``"cuda"``;
the residual metric is selected by ``kernel=`` (V built here in FP64 exactly as
the reference's host backend) or by a caller's ``v_matrix=`` / ``p_diag=``.
``kernel_diag`` defaults to ones (variance 1), as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional, Sequence

import numpy as np

from .engine import CoverTree, get_engine
from .kernels import Kernel
from .residual import ResidualCorrHostData, build_residual_backend


@dataclass
class BuiltCoverTree:
    _tree: Any
    _n_points: int
    _is_residual: bool = True

    def knn(self, k: int, *, queries: Optional[np.ndarray | Sequence[int]] = None, return_distances: bool = False,
            predecessor_mode: bool = False, form: str = "auto"):
        """k nearest neighbours of `queries` (dataset ids for the residual metric,
        points for Euclidean), all N points when None.  Rows are padded with -1
        (and FLT_MAX distances) when fewer than k neighbours exist."""
        if queries is None:
            query_data = np.arange(self._n_points, dtype=np.int64).reshape(-1, 1)
        else:
            query_data = np.asarray(queries)
            if query_data.ndim == 1 and self._is_residual:
                query_data = query_data.reshape(-1, 1)
        return self._tree.knn(query_data, k=k, return_distances=return_distances, predecessor_mode=predecessor_mode,
                              form=form)

    @property
    def n_points(self) -> int:
        return self._n_points

    @property
    def build_time(self) -> Optional[float]:
        """Seconds spent building the device index.  The default search forms (screened,
        dense) need no cover tree, so by default no tree is built and this is the time of
        the device-resident metric setup (V relayout, scaled coordinates, norms, copies);
        the reference's ``build_time`` counts its Rust tree build instead.  The cover tree
        itself is built only for the tree form."""
        return self._tree.build_seconds

    def __repr__(self) -> str:
        return f"BuiltCoverTree(n={self._n_points}, metric={'residual' if self._is_residual else 'euclidean'!r})"


def cover_tree(coords: np.ndarray, *, kernel: Optional[Kernel] = None, v_matrix: Optional[np.ndarray] = None,
               p_diag: Optional[np.ndarray] = None, kernel_diag: Optional[np.ndarray] = None,
               inducing_count: int = 512, seed: int = 42, chunk_size: int = 512, engine: str = "cuda",
               device: Any = None, vmatrix_device: str = "host") -> BuiltCoverTree:
    """``vmatrix_device="cuda"`` builds V and p from ``kernel`` on the GPU in FP64
    (``ct_vfactor_*``); the default ``"host"`` keeps the reference's numpy algebra."""
    coords_f32 = np.asarray(coords, dtype=np.float32)
    if coords_f32.ndim == 1:
        coords_f32 = coords_f32.reshape(-1, 1)
    n_points = coords_f32.shape[0]
    use_residual = kernel is not None or v_matrix is not None
    if not use_residual:
        from .euclidean import EuclideanTree

        return BuiltCoverTree(_tree=EuclideanTree(coords_f32, device=device), _n_points=n_points, _is_residual=False)
    if kernel is not None and v_matrix is not None:
        raise ValueError("Provide either 'kernel' or 'v_matrix', not both.")
    if v_matrix is not None:
        if p_diag is None:
            raise ValueError("p_diag is required when v_matrix is provided.")
        kd = np.ones(n_points, dtype=np.float32) if kernel_diag is None else np.asarray(kernel_diag, np.float32)
        backend = ResidualCorrHostData(v_matrix=v_matrix, p_diag=p_diag, kernel_diag=kd,
                                       kernel_points_f32=coords_f32, rbf_variance=1.0,
                                       rbf_lengthscale=np.ones(coords_f32.shape[1], np.float32), kernel_type=0,
                                       chunk_size=chunk_size)
        params = {"variance": 1.0, "lengthscale": 1.0, "kernel_type": 0, "chunk_size": chunk_size}
    else:
        backend = build_residual_backend(coords_f32, seed=seed, inducing_count=inducing_count,
                                         variance=kernel.variance, lengthscale=kernel.lengthscale,
                                         chunk_size=chunk_size, kernel_type=kernel.kernel_type,
                                         device=vmatrix_device)
        params = {"variance": kernel.variance, "lengthscale": kernel.lengthscale,
                  "kernel_type": kernel.kernel_type, "chunk_size": chunk_size}
    engine_impl = get_engine(engine)
    tree: CoverTree = engine_impl.build(coords_f32, residual_backend=backend, residual_params=params,
                                        compute_predecessor_bounds=True, device=device)
    return BuiltCoverTree(_tree=tree, _n_points=n_points, _is_residual=True)


__all__ = ["cover_tree", "BuiltCoverTree"]
