"""Runtime-configured API: ``CoverTree(runtime).fit(points).knn(...)``.

Mirrors covertreex/api/pcct.py:59-295 (``CoverTree.fit / insert / delete / knn /
nearest / num_points``), covertreex/api/runtime.py:105-231 (``Residual``,
``Runtime``) and the residual-backend registry of
covertreex/metrics/residual/core.py (``configure_residual_correlation``,
``get_residual_backend``).  With ``Runtime(metric="residual_correlation")`` the
configured backend's V, p and coordinates are served by this package's GPU
engine; query payloads are dataset indices (an [n, 1] or [n] integer array), as
in the reference's residual path (covertreex/queries/knn.py:189-193).  With the
Euclidean metric, queries are points and the search is the exact GPU kNN.

Trees are immutable as in the reference: ``fit``, ``insert`` and ``delete``
return new ``CoverTree`` instances.  ``insert`` appends the next rows of the
configured backend (the reference's index payload: point i of the tree is
backend row i); ``delete`` removes dataset indices, and later queries and
results keep the original dataset numbering.  Runtime fields that tune the
reference's CPU traversal (scope caps, chunking, numba / rust switches) are
accepted and have no effect on the GPU search, which is exact.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Any, Dict, Optional, Tuple

import numpy as np

_RESIDUAL_BACKEND: Any = None


def configure_residual_correlation(backend: Any) -> None:
    """Register the residual backend (a ``ResidualCorrHostData`` or any object with
    ``v_matrix``, ``p_diag`` and optionally ``kernel_points_f32``, ``rbf_variance``,
    ``rbf_lengthscale``, ``kernel_type``) used by residual-correlation trees."""
    global _RESIDUAL_BACKEND
    if backend is None:
        raise ValueError("configure_residual_correlation expects a residual backend, got None.")
    _RESIDUAL_BACKEND = backend


def get_residual_backend() -> Any:
    if _RESIDUAL_BACKEND is None:
        raise RuntimeError("Residual correlation backend has not been configured.")
    return _RESIDUAL_BACKEND


def reset_residual_correlation() -> None:
    global _RESIDUAL_BACKEND
    _RESIDUAL_BACKEND = None


@dataclass(frozen=True)
class Residual:
    """Scope options of the reference's residual traversal (api/runtime.py:105-143).
    Accepted for compatibility; the GPU search is exhaustive, so they do not apply."""

    radius_floor: Optional[float] = None
    scope_cap_path: Optional[str] = None
    scope_cap_default: Optional[float] = None


@dataclass(frozen=True)
class Runtime:
    """Field-for-field the reference's ``Runtime`` (api/runtime.py:147-231).  The
    fields read here: ``metric`` ("residual_correlation" or "euclidean"), ``engine``
    ("cuda"; the reference's engine names are accepted and mapped to it),
    ``batch_order`` ("natural" / otherwise Hilbert), ``mis_seed`` / ``global_seed``."""

    backend: Optional[str] = None
    precision: Optional[str] = None
    engine: Optional[str] = None
    metric: Optional[str] = None
    devices: Optional[Tuple[str, ...]] = None
    enable_numba: Optional[bool] = None
    enable_rust: Optional[bool] = None
    enable_sparse_traversal: Optional[bool] = None
    diagnostics: Optional[bool] = None
    log_level: Optional[str] = None
    global_seed: Optional[int] = None
    mis_seed: Optional[int] = None
    conflict_graph: Optional[str] = None
    scope_segment_dedupe: Optional[bool] = None
    scope_chunk_target: Optional[int] = None
    scope_chunk_max_segments: Optional[int] = None
    degree_cap: Optional[int] = None
    batch_order: Optional[str] = None
    batch_order_seed: Optional[int] = None
    residual_grid_seed: Optional[int] = None
    prefix_schedule: Optional[str] = None
    prefix_density_low: Optional[float] = None
    prefix_density_high: Optional[float] = None
    prefix_growth_small: Optional[float] = None
    prefix_growth_mid: Optional[float] = None
    prefix_growth_large: Optional[float] = None
    residual: Optional[Residual] = None
    residual_scope_member_limit: Optional[int] = None
    residual_stream_tile: Optional[int] = None
    residual_scope_bitset: Optional[bool] = None
    residual_masked_scope_append: Optional[bool] = None
    residual_dynamic_query_block: Optional[bool] = None
    residual_dense_scope_streamer: Optional[bool] = None
    residual_level_cache_batching: Optional[bool] = None
    residual_use_static_euclidean_tree: Optional[bool] = None
    extra: Dict[str, Any] = field(default_factory=dict)

    def with_updates(self, **kwargs) -> "Runtime":
        return replace(self, **kwargs)

    @property
    def is_residual(self) -> bool:
        return (self.metric or "euclidean") == "residual_correlation"


@dataclass
class _Resident:
    """A fitted tree: the dataset rows (original numbering) and the device index."""

    metric: str
    ids: np.ndarray          # int64, increasing: dataset index of each row
    coords: np.ndarray       # f32 [rows, D] (tree points)
    index: Any               # CudaResidualIndex or EuclideanTree
    seed: int
    order: str

    @property
    def n(self) -> int:
        return int(self.ids.size)


def _resident_residual(coords: np.ndarray, ids: np.ndarray, *, seed: int, order: str) -> _Resident:
    from .device import CudaResidualIndex

    hb = get_residual_backend()
    V = np.asarray(hb.v_matrix)
    p = np.asarray(hb.p_diag).reshape(-1)
    if ids.size and int(ids.max()) >= V.shape[0]:
        raise ValueError(f"residual backend holds {V.shape[0]} rows; the tree needs index {int(ids.max())}")
    kp = getattr(hb, "kernel_points_f32", None)
    X = np.asarray(kp, dtype=np.float32)[ids] if kp is not None else coords
    ls = getattr(hb, "rbf_lengthscale", None)
    ls = np.ones(X.shape[1], np.float32) if ls is None else np.atleast_1d(np.asarray(ls, dtype=np.float32))
    var = float(getattr(hb, "rbf_variance", 1.0))
    kt = getattr(hb, "kernel_type", 0)
    kt = 1 if (kt == 1 or str(kt).lower() in ("matern52", "matern")) else 0
    index = CudaResidualIndex(V[ids], p[ids], X, variance=var, lengthscale=ls, kernel_type=kt,
                              order=order, seed=seed, build_tree=True)
    return _Resident("residual_correlation", ids, coords, index, seed, order)


def _extend_residual(old: _Resident, new_coords: np.ndarray, new_ids: np.ndarray) -> _Resident:
    """The residual tree with the configured backend's rows new_ids appended: a new device
    handle grown from the old one (its rows copied on the device, its cover tree kept and
    the new rows inserted), the old tree left valid."""
    hb = get_residual_backend()
    V = np.asarray(hb.v_matrix)
    p = np.asarray(hb.p_diag).reshape(-1)
    if new_ids.size and int(new_ids.max()) >= V.shape[0]:
        raise ValueError(f"residual backend holds {V.shape[0]} rows; the tree needs index {int(new_ids.max())}")
    kp = getattr(hb, "kernel_points_f32", None)
    X = np.asarray(kp, dtype=np.float32)[new_ids] if kp is not None else new_coords
    index = old.index.extend(V[new_ids], p[new_ids], X)
    return _Resident("residual_correlation", np.concatenate([old.ids, new_ids]),
                     np.concatenate([old.coords, new_coords], axis=0), index, old.seed, old.order)


def _resident_euclidean(coords: np.ndarray, ids: np.ndarray, *, seed: int, order: str) -> _Resident:
    from .euclidean import EuclideanTree

    return _Resident("euclidean", ids, coords, EuclideanTree(coords), seed, order)


@dataclass
class CoverTree:
    """``CoverTree(runtime).fit(points)``, ``.insert(points)``, ``.delete(indices)``,
    ``.knn(queries, k=, return_distances=, predecessor_mode=)`` and ``.nearest``."""

    runtime: Runtime = field(default_factory=Runtime)
    tree: Optional[_Resident] = None

    # ------------------------------------------------------------------
    def _seed(self, mis_seed: Optional[int]) -> int:
        for s in (mis_seed, self.runtime.mis_seed, self.runtime.global_seed):
            if s is not None:
                return int(s)
        return 0

    def _order(self, apply_batch_order: Optional[bool]) -> str:
        if apply_batch_order is False or (self.runtime.batch_order or "").lower() == "natural":
            return "natural"
        return "hilbert"

    def _make(self, coords: np.ndarray, ids: np.ndarray, seed: int, order: str) -> _Resident:
        if self.runtime.engine not in (None, "cuda", "rust-hilbert", "rust-natural", "rust-fast", "python-numba"):
            raise ValueError(f"Unknown engine '{self.runtime.engine}'.")
        if self.runtime.is_residual:
            return _resident_residual(coords, ids, seed=seed, order=order)
        return _resident_euclidean(coords, ids, seed=seed, order=order)

    def _require_tree(self) -> _Resident:
        if self.tree is None:
            raise RuntimeError("CoverTree has not been fitted; call fit() first.")
        return self.tree

    # ------------------------------------------------------------------
    def fit(self, points: Any, *, apply_batch_order: bool = True, mis_seed: Optional[int] = None,
            return_plan: bool = False):
        coords = np.asarray(points, dtype=np.float32)
        if coords.ndim == 1:
            coords = coords.reshape(-1, 1)
        if coords.shape[0] == 0:
            raise ValueError("Cannot fit a cover tree on zero points.")
        ids = np.arange(coords.shape[0], dtype=np.int64)
        res = self._make(coords, ids, self._seed(mis_seed), self._order(apply_batch_order))
        out = CoverTree(runtime=self.runtime, tree=res)
        return (out, {"inserted": res.n}) if return_plan else out

    def insert(self, batch_points: Any, *, mis_seed: Optional[int] = None, apply_batch_order: Optional[bool] = None,
               return_plan: bool = False):
        old = self._require_tree()
        new = np.asarray(batch_points, dtype=np.float32)
        if new.ndim == 1:
            new = new.reshape(-1, old.coords.shape[1])
        if new.shape[1] != old.coords.shape[1]:
            raise ValueError(f"points have {new.shape[1]} coordinates, the tree {old.coords.shape[1]}")
        start = int(old.ids.max()) + 1 if old.n else 0
        ids = np.concatenate([old.ids, np.arange(start, start + new.shape[0], dtype=np.int64)])
        coords = np.concatenate([old.coords, new], axis=0)
        seed = self._seed(mis_seed) if mis_seed is not None else old.seed
        order = self._order(apply_batch_order) if apply_batch_order is not None else old.order
        if old.metric == "residual_correlation" and seed == old.seed and order == old.order and new.shape[0]:
            # the new rows go into a handle grown from the resident one (no rebuild)
            res = _extend_residual(old, new, ids[old.n:])
        else:
            res = self._make(coords, ids, seed, order)
        out = CoverTree(runtime=self.runtime, tree=res)
        return (out, {"inserted": int(new.shape[0])}) if return_plan else out

    def delete(self, indices: Any, *, return_plan: bool = False):
        old = self._require_tree()
        remove = np.unique(np.asarray(indices, dtype=np.int64).reshape(-1))
        keep = ~np.isin(old.ids, remove)
        if not keep.any():
            raise ValueError("delete would remove every point of the tree")
        if old.metric == "residual_correlation":
            # the kept rows are gathered on the device and the handle built from them
            res = _Resident("residual_correlation", old.ids[keep], old.coords[keep],
                            old.index.subset(np.nonzero(keep)[0]), old.seed, old.order)
        else:
            res = self._make(old.coords[keep], old.ids[keep], old.seed, old.order)
        out = CoverTree(runtime=self.runtime, tree=res)
        return (out, {"removed": int((~keep).sum())}) if return_plan else out

    # ------------------------------------------------------------------
    def knn(self, query_points: Any, *, k: int, return_distances: bool = False, predecessor_mode: bool = False,
            form: str = "auto"):
        from .engine import CudaEngine, _format_knn_output

        res = self._require_tree()
        k = int(k)
        if k <= 0:
            raise ValueError("k must be positive.")
        if k > res.n:
            raise ValueError("k cannot exceed the number of points in the tree.")
        if res.metric == "euclidean":
            qp = np.asarray(query_points, dtype=np.float32)
            idx, dist = res.index.knn_device(qp, k, predecessor=bool(predecessor_mode))
            idx, dist = idx.cpu().numpy(), dist.cpu().numpy()
            out = np.where(idx >= 0, res.ids[np.maximum(idx, 0)], -1)
            return _format_knn_output(out, dist, return_distances=return_distances)
        q = np.asarray(query_points)
        if q.dtype.kind not in {"i", "u"}:
            raise ValueError("residual_correlation queries are dataset indices (an integer array).")
        q = q.astype(np.int64).reshape(-1)
        rows = np.searchsorted(res.ids, q)
        rows_c = np.minimum(rows, res.n - 1)
        if q.size and (np.any(q < 0) or np.any(res.ids[rows_c] != q)):
            raise ValueError("Residual point decoder received unknown payload.")
        chosen = CudaEngine._pick_form(res.index, k, form)
        idx, dist = res.index.knn(rows_c, k, predecessor=bool(predecessor_mode), form=chosen)
        out = np.where(idx >= 0, res.ids[np.maximum(idx, 0)], -1)
        return _format_knn_output(out, dist.astype(np.float32), return_distances=return_distances)

    def nearest(self, query_points: Any, *, return_distances: bool = False):
        return self.knn(query_points, k=1, return_distances=return_distances)

    @property
    def num_points(self) -> int:
        return 0 if self.tree is None else self.tree.n


__all__ = ["CoverTree", "Runtime", "Residual", "configure_residual_correlation", "get_residual_backend",
           "reset_residual_correlation"]
