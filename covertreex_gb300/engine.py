"""Engine registry with the GB300 engine ``"cuda"``.

Mirrors the reference's plugin surface for the residual-correlation path
(covertreex/engine.py): the ``TreeEngine`` protocol (:97-130), the ``CoverTree``
handle (:59-95), the output squeezing of ``_format_knn_output`` (:35-57), and
``get_engine`` / ``build_tree`` (:473-523).  ``CudaEngine.build`` / ``.knn`` take
the arguments of ``RustHilbertEngine.build`` / ``.knn`` (:955-1135) and run on the
GPU through libcovertree_cuda; there is no CPU fallback.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, Mapping, Optional, Protocol

import numpy as np

from .device import CudaResidualIndex
from .residual import ResidualCorrHostData, build_residual_backend

DEFAULT_ENGINE = "cuda"


def _format_knn_output(indices: np.ndarray, distances: np.ndarray, *, return_distances: bool) -> Any:
    """Legacy PCCT return shapes (covertreex/engine.py:35-57): a single query is squeezed."""
    if not return_distances:
        if indices.shape[0] == 1:
            squeezed = indices[0]
            return squeezed if squeezed.shape[0] > 1 else squeezed[0]
        return indices
    if indices.shape[0] == 1:
        si, sd = indices[0], distances[0]
        if si.shape[0] == 1:
            return si[0], sd[0]
        return si, sd
    return indices, distances


@dataclass(frozen=True)
class CoverTree:
    """Handle returned by ``TreeEngine.build``; ``knn`` delegates to the engine."""

    engine: "TreeEngine"
    handle: Any
    metric: str
    backend: Any = None
    meta: Mapping[str, Any] = field(default_factory=dict)

    def knn(self, query_points: Any, *, k: int, return_distances: bool = False, predecessor_mode: bool = False,
            context: Any = None, **kwargs) -> Any:
        return self.engine.knn(self, query_points, k=k, return_distances=return_distances,
                               predecessor_mode=predecessor_mode, context=context, runtime=None, **kwargs)

    @property
    def build_seconds(self) -> Optional[float]:
        v = self.meta.get("build_seconds")
        return float(v) if v is not None else None


class TreeEngine(Protocol):
    name: str

    def build(self, points: np.ndarray, *, runtime: Any = None, context: Any = None, batch_size: int = 512,
              seed: int = 0, build_mode: str = "batch", log_writer: Any = None, scope_cap_recorder: Any = None,
              plan_callback: Optional[Callable] = None, residual_backend: Any = None,
              residual_params: Optional[Mapping[str, Any]] = None) -> CoverTree:
        ...

    def knn(self, tree: CoverTree, query_points: Any, *, k: int, return_distances: bool,
            predecessor_mode: bool = False, context: Any = None, runtime: Any = None) -> Any:
        ...


@dataclass
class CudaHandle:
    index: CudaResidualIndex
    backend: ResidualCorrHostData
    n_points: int


class CudaEngine:
    """Residual-correlation engine on one GB300.

    Forms (``form=`` on ``knn``): ``"screened"`` (BF16 tcgen05 screening + FP64-grade
    rescoring; neighbour sets of the FP64 answer), ``"dense"`` (plain FP32, bit-exact to
    the reference's f32 batch-path distance), ``"auto"`` (screened when its limits
    hold: D <= 8, m a multiple of 32 up to 1024, k <= 64; dense otherwise).
    """

    name = "cuda"

    def build(self, points: np.ndarray, *, runtime: Any = None, context: Any = None, batch_size: int = 512,
              seed: int = 0, build_mode: str = "batch", log_writer: Any = None, scope_cap_recorder: Any = None,
              plan_callback: Optional[Callable] = None, residual_backend: Any = None,
              residual_params: Optional[Mapping[str, Any]] = None, compute_predecessor_bounds: bool = True,
              device: Any = None) -> CoverTree:
        metric = getattr(runtime, "metric", "residual_correlation") if runtime is not None else "residual_correlation"
        if metric != "residual_correlation":
            raise ValueError("cuda engine only supports the residual_correlation metric.")
        params = dict(residual_params or {})
        variance = float(params.get("variance", 1.0))
        lengthscale = params.get("lengthscale", 1.0)
        kernel_type = int(params.get("kernel_type", 0))
        chunk_size = int(params.get("chunk_size", batch_size))
        pts = np.asarray(points, dtype=np.float32)
        if residual_backend is None:
            residual_backend = build_residual_backend(
                pts, seed=int(params.get("seed", seed)), inducing_count=int(params.get("inducing_count", 512)),
                variance=variance, lengthscale=float(np.atleast_1d(lengthscale)[0]), chunk_size=chunk_size,
                kernel_type=kernel_type)
        hb = residual_backend
        coords = hb.kernel_points_f32 if getattr(hb, "kernel_points_f32", None) is not None else pts
        ls = getattr(hb, "rbf_lengthscale", None)
        if ls is None:
            ls = np.full(coords.shape[1], float(np.atleast_1d(lengthscale)[0]), dtype=np.float32)
        var = float(getattr(hb, "rbf_variance", variance))
        t0 = time.perf_counter()
        index = CudaResidualIndex(hb.v_matrix, hb.p_diag, coords, variance=var, lengthscale=ls,
                                  kernel_type=kernel_type, chunk_size=chunk_size, build_tree=False, device=device)
        build_seconds = time.perf_counter() - t0
        meta = {"build_seconds": build_seconds, "dataset_size": int(coords.shape[0]), "kernel_type": kernel_type,
                "backend_dtype": "float32", "engine": self.name}
        return CoverTree(engine=self, handle=CudaHandle(index, hb, int(coords.shape[0])), metric=metric,
                         backend="cuda", meta=meta)

    @staticmethod
    def _pick_form(index: CudaResidualIndex, k: int, form: str) -> str:
        if form != "auto":
            return form
        if index.d <= 8 and index.m % 32 == 0 and index.m <= 1024 and k <= 64:
            return "screened"
        return "dense"

    def knn(self, tree: CoverTree, query_points: Any, *, k: int, return_distances: bool,
            predecessor_mode: bool = False, context: Any = None, runtime: Any = None, form: str = "auto") -> Any:
        handle: CudaHandle = tree.handle
        queries = np.asarray(query_points)
        if queries.ndim == 1:
            queries = queries.reshape(-1, 1)
        if queries.dtype.kind not in {"i", "u"}:
            raise ValueError("cuda engine expects integer query payloads representing dataset indices.")
        if int(k) <= 0:
            raise ValueError("k must be positive")
        q = np.asarray(queries, dtype=np.int64).reshape(-1)
        chosen = self._pick_form(handle.index, int(k), form)
        idx, dist = handle.index.knn(q, int(k), predecessor=bool(predecessor_mode), form=chosen)
        return _format_knn_output(idx, dist.astype(np.float32), return_distances=return_distances)


_CUDA_ENGINE = CudaEngine()
_ENGINE_REGISTRY: Dict[str, TreeEngine] = {_CUDA_ENGINE.name: _CUDA_ENGINE}
SUPPORTED_ENGINES = tuple(_ENGINE_REGISTRY)


def get_engine(name: str) -> TreeEngine:
    engine = _ENGINE_REGISTRY.get(name)
    if engine is None:
        raise ValueError(f"Unknown engine '{name}'. Supported engines: {', '.join(SUPPORTED_ENGINES)}")
    return engine


def register_engine(engine: TreeEngine) -> None:
    _ENGINE_REGISTRY[engine.name] = engine


def build_tree(points: np.ndarray, *, runtime: Any = None, engine: Optional[str] = None, context: Any = None,
               batch_size: int = 512, seed: int = 0, build_mode: str = "batch", log_writer: Any = None,
               scope_cap_recorder: Any = None, plan_callback: Optional[Callable] = None,
               residual_backend: Any = None, residual_params: Optional[Mapping[str, Any]] = None,
               compute_predecessor_bounds: bool = True) -> CoverTree:
    engine_impl = get_engine(engine or getattr(runtime, "engine", None) or DEFAULT_ENGINE)
    return engine_impl.build(points, runtime=runtime, context=context, batch_size=batch_size, seed=seed,
                             build_mode=build_mode, log_writer=log_writer, scope_cap_recorder=scope_cap_recorder,
                             plan_callback=plan_callback, residual_backend=residual_backend,
                             residual_params=residual_params, compute_predecessor_bounds=compute_predecessor_bounds)


__all__ = ["CoverTree", "TreeEngine", "CudaEngine", "DEFAULT_ENGINE", "SUPPORTED_ENGINES", "build_tree",
           "get_engine", "register_engine"]
