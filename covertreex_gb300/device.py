"""Device-side handle: owns a ``ct_tree`` of libcovertree_cuda and its inputs.

PyTorch is used only to hold device memory and to name the CUDA stream; all
arithmetic happens in the library's own kernels.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("covertreex_gb300 requires a CUDA device (GB300, sm_103a); none is visible")
    return torch


def _stream_ptr(stream) -> ctypes.c_void_p:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(int(s.cuda_stream))


def _as_device(a, dtype, device):
    torch = _torch()
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=dtype)
    else:
        t = torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device)
    return t.contiguous()


class CudaResidualIndex:
    """A residual-correlation metric (and optionally its cover tree) resident on one GPU.

    Mirrors what ``build_pcct2_residual_tree`` returns in the reference
    (src/lib.rs:1374-1564): the tree handle plus its cached f32 copies.
    """

    def __init__(self, v_matrix, p_diag, coords, *, variance: float = 1.0, lengthscale=1.0, kernel_type: int = 0,
                 chunk_size: int = 512, order: str = "hilbert", seed: int = 0, build_tree: bool = True,
                 query_slab: bool = False, device=None, stream=None):
        torch = _torch()
        self.device = torch.device(device if device is not None else "cuda")
        L = _lib.load()
        v = _as_device(v_matrix, torch.float32, self.device)
        p = _as_device(p_diag, torch.float32, self.device).reshape(-1)
        c = _as_device(coords, torch.float32, self.device)
        if c.dim() == 1:
            c = c.reshape(-1, 1)
        if v.dim() != 2 or v.shape[0] != p.shape[0] or c.shape[0] != v.shape[0]:
            raise ValueError("v_matrix [N,m], p_diag [N] and coords [N,D] must agree on N")
        self.n, self.m = int(v.shape[0]), int(v.shape[1])
        self.d = int(c.shape[1])
        ls = np.atleast_1d(np.asarray(lengthscale, dtype=np.float32))
        self.lengthscale = ls
        self.variance = float(variance)
        self.kernel_type = int(kernel_type)
        self.has_tree = bool(build_tree)
        order_code = _lib.CT_ORDER_NATURAL if str(order).lower() == "natural" else _lib.CT_ORDER_HILBERT
        flags = 0 if build_tree else _lib.CT_BUILD_METRIC_ONLY
        if query_slab:
            flags |= _lib.CT_BUILD_QUERY_SLAB
        h = ctypes.c_void_p()
        ls_c = (ctypes.c_float * ls.size)(*ls.tolist())
        with torch.cuda.device(self.device):
            rc = L.ct_build_residual(v.data_ptr(), p.data_ptr(), c.data_ptr(), self.n, self.m, self.d,
                                     self.variance, ls_c, int(ls.size), self.kernel_type, int(chunk_size),
                                     order_code, int(seed) & 0xFFFFFFFFFFFFFFFF, flags, _stream_ptr(stream),
                                     ctypes.byref(h))
        _lib.check(rc)
        self._h = h
        self.last_stats: dict = {}
        self.last_form: str = ""
        self.build_params = {"chunk_size": int(chunk_size), "order": str(order), "seed": int(seed),
                             "build_tree": bool(build_tree), "query_slab": bool(query_slab)}

    def extend(self, v_new, p_new, coords_new, *, stream=None) -> "CudaResidualIndex":
        """A NEW index over this index's rows followed by the given rows (dataset ids n ..
        n + len - 1), the counterpart of the reference's immutable ``CoverTree.insert``
        (api/pcct.py:171-197): this index stays valid.  Existing rows are copied device to
        device; a cover tree, if built, keeps its nodes and receives the new rows by
        prefix-doubling group insertion (ct_tree_extend)."""
        torch = _torch()
        if self._h is None:
            raise RuntimeError("index has been freed")
        v = _as_device(v_new, torch.float32, self.device)
        p = _as_device(p_new, torch.float32, self.device).reshape(-1)
        c = _as_device(coords_new, torch.float32, self.device)
        if c.dim() == 1:
            c = c.reshape(-1, self.d)
        b = int(p.shape[0])
        if v.shape != (b, self.m) or c.shape != (b, self.d):
            raise ValueError(f"new rows must be V [b, {self.m}], p [b] and coords [b, {self.d}]")
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().ct_tree_extend(self._h, v.data_ptr(), p.data_ptr(), c.data_ptr(), b,
                                                  _stream_ptr(stream), ctypes.byref(h)))
        out = CudaResidualIndex.__new__(CudaResidualIndex)
        out.device = self.device
        out.n, out.m, out.d = self.n + b, self.m, self.d
        out.lengthscale = self.lengthscale
        out.variance = self.variance
        out.kernel_type = self.kernel_type
        out.has_tree = self.has_tree
        out._h = h
        out.last_stats = {}
        out.last_form = ""
        out.build_params = dict(self.build_params)
        return out

    def subset(self, rows, *, stream=None) -> "CudaResidualIndex":
        """A NEW index over the given rows (ascending row numbers of this index), renumbered
        0 .. len - 1: the counterpart of the reference's immutable ``CoverTree.delete``.
        Rows are gathered on the device (ct_tree_subset); this index stays valid."""
        torch = _torch()
        if self._h is None:
            raise RuntimeError("index has been freed")
        r = _as_device(np.asarray(rows, dtype=np.int64).reshape(-1), torch.int64, self.device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().ct_tree_subset(self._h, r.data_ptr(), int(r.shape[0]), _stream_ptr(stream),
                                                  ctypes.byref(h)))
        out = CudaResidualIndex.__new__(CudaResidualIndex)
        out.device = self.device
        out.n, out.m, out.d = int(r.shape[0]), self.m, self.d
        out.lengthscale = self.lengthscale
        out.variance = self.variance
        out.kernel_type = self.kernel_type
        out.has_tree = self.has_tree
        out._h = h
        out.last_stats = {}
        out.last_form = ""
        out.build_params = dict(self.build_params)
        return out

    # ------------------------------------------------------------------
    def knn_device(self, q_ids, k: int, *, predecessor: bool = False, form: str = "dense", stream=None,
                   out=None):
        """Device-in / device-out kNN.  q_ids: int64 CUDA tensor.  Returns (idx, dist) CUDA tensors."""
        torch = _torch()
        if self._h is None:
            raise RuntimeError("index has been freed")
        k = int(k)
        if k <= 0:
            raise ValueError("k must be positive")
        q = _as_device(q_ids, torch.int64, self.device).reshape(-1)
        nq = int(q.shape[0])
        if out is None:
            idx = torch.empty((nq, k), dtype=torch.int64, device=self.device)
            dist = torch.empty((nq, k), dtype=torch.float32, device=self.device)
        else:
            idx, dist = out
        st = _lib.CtStats()
        rc = _lib.load().ct_knn_residual(self._h, q.data_ptr(), nq, k, 1 if predecessor else 0,
                                         _lib.FORMS[form], idx.data_ptr(), dist.data_ptr(), ctypes.byref(st),
                                         _stream_ptr(stream))
        _lib.check(rc)
        self.last_stats = st.as_dict()
        self.last_form = form
        return idx, dist

    # ------------------------------------------------------------------ telemetry
    def last_query_telemetry(self):
        """The last query's counters in the reference's ResidualQueryTelemetry shape
        (src/telemetry.rs:1-19, returned by CoverTreeWrapper.last_query_telemetry,
        src/lib.rs:357-363), with the GPU forms' own counters under "gpu"."""
        from .telemetry import query_telemetry

        return query_telemetry(self.last_stats, self.last_form) if self.last_stats else None

    def clear_last_query_telemetry(self):
        self.last_stats = {}
        self.last_form = ""

    # ------------------------------------------------------------------ persistence
    def save(self, path) -> None:
        """Write the index to a flat binary file: a JSON header line, then V [n, m],
        p [n] and the raw coordinates [n, d] as little-endian f32.  ``load`` rebuilds
        the device layouts and the cover tree from them with the same parameters, so
        the loaded index answers every query exactly as this one."""
        from .persist import save_index

        save_index(self, path)

    @classmethod
    def load(cls, path, device=None, stream=None) -> "CudaResidualIndex":
        from .persist import load_index

        return load_index(path, device=device, stream=stream)

    def inputs_device(self, stream=None):
        """Device copies of (V natural [n, m], p [n], raw coordinates [n, d])."""
        torch = _torch()
        v = torch.empty((self.n, self.m), dtype=torch.float32, device=self.device)
        p = torch.empty((self.n,), dtype=torch.float32, device=self.device)
        c = torch.empty((self.n, self.d), dtype=torch.float32, device=self.device)
        _lib.check(_lib.load().ct_tree_inputs(self._h, v.data_ptr(), p.data_ptr(), c.data_ptr(), _stream_ptr(stream)))
        return v, p, c

    def knn(self, q_ids, k: int, *, predecessor: bool = False, form: str = "dense"):
        """Host-in / host-out kNN (numpy int64 [Q,k], float32 [Q,k])."""
        q = np.asarray(q_ids, dtype=np.int64).reshape(-1)
        if q.size and (q.min() < 0 or q.max() >= self.n):
            raise ValueError("Residual point decoder received out-of-range indices.")
        idx, dist = self.knn_device(q, k, predecessor=predecessor, form=form)
        return idx.cpu().numpy(), dist.cpu().numpy()

    def knn_points_device(self, qv, qp, qcoords, k: int, *, form: str = "dense", stream=None, out=None):
        """kNN of NEW points: V rows qv [Q,m] (e.g. from CudaVFactor.embed_device), p values
        qp [Q] and raw coordinates qcoords [Q,d].  form: "dense" (plain FP32) or
        "screened".  Returns (idx, dist) CUDA tensors."""
        torch = _torch()
        qv = _as_device(qv, torch.float32, self.device)
        qp = _as_device(qp, torch.float32, self.device).reshape(-1)
        qc = _as_device(qcoords, torch.float32, self.device).reshape(qp.shape[0], self.d)
        if qv.shape != (qp.shape[0], self.m):
            raise ValueError(f"qv must be [Q, {self.m}]")
        nq, k = int(qp.shape[0]), int(k)
        if out is None:
            idx = torch.empty((nq, k), dtype=torch.int64, device=self.device)
            dist = torch.empty((nq, k), dtype=torch.float32, device=self.device)
        else:
            idx, dist = out
        st = _lib.CtStats()
        _lib.check(_lib.load().ct_knn_residual_points(self._h, qv.data_ptr(), qp.data_ptr(), qc.data_ptr(), nq, k,
                                                      _lib.FORMS[form], idx.data_ptr(), dist.data_ptr(),
                                                      ctypes.byref(st), _stream_ptr(stream)))
        self.last_stats = st.as_dict()
        return idx, dist

    def prepare_screened(self, stream=None):
        """Build the screened form's BF16 operands now (otherwise done by the first screened query)."""
        _lib.check(_lib.load().ct_prepare_screened(self._h, _stream_ptr(stream)))

    def device_bytes(self) -> int:
        b = ctypes.c_int64()
        _lib.check(_lib.load().ct_tree_device_bytes(self._h, ctypes.byref(b)))
        return int(b.value)

    def debug_screen_dots(self, rows_a, rows_b):
        """Raw BF16-screened dot products (hi.hi + hi.lo + lo.hi) of 128 x 256 dataset rows."""
        torch = _torch()
        ra = torch.full((128,), -1, dtype=torch.int32, device=self.device)
        rb = torch.full((256,), -1, dtype=torch.int32, device=self.device)
        a = torch.as_tensor(np.asarray(rows_a, dtype=np.int32))
        b = torch.as_tensor(np.asarray(rows_b, dtype=np.int32))
        ra[: a.numel()] = a.to(self.device)
        rb[: b.numel()] = b.to(self.device)
        out = torch.empty((128, 256), dtype=torch.float32, device=self.device)
        rc = _lib.load().ct_debug_screen_dots(self._h, ra.data_ptr(), rb.data_ptr(), out.data_ptr(), _stream_ptr(None))
        _lib.check(rc)
        return out.cpu().numpy()

    def tree_arrays(self):
        torch = _torch()
        if not self.has_tree:
            raise RuntimeError("index was built without a cover tree")
        n = self.n
        parents = torch.empty(n, dtype=torch.int64, device=self.device)
        levels = torch.empty(n, dtype=torch.int32, device=self.device)
        si = torch.empty(n, dtype=torch.float32, device=self.device)
        order = torch.empty(n, dtype=torch.int64, device=self.device)
        smin = torch.empty(n, dtype=torch.int64, device=self.device)
        rc = _lib.load().ct_tree_arrays(self._h, parents.data_ptr(), levels.data_ptr(), si.data_ptr(),
                                        order.data_ptr(), smin.data_ptr(), _stream_ptr(None))
        _lib.check(rc)
        torch.cuda.synchronize(self.device)
        return {"parents": parents.cpu().numpy(), "levels": levels.cpu().numpy(), "si": si.cpu().numpy(),
                "node_to_dataset": order.cpu().numpy(), "subtree_min": smin.cpu().numpy()}

    def build_info(self) -> dict:
        """Telemetry of the device cover-tree build (``ct_tree_build_info``)."""
        vals = [ctypes.c_int64() for _ in range(5)]
        ms = ctypes.c_double()
        _lib.check(_lib.load().ct_tree_build_info(self._h, *[ctypes.byref(v) for v in vals], ctypes.byref(ms)))
        keys = ("groups", "conflict_edges", "selected", "side_rows", "roots")
        out = {k: int(v.value) for k, v in zip(keys, vals)}
        out["build_ms"] = float(ms.value)
        return out

    def free(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().ct_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class CudaBatch:
    """Batching form (``ct_batch_*``): query sets against many resident
    :class:`CudaResidualIndex` trees in one persistent launch, optionally replayed
    as a CUDA graph.  Outputs are allocated here and returned by ``add_*``; they are
    valid once :meth:`run` has completed on its stream."""

    def __init__(self, device=None):
        torch = _torch()
        self.device = torch.device(device if device is not None else "cuda")
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().ct_batch_create(ctypes.byref(self._h)))
        self._keep: list = []
        self.last_stats: dict = {}

    def _outputs(self, nq, k, out):
        torch = _torch()
        if out is not None:
            return out
        return (torch.empty((nq, k), dtype=torch.int64, device=self.device),
                torch.empty((nq, k), dtype=torch.float32, device=self.device))

    def add_ids(self, index: CudaResidualIndex, q_ids, k: int, *, predecessor: bool = False, out=None):
        torch = _torch()
        q = _as_device(q_ids, torch.int64, self.device).reshape(-1)
        idx, dist = self._outputs(int(q.shape[0]), int(k), out)
        _lib.check(_lib.load().ct_batch_add_ids(self._h, index._h, q.data_ptr(), int(q.shape[0]), int(k),
                                                1 if predecessor else 0, idx.data_ptr(), dist.data_ptr()))
        self._keep += [index, q, idx, dist]
        return idx, dist

    def add_points(self, index: CudaResidualIndex, qv, qp, qcoords, k: int, *, out=None):
        torch = _torch()
        qv = _as_device(qv, torch.float32, self.device)
        qp = _as_device(qp, torch.float32, self.device).reshape(-1)
        qc = _as_device(qcoords, torch.float32, self.device).reshape(qp.shape[0], index.d)
        if qv.shape != (qp.shape[0], index.m):
            raise ValueError(f"qv must be [Q, {index.m}]")
        idx, dist = self._outputs(int(qp.shape[0]), int(k), out)
        _lib.check(_lib.load().ct_batch_add_points(self._h, index._h, qv.data_ptr(), qp.data_ptr(), qc.data_ptr(),
                                                   int(qp.shape[0]), int(k), idx.data_ptr(), dist.data_ptr()))
        self._keep += [index, qv, qp, qc, idx, dist]
        return idx, dist

    def set_shape(self, qt: int = 0, ctas_per_sm: int = 0, items_per_slot: int = 0):
        _lib.check(_lib.load().ct_batch_set_shape(self._h, int(qt), int(ctas_per_sm), int(items_per_slot)))

    def reserve(self, m: int, d: int, k: int):
        """Size the launch for at least (m, d, k) so varying mixes reuse one shape and graph."""
        _lib.check(_lib.load().ct_batch_reserve(self._h, int(m), int(d), int(k)))

    def autotune(self, reps: int = 1, stream=None):
        q, c, i = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.check(_lib.load().ct_batch_autotune(self._h, int(reps), _stream_ptr(stream), ctypes.byref(q),
                                                 ctypes.byref(c), ctypes.byref(i)))
        return {"qt": q.value, "ctas_per_sm": c.value, "items_per_slot": i.value}

    def run(self, *, use_graph: bool = True, stream=None):
        st = _lib.CtStats()
        _lib.check(_lib.load().ct_batch_run(self._h, 1 if use_graph else 0, ctypes.byref(st), _stream_ptr(stream)))
        self.last_stats = st.as_dict()
        return self.last_stats

    def shape(self):
        q, c, i, g = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        items = ctypes.c_int64()
        _lib.check(_lib.load().ct_batch_get_shape(self._h, ctypes.byref(q), ctypes.byref(c), ctypes.byref(i),
                                                  ctypes.byref(g), ctypes.byref(items)))
        return {"qt": q.value, "ctas_per_sm": c.value, "items_per_slot": i.value, "grid": g.value,
                "items": items.value}

    def clear(self):
        _lib.check(_lib.load().ct_batch_clear(self._h))
        self._keep = []

    def free(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().ct_batch_free(self._h)
        self._h = None
        self._keep = []

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class CudaVFactor:
    """FP64 factor of the residual backend on one GPU (``ct_vfactor_*``).

    ``chol(K(Z,Z) + 1e-6 var I)`` and its inverse stay resident; :meth:`embed` turns
    points (dataset rows, or new query points when serving) into f32 V rows and p
    values exactly as build_residual_backend does for the dataset
    (covertreex/metrics/residual/host_backend.py:202-219).
    """

    def __init__(self, inducing_points, *, kernel_type: int = 0, variance: float = 1.0, lengthscale: float = 1.0,
                 device=None, stream=None):
        torch = _torch()
        self.device = torch.device(device if device is not None else "cuda")
        L = _lib.load()
        z = _as_device(inducing_points, torch.float64, self.device)
        if z.dim() == 1:
            z = z.reshape(-1, 1)
        self.m, self.d = int(z.shape[0]), int(z.shape[1])
        self.kernel_type, self.variance, self.lengthscale = int(kernel_type), float(variance), float(lengthscale)
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(L.ct_vfactor_create(ctypes.c_void_p(z.data_ptr()), self.m, self.d, self.kernel_type,
                                           self.variance, self.lengthscale, _stream_ptr(stream),
                                           ctypes.byref(self._h)))

    def embed_device(self, x, *, stream=None):
        """V rows [n, m] and p [n] (device f32 tensors) for points x [n, d]."""
        torch = _torch()
        xs = _as_device(x, torch.float64, self.device)
        if xs.dim() == 1:
            xs = xs.reshape(-1, self.d)
        if xs.shape[1] != self.d:
            raise ValueError(f"points have {xs.shape[1]} coordinates, the factor {self.d}")
        n = int(xs.shape[0])
        v = torch.empty((n, self.m), dtype=torch.float32, device=self.device)
        p = torch.empty((n,), dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().ct_vfactor_embed(self._h, ctypes.c_void_p(xs.data_ptr()), n,
                                                    ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(p.data_ptr()),
                                                    _stream_ptr(stream)))
        return v, p

    def embed(self, x):
        v, p = self.embed_device(x)
        return v.cpu().numpy(), p.cpu().numpy()

    def device_bytes(self) -> int:
        return 8 * (self.m * self.d + 2 * self.m * self.m)

    def chol(self) -> np.ndarray:
        torch = _torch()
        out = torch.empty((self.m, self.m), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().ct_vfactor_chol(self._h, ctypes.c_void_p(out.data_ptr()), _stream_ptr(None)))
        return out.cpu().numpy()

    def free(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().ct_vfactor_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def build_vmatrix_cuda(points: np.ndarray, inducing_idx: np.ndarray, *, kernel_type: int, variance: float,
                       lengthscale: float):
    """V [N, m] f32, p [N] f32 and L [m, m] FP64 of build_residual_backend, on the GPU."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(-1, 1)
    f = CudaVFactor(pts[np.asarray(inducing_idx, dtype=np.int64)], kernel_type=kernel_type, variance=variance,
                    lengthscale=lengthscale)
    try:
        V, p = f.embed(pts)
        L = f.chol()
    finally:
        f.free()
    return V, p, L


_ORDER_MODES = {"natural": _lib.CT_ORDER_NATURAL, "hilbert": _lib.CT_ORDER_HILBERT, "morton": _lib.CT_ORDER_MORTON}


def batch_order(coords, mode: str = "hilbert", device=None) -> np.ndarray:
    """Stable batch order of points on the GPU (``ct_batch_order``).

    ``mode="hilbert"``: the Python PCCT path's Hilbert permutation
    (covertreex/algo/order/strategy.py:38-100); ``mode="morton"``: the Rust crate's
    ``hilbert_order`` (src/lib.rs:954-962, src/pcct.rs:27-67; identity unless D = 3)."""
    torch = _torch()
    if mode not in _ORDER_MODES:
        raise ValueError(f"unknown order mode {mode!r}")
    dev = torch.device(device if device is not None else "cuda")
    c = _as_device(coords, torch.float32, dev)
    if c.dim() == 1:
        c = c.reshape(-1, 1)
    n, d = int(c.shape[0]), int(c.shape[1])
    out = torch.empty(n, dtype=torch.int64, device=dev)
    _lib.check(_lib.load().ct_batch_order(c.data_ptr(), n, d, _ORDER_MODES[mode], out.data_ptr(), _stream_ptr(None)))
    return out.cpu().numpy()


def luby_mis(indptr, indices, seed: int, device=None):
    """Maximal independent set of a CSR conflict graph on the GPU (``ct_luby_mis``), with
    run_mis_numba's semantics (covertreex/algo/_mis_numba.py:64-140).  Returns
    (int8 indicator, iterations)."""
    torch = _torch()
    dev = torch.device(device if device is not None else "cuda")
    ip = _as_device(np.asarray(indptr, dtype=np.int64), torch.int64, dev)
    ix = _as_device(np.asarray(indices, dtype=np.int64).reshape(-1), torch.int64, dev)
    n = int(ip.numel()) - 1
    if n < 0:
        raise ValueError("indptr must hold n + 1 entries")
    sel = torch.zeros(max(n, 1), dtype=torch.int8, device=dev)
    it = ctypes.c_int32(0)
    _lib.check(_lib.load().ct_luby_mis(ip.data_ptr(), ix.data_ptr() if ix.numel() else None, n,
                                       int(seed) & 0xFFFFFFFFFFFFFFFF, sel.data_ptr(), ctypes.byref(it),
                                       _stream_ptr(None)))
    return sel[:n].cpu().numpy(), int(it.value)
