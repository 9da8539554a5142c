"""CPU oracle for the residual-correlation cover tree — TEST INFRASTRUCTURE ONLY.

This module is the parity checker used by ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The
product package (``covertreex_gb300``) never imports it.

Contents:
  * ctypes bindings for ``ct_oracle.c`` — a C restatement of the reference's
    Rust crate ``covertreex_backend`` (``src/metric.rs``, ``src/algo.rs``,
    ``src/algo/batch/{mod,mis}.rs``, ``src/pcct.rs``, ``src/tree.rs``,
    ``src/lib.rs``), plus the Python-side Luby MIS / Hilbert keys;
  * ``build_residual_backend_np`` — numpy restatement of
    ``covertreex/metrics/residual/host_backend.py:165-246``;
  * ``brute_knn_f64`` — the FP64 brute-force ground truth (ties -> lower index),
    with ``near_ties`` listing pairs whose FP64 distances differ by < 1e-6.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libct_oracle.so"
_lib = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i8p = ctypes.POINTER(ctypes.c_int8)


def build_oracle() -> Path:
    """Compile ct_oracle.c (gcc, OpenMP) into oracle/_build/."""
    subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < (_HERE / "ct_oracle.c").stat().st_mtime:
        build_oracle()
    L = ctypes.CDLL(str(_LIB_PATH))
    L.ct_expf.restype = ctypes.c_float
    L.ct_expf.argtypes = [ctypes.c_float]
    L.ct_dot_simd_inline.restype = ctypes.c_float
    L.ct_dot_simd_inline.argtypes = [_f32p, _f32p, ctypes.c_int]
    L.ct_dot_simd_slice.restype = ctypes.c_float
    L.ct_dot_simd_slice.argtypes = [_f32p, _f32p, ctypes.c_int]
    L.ct_morton3.restype = ctypes.c_uint64
    L.ct_morton3.argtypes = [ctypes.c_uint32] * 3
    L.ct_morton_order.restype = None
    L.ct_morton_order.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, _i64p, _u64p]
    L.ct_subtree_bounds.restype = None
    L.ct_subtree_bounds.argtypes = [_i64p, _i64p, ctypes.c_int64, _i64p, _i64p]
    L.ct_oracle_build_residual.restype = ctypes.c_void_p
    L.ct_oracle_build_residual.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_float, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                           ctypes.c_int, ctypes.c_float, ctypes.c_int]
    L.ct_oracle_free.restype = None
    L.ct_oracle_free.argtypes = [ctypes.c_void_p]
    L.ct_oracle_tree_arrays.restype = None
    L.ct_oracle_tree_arrays.argtypes = [ctypes.c_void_p, _i64p, _i64p, _i64p, _i32p, _f32p, _i64p]
    L.ct_oracle_knn_residual.restype = ctypes.c_int64
    L.ct_oracle_knn_residual.argtypes = [ctypes.c_void_p, _i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                         _i64p, ctypes.c_int, _i64p, _f32p, ctypes.c_int]
    L.ct_oracle_brute_f32.restype = None
    L.ct_oracle_brute_f32.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_float, _f32p, ctypes.c_int, ctypes.c_int,
                                      _i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _i64p, _f32p, ctypes.c_int]
    L.ct_oracle_brute_points_f32.restype = None
    L.ct_oracle_brute_points_f32.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_float, _f32p, ctypes.c_int, ctypes.c_int,
                                             _f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, _i64p, _f32p,
                                             ctypes.c_int]
    L.ct_oracle_pair_dist.restype = None
    L.ct_oracle_pair_dist.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_float, _f32p, ctypes.c_int, ctypes.c_int,
                                      _i64p, _i64p, ctypes.c_int64, _f32p, ctypes.c_int]
    L.ct_oracle_build_euclidean.restype = ctypes.c_void_p
    L.ct_oracle_build_euclidean.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int64]
    L.ct_oracle_free_euclidean.restype = None
    L.ct_oracle_free_euclidean.argtypes = [ctypes.c_void_p]
    L.ct_oracle_euclidean_arrays.restype = None
    L.ct_oracle_euclidean_arrays.argtypes = [ctypes.c_void_p, _i64p, _i32p]
    L.ct_oracle_knn_euclidean.restype = None
    L.ct_oracle_knn_euclidean.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                          _i64p, _f32p]
    L.ct_hash_priority.restype = ctypes.c_double
    L.ct_hash_priority.argtypes = [ctypes.c_int64] * 3
    L.ct_oracle_luby_mis.restype = ctypes.c_int
    L.ct_oracle_luby_mis.argtypes = [_i64p, _i64p, ctypes.c_int64, ctypes.c_int64, _i8p]
    L.ct_hilbert_codes.restype = None
    L.ct_hilbert_codes.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int, _u64p]
    L.ct_oracle_brute_f64.restype = None
    L.ct_oracle_brute_f64.argtypes = [_f32p, _f32p, _f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, _f32p, ctypes.c_int, ctypes.c_int, _i64p, ctypes.c_int64,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int64, _i64p, _f64p, ctypes.c_int]
    _lib = L
    return L


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# --------------------------------------------------------------------------
# numpy restatement of build_residual_backend (host_backend.py:165-246)
# --------------------------------------------------------------------------
def kernel_f64(x: np.ndarray, y: np.ndarray, kernel_type: int, variance: float, lengthscale: float) -> np.ndarray:
    """RBF / Matern 5/2 in FP64 (host_backend.py:14-43), pairwise by differences."""
    diff = x[:, None, :] - y[None, :, :]
    sq = np.sum(diff * diff, axis=2, dtype=np.float64)
    denom = max(float(lengthscale), 1e-12)
    if kernel_type == 1:
        r = np.sqrt(sq) / denom
        a = np.sqrt(5.0) * r
        return float(variance) * (1.0 + a + (a * a) / 3.0) * np.exp(-a)
    return float(variance) * np.exp(-0.5 * sq / (denom * denom))


def build_residual_backend_np(points, *, seed: int, inducing_count: int, variance: float,
                              lengthscale: float, kernel_type: int = 0, block: int = 4096):
    """Returns (V f32 [N,m], p f32 [N], inducing_idx, L f64 [m,m])."""
    pts = np.asarray(points, dtype=np.float64)
    n = pts.shape[0]
    m = min(inducing_count, n)
    if m <= 0:
        m = min(32, n)
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, size=m, replace=False)) if m < n else np.arange(n)
    Z = pts[idx]
    kmm = kernel_f64(Z, Z, kernel_type, variance, lengthscale) + np.eye(m) * (1e-6 * variance)
    L = np.linalg.cholesky(kmm)
    V = np.empty((n, m), dtype=np.float64)
    for s in range(0, n, block):
        kxm = kernel_f64(pts[s:s + block], Z, kernel_type, variance, lengthscale)
        V[s:s + block] = np.linalg.solve(L, kxm.T).T
    p = np.maximum(variance - np.sum(V * V, axis=1), 1e-9)
    return V.astype(np.float32), p.astype(np.float32), idx, L


# --------------------------------------------------------------------------
# FP64 brute force (ground truth)
# --------------------------------------------------------------------------
def residual_dist_f64(V, p, coords, var, ls, kernel_type, qi, cj):
    """FP64 residual distance sqrt(1-|rho|) over the stored f32 inputs, for rows qi x cols cj."""
    qi = np.asarray(qi, dtype=np.int64).reshape(-1)
    cj = np.asarray(cj, dtype=np.int64).reshape(-1)
    inv_ls = 1.0 / np.broadcast_to(np.asarray(ls, dtype=np.float64).reshape(-1), (coords.shape[1],))
    xq = np.asarray(coords[qi], dtype=np.float64) * inv_ls
    xc = np.asarray(coords[cj], dtype=np.float64) * inv_ls
    # squared distance one axis at a time (no q x c x D temporary at large N)
    d2 = np.zeros((qi.size, cj.size))
    for a in range(xq.shape[1]):
        t = xq[:, a][:, None] - xc[:, a][None, :]
        t *= t
        d2 += t
    if kernel_type == 1:
        a_ = np.sqrt(d2)
        a_ *= np.sqrt(5.0)
        K = var * (1.0 + a_ + a_ * a_ / 3.0) * np.exp(-a_)
    else:
        d2 *= -0.5
        K = var * np.exp(d2)
    K -= np.asarray(V[qi], dtype=np.float64) @ np.asarray(V[cj], dtype=np.float64).T
    pq = np.asarray(p[qi], dtype=np.float64)
    pc = np.asarray(p[cj], dtype=np.float64)
    K /= np.sqrt(np.maximum(pq[:, None] * pc[None, :], 1e-18))
    np.clip(K, -1.0, 1.0, out=K)
    np.abs(K, out=K)
    d = np.sqrt(np.maximum(1.0 - K, 0.0))
    d[qi[:, None] == cj[None, :]] = 0.0
    return d


def brute_knn_f64(V, p, coords, var, ls, kernel_type, queries, k, predecessor, block=256, cand_limit=None):
    """Exact kNN in FP64, ascending by (dist, idx); -1 / +inf padding.  Returns (idx, dist).
    cand_limit: candidates are rows [0, cand_limit) (rows beyond hold new query points)."""
    n = V.shape[0] if cand_limit is None else int(cand_limit)
    queries = np.asarray(queries, dtype=np.int64)
    out_i = np.full((queries.size, k), -1, dtype=np.int64)
    out_d = np.full((queries.size, k), np.inf, dtype=np.float64)
    # blocks of queries close in id, so that predecessor mode only scores [0, max id)
    order_q = np.argsort(queries, kind="stable")
    for s in range(0, queries.size, block):
        rows = order_q[s:s + block]
        qb = queries[rows]
        hi = n if not predecessor else int(min(n, max(int(qb.max()), 0)))
        if hi <= 0:
            continue
        allc = np.arange(hi)
        D = residual_dist_f64(V, p, coords, var, ls, kernel_type, qb, allc)
        if predecessor:
            D[allc[None, :] >= qb[:, None]] = np.inf
        kk = min(k, hi)
        part = np.argpartition(D, kk - 1, axis=1)[:, :kk] if kk < hi else np.tile(allc, (qb.size, 1))
        for r in range(qb.size):
            cand = part[r]
            # widen to include exact ties at the boundary, then lexsort (dist, idx)
            thr = D[r, cand].max()
            cand = np.nonzero(D[r] <= thr)[0]
            order = np.lexsort((cand, D[r, cand]))
            sel = cand[order][:k]
            sel = sel[np.isfinite(D[r, sel])]
            out_i[rows[r], :sel.size] = sel
            out_d[rows[r], :sel.size] = D[r, sel]
    return out_i, out_d


def brute_knn_f64_c(V, p, coords, var, ls, kernel_type, queries, k, predecessor, cand_limit=None, threads=0):
    """The FP64 brute force of ``brute_knn_f64`` in C (OpenMP, query blocks sharing each
    candidate row), for the full-size shapes; same formula, ordering and padding."""
    L = lib()
    V = _c(V, np.float32); p = _c(p, np.float32).reshape(-1); coords = _c(coords, np.float32)
    ls = _c(np.atleast_1d(ls), np.float32)
    q = _c(queries, np.int64).reshape(-1)
    oi = np.empty((q.size, k), np.int64)
    od = np.empty((q.size, k), np.float64)
    L.ct_oracle_brute_f64(_p(V, _f32p), _p(p, _f32p), _p(coords, _f32p), V.shape[0], V.shape[1], coords.shape[1],
                          float(var), _p(ls, _f32p), ls.size, int(kernel_type), _p(q, _i64p), q.size, int(k),
                          int(predecessor), int(cand_limit or 0), _p(oi, _i64p), _p(od, _f64p), int(threads))
    return oi, od


# --------------------------------------------------------------------------
# C restatement wrappers
# --------------------------------------------------------------------------
class OracleResidualTree:
    """build_pcct2_residual_tree + knn_query_residual (src/lib.rs:370-507, 1374-1564)."""

    def __init__(self, V, p, coords, var, ls, kernel_type=0, chunk=512, order="hilbert",
                 grid_scale=1.0, parity=True):
        L = lib()
        self.V = _c(V, np.float32)
        self.p = _c(p, np.float32)
        self.coords = _c(coords, np.float32)
        self.ls = _c(np.atleast_1d(ls), np.float32)
        self.n, self.m = self.V.shape
        self.d = self.coords.shape[1]
        self.parity = bool(parity)
        order_mode = 0 if order == "natural" else 1
        self._h = L.ct_oracle_build_residual(
            _p(self.V, _f32p), _p(self.p, _f32p), _p(self.coords, _f32p), self.n, self.m, self.d,
            float(var), _p(self.ls, _f32p), self.ls.size, int(kernel_type), int(chunk), order_mode,
            float(grid_scale), int(parity))
        n = self.n
        self.parents = np.empty(n, np.int64)
        self.children = np.empty(n, np.int64)
        self.next = np.empty(n, np.int64)
        self.levels = np.empty(n, np.int32)
        self.si = np.empty(n, np.float32)
        self.order = np.empty(n, np.int64)
        L.ct_oracle_tree_arrays(self._h, _p(self.parents, _i64p), _p(self.children, _i64p),
                                _p(self.next, _i64p), _p(self.levels, _i32p), _p(self.si, _f32p),
                                _p(self.order, _i64p))
        self.subtree_min, self.subtree_max = subtree_bounds(self.parents, self.order)

    def knn(self, queries, k, predecessor=False, parity=None, threads=0):
        L = lib()
        q = _c(queries, np.int64).reshape(-1)
        oi = np.empty((q.size, k), np.int64)
        od = np.empty((q.size, k), np.float32)
        par = self.parity if parity is None else bool(parity)
        evals = L.ct_oracle_knn_residual(self._h, _p(q, _i64p), q.size, int(k), int(predecessor),
                                         _p(self.subtree_min, _i64p), int(par), _p(oi, _i64p), _p(od, _f32p),
                                         int(threads))
        # the reference's `distance_evals` (src/algo.rs:1087-1092) counts the batch-path
        # child evaluations only; every query also scores every root (algo.rs:688-734)
        self.last_evals = int(evals)
        self.last_root_evals = int(q.size) * int(np.count_nonzero(self.parents == -1))
        return oi, od

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().ct_oracle_free(self._h)
                self._h = None
        except Exception:
            pass


def subtree_bounds(parents, node_to_dataset):
    L = lib()
    par = _c(parents, np.int64)
    n2d = _c(node_to_dataset, np.int64)
    mn = np.empty_like(n2d)
    mx = np.empty_like(n2d)
    L.ct_subtree_bounds(_p(par, _i64p), _p(n2d, _i64p), par.size, _p(mn, _i64p), _p(mx, _i64p))
    return mn, mx


def brute_knn_f32(V, p, coords, var, ls, kernel_type, queries, k, predecessor, threads=0):
    """Exact kNN over the reference's batch-path f32 distance (ties -> lower index)."""
    L = lib()
    V = _c(V, np.float32); p = _c(p, np.float32); coords = _c(coords, np.float32)
    ls = _c(np.atleast_1d(ls), np.float32)
    q = _c(queries, np.int64).reshape(-1)
    oi = np.empty((q.size, k), np.int64)
    od = np.empty((q.size, k), np.float32)
    L.ct_oracle_brute_f32(_p(V, _f32p), _p(p, _f32p), _p(coords, _f32p), V.shape[0], V.shape[1], coords.shape[1],
                          float(var), _p(ls, _f32p), ls.size, int(kernel_type), _p(q, _i64p), q.size, int(k),
                          int(predecessor), _p(oi, _i64p), _p(od, _f32p), int(threads))
    return oi, od


def brute_knn_points_f32(V, p, coords, var, ls, kernel_type, qv, qp, qcoords, k, threads=0):
    """Exact kNN of new points (rows qv/qp/qcoords) over the batch-path f32 distance,
    each point handled like one more dataset row; candidates = the dataset."""
    L = lib()
    V = _c(V, np.float32); p = _c(p, np.float32); coords = _c(coords, np.float32)
    qv = _c(qv, np.float32); qp = _c(qp, np.float32).reshape(-1); qcoords = _c(qcoords, np.float32)
    ls = _c(np.atleast_1d(ls), np.float32)
    nq = qp.size
    oi = np.empty((nq, k), np.int64)
    od = np.empty((nq, k), np.float32)
    L.ct_oracle_brute_points_f32(_p(V, _f32p), _p(p, _f32p), _p(coords, _f32p), V.shape[0], V.shape[1],
                                 coords.shape[1], float(var), _p(ls, _f32p), ls.size, int(kernel_type),
                                 _p(qv, _f32p), _p(qp, _f32p), _p(qcoords, _f32p), nq, int(k), _p(oi, _i64p),
                                 _p(od, _f32p), int(threads))
    return oi, od


def pair_dist_f32(V, p, coords, var, ls, kernel_type, qi, cj, scalar_path=False):
    L = lib()
    V = _c(V, np.float32); p = _c(p, np.float32); coords = _c(coords, np.float32)
    ls = _c(np.atleast_1d(ls), np.float32)
    qi = _c(qi, np.int64).reshape(-1); cj = _c(cj, np.int64).reshape(-1)
    out = np.empty(qi.size, np.float32)
    L.ct_oracle_pair_dist(_p(V, _f32p), _p(p, _f32p), _p(coords, _f32p), V.shape[0], V.shape[1], coords.shape[1],
                          float(var), _p(ls, _f32p), ls.size, int(kernel_type), _p(qi, _i64p), _p(cj, _i64p),
                          qi.size, _p(out, _f32p), int(scalar_path))
    return out


def morton_order(coords):
    L = lib()
    c = _c(coords, np.float32)
    n, d = c.shape
    order = np.empty(n, np.int64)
    codes = np.empty(n, np.uint64)
    L.ct_morton_order(_p(c, _f32p), n, d, _p(order, _i64p), _p(codes, _u64p))
    return order, codes


def hilbert_codes(points):
    L = lib()
    pts = _c(points, np.float64)
    n, d = pts.shape
    codes = np.empty(n, np.uint64)
    L.ct_hilbert_codes(_p(pts, _f64p), n, d, _p(codes, _u64p))
    return codes


def hilbert_order(points):
    codes = hilbert_codes(points)
    return np.lexsort((np.arange(codes.size), codes)).astype(np.int64), codes


def luby_mis(indptr, indices, seed):
    L = lib()
    ip = _c(indptr, np.int64); ix = _c(indices, np.int64)
    n = ip.size - 1
    sel = np.zeros(max(n, 1), np.int8)
    it = L.ct_oracle_luby_mis(_p(ip, _i64p), _p(ix, _i64p), n, int(seed), _p(sel, _i8p))
    return sel[:n], it


def prefix_slices(length: int):
    """covertreex/algo/order/helpers.py:59-71 restated."""
    out = []
    size, start = 1, 0
    while start < length:
        end = min(start + size, length)
        out.append((start, end))
        start = end
        remaining = length - start
        if remaining <= 0:
            break
        size = min(size * 2, remaining)
    return out


class OracleEuclideanTree:
    """CoverTreeWrapper.insert + knn_query (src/lib.rs:207-223, 299-326; src/algo.rs:179-323)."""

    def __init__(self, points, chunk=512):
        L = lib()
        self.pts = _c(points, np.float32)
        self.n, self.d = self.pts.shape
        self._h = L.ct_oracle_build_euclidean(_p(self.pts, _f32p), self.n, self.d, int(chunk))

    def knn(self, queries, k, predecessor=False):
        L = lib()
        q = _c(queries, np.float32)
        oi = np.empty((q.shape[0], k), np.int64)
        od = np.empty((q.shape[0], k), np.float32)
        L.ct_oracle_knn_euclidean(self._h, _p(q, _f32p), q.shape[0], int(k), int(predecessor),
                                  _p(oi, _i64p), _p(od, _f32p))
        return oi, od

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().ct_oracle_free_euclidean(self._h)
                self._h = None
        except Exception:
            pass


def brute_knn_euclidean_f64(points, queries, k, predecessor=False):
    P = np.asarray(points, np.float64)
    Qp = np.asarray(queries, np.float64)
    n = P.shape[0]
    out_i = np.full((Qp.shape[0], k), -1, np.int64)
    out_d = np.full((Qp.shape[0], k), np.inf)
    for s in range(0, Qp.shape[0], 512):
        qb = Qp[s:s + 512]
        D = np.zeros((qb.shape[0], n))
        for a in range(P.shape[1]):
            t = qb[:, a][:, None] - P[:, a][None, :]
            t *= t
            D += t
        np.sqrt(D, out=D)
        if predecessor:
            rows = np.arange(s, s + qb.shape[0])
            D[np.arange(n)[None, :] >= rows[:, None]] = np.inf
        kk = min(k, n)
        part = np.argpartition(D, kk - 1, axis=1)[:, :kk] if kk < n else np.tile(np.arange(n), (qb.shape[0], 1))
        for r in range(qb.shape[0]):
            # widen to the exact ties at the boundary, then order by (dist, idx)
            cand = np.nonzero(D[r] <= D[r, part[r]].max())[0]
            order = cand[np.lexsort((cand, D[r, cand]))][:k]
            order = order[np.isfinite(D[r, order])]
            out_i[s + r, :order.size] = order
            out_d[s + r, :order.size] = D[r, order]
    return out_i, out_d


def near_tie_mismatches(got_idx, ref_idx, dist_fn, tol=1e-6):
    """Compare neighbour sets row by row.

    Returns (n_rows_exact, mismatches) where mismatches lists (row, extra_got, extra_ref, gap)
    with gap = |d64(extra_got) - d64(extra_ref)| evaluated by ``dist_fn(row, ids)``.
    A row whose every swapped pair has gap < tol is a listed near-tie, not a failure.
    """
    exact = 0
    out = []
    for r in range(got_idx.shape[0]):
        g = set(int(x) for x in got_idx[r] if x >= 0)
        f = set(int(x) for x in ref_idx[r] if x >= 0)
        if g == f:
            exact += 1
            continue
        eg = sorted(g - f)
        ef = sorted(f - g)
        dg = dist_fn(r, np.array(eg, dtype=np.int64)) if eg else np.array([])
        df = dist_fn(r, np.array(ef, dtype=np.int64)) if ef else np.array([])
        if len(eg) != len(ef):
            out.append((r, eg, ef, float("inf")))
            continue
        gap = float(np.max(np.abs(np.sort(dg) - np.sort(df)))) if eg else 0.0
        out.append((r, eg, ef, gap))
    return exact, out
