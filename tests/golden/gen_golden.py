"""Generate golden vectors by running the covertreex reference's own Python code.

Run in a container where the reference source tree is available:

    python tests/golden/gen_golden.py /path/to/covertreex

The reference package imports numba at module import; numba is not installed
here, so a stand-in module is registered whose ``njit``/``jit`` decorators
return the Python function unchanged (the reference's jitted functions then run
as plain Python).  One adaptation follows numba's integer semantics:
``np.uint32(x)`` of an out-of-range Python int wraps modulo 2**32 under numba
(NumPy 2 raises), so the MIS module sees a numpy namespace whose ``uint32``
masks its argument first.  Nothing else in the reference is altered.

Outputs (small .npz files next to this script):
  residual_backend.npz  build_residual_backend (host_backend.py:165-246): V, p, inducing ids
  mis.npz               _run_mis_numba_impl (_mis_numba.py:64-131) on seeded CSR graphs
  hilbert.npz           _hilbert_permutation (order/strategy.py:38-100) permutations
  prefix.npz            prefix_slices (order/helpers.py:59-71)
  distance.npz          compute_distance_chunk (metrics/_residual_numba.py:148-221) distances
  residual_knn.npz      _single_query_residual_knn (queries/residual_knn.py:249-386), the
                        reference's Python residual kNN, on a flat tree (every point a root,
                        so the best-first search visits every point): neighbour ids and
                        distances for 4 small cases, with and without predecessor mode
"""
from __future__ import annotations

import contextlib
import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


class _NumbaStub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Passthrough()


class _Passthrough:
    def __call__(self, *a, **k):
        if a and callable(a[0]) and len(a) == 1 and not k:
            return a[0]
        return lambda f: f

    def __getattr__(self, name):
        return _Passthrough()

    def __getitem__(self, k):
        return self

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def _install_numba_stub():
    nb = _NumbaStub("numba")

    def njit(*a, **k):
        if a and callable(a[0]) and len(a) == 1 and not k:
            return a[0]
        return lambda f: f

    nb.njit = njit
    nb.jit = njit
    nb.prange = range
    nb.objmode = lambda *a, **k: contextlib.nullcontext()
    nb.get_num_threads = lambda: 1
    nb.set_num_threads = lambda n: None
    sys.modules["numba"] = nb
    for sub in ("numba.typed", "numba.core", "numba.types", "numba.np", "numba.core.errors"):
        sys.modules[sub] = _NumbaStub(sub)


class _WrapNumpy(types.ModuleType):
    """numpy namespace whose uint32() wraps like a numba integer cast."""

    def __init__(self):
        super().__init__("numpy_wrapped")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def uint32(x):
        return np.uint32(int(x) & 0xFFFFFFFF)


def random_csr(n, p_edge, seed):
    r = np.random.default_rng(seed)
    A = r.random((n, n)) < p_edge
    A = np.triu(A, 1)
    A = A | A.T
    indptr = np.zeros(n + 1, np.int64)
    indices = []
    for v in range(n):
        nb = np.nonzero(A[v])[0]
        indices.extend(nb.tolist())
        indptr[v + 1] = len(indices)
    return indptr, np.asarray(indices, np.int64)


def main(ref_root: str) -> None:
    _install_numba_stub()
    sys.path.insert(0, ref_root)
    from covertreex.algo import _mis_numba as mis_mod
    from covertreex.algo.order import helpers as order_helpers
    from covertreex.algo.order import strategy as order_strategy
    from covertreex.metrics import _residual_numba as resn
    from covertreex.metrics.residual.host_backend import build_residual_backend

    # ---- build_residual_backend
    cases = []
    for (n, d, m, kt, ls, seed) in [(300, 3, 32, 1, 1.0, 0), (257, 2, 40, 0, 0.7, 3), (200, 5, 64, 0, 2.0, 9),
                                    (120, 3, 200, 1, 1.5, 1)]:
        X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
        hb = build_residual_backend(X, seed=42, inducing_count=m, variance=1.0, lengthscale=ls, kernel_type=kt)
        cases.append((X, hb.v_matrix, hb.p_diag, kt, ls, m))
    np.savez_compressed(
        OUT / "residual_backend.npz",
        **{f"X{i}": c[0] for i, c in enumerate(cases)},
        **{f"V{i}": c[1] for i, c in enumerate(cases)},
        **{f"p{i}": c[2] for i, c in enumerate(cases)},
        meta=np.array([[c[3], c[4], c[5]] for c in cases], dtype=np.float64),
    )

    # ---- Luby MIS (numba function run as Python, uint32 casts wrapped)
    mis_mod.np = _WrapNumpy()
    graphs = {}
    for gi, (n, pe, seed, mseed) in enumerate([(40, 0.05, 1, 7), (60, 0.3, 2, 11), (80, 0.15, 3, 0), (33, 0.5, 4, 99)]):
        indptr, indices = random_csr(n, pe, seed)
        sel, iters = mis_mod._run_mis_numba_impl(indptr, indices, n, mseed)
        graphs[f"indptr{gi}"] = indptr
        graphs[f"indices{gi}"] = indices
        graphs[f"seed{gi}"] = np.array(mseed)
        graphs[f"sel{gi}"] = np.asarray(sel, np.int8)
        graphs[f"iters{gi}"] = np.array(iters)
    np.savez_compressed(OUT / "mis.npz", **graphs)

    # ---- Hilbert permutation
    hil = {}
    for hi_, (n, d, seed) in enumerate([(500, 2, 0), (400, 3, 1), (300, 5, 2), (256, 8, 3)]):
        P = np.random.default_rng(seed).standard_normal((n, d))
        perm, _ = order_strategy._hilbert_permutation(P, seed=None)
        hil[f"P{hi_}"] = P
        hil[f"perm{hi_}"] = np.asarray(perm, np.int64)
    np.savez_compressed(OUT / "hilbert.npz", **hil)

    # ---- prefix slices
    lens = [1, 2, 3, 7, 8, 100, 512, 1000, 4097]
    pre = {f"len{i}": np.array(L) for i, L in enumerate(lens)}
    pre.update({f"slices{i}": np.asarray(order_helpers.prefix_slices(L), np.int64) for i, L in enumerate(lens)})
    np.savez_compressed(OUT / "prefix.npz", **pre)

    # ---- residual distance (f64 formula given kernel values)
    r = np.random.default_rng(5)
    X = r.standard_normal((150, 3)).astype(np.float32)
    hb = build_residual_backend(X, seed=42, inducing_count=48, variance=1.0, lengthscale=1.0, kernel_type=0)
    V = hb.v_matrix.astype(np.float64)
    p = hb.p_diag.astype(np.float64)
    dist = np.zeros((20, 150))
    kern = hb.kernel_provider(np.arange(20), np.arange(150)).astype(np.float64)
    norms = np.sum(V * V, axis=1)
    for q in range(20):
        dq, _ = resn.compute_distance_chunk(V[q], V, kern[q], float(p[q]), p, float(norms[q]), norms, 1.0, 1e-9)
        dist[q] = dq
    np.savez_compressed(OUT / "distance.npz", X=X, V=hb.v_matrix, p=hb.p_diag, dist=dist)

    # ---- the reference's own residual kNN search (Python path), exhaustive on a flat tree
    from covertreex.queries import residual_knn as rknn
    from covertreex.queries.utils import ChildChainCache

    knn = {}
    for ci, (n, d, m, kt, ls, k, pred, seed) in enumerate([(400, 3, 32, 0, 1.0, 10, False, 31),
                                                          (500, 2, 48, 1, 0.8, 16, True, 32),
                                                          (300, 5, 64, 0, 2.0, 8, True, 33),
                                                          (350, 3, 40, 1, 1.3, 12, False, 34)]):
        X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
        hb = build_residual_backend(X, seed=42, inducing_count=m, variance=1.0, lengthscale=ls, kernel_type=kt)
        flat_children = np.full(n, -1, np.int64)
        cache = ChildChainCache(flat_children, np.full(n, -1, np.int64))
        rows_i = np.full((n, k), -1, np.int64)
        rows_d = np.full((n, k), np.inf)
        for q in range(n):
            kk = min(k, q) if pred else k
            if kk <= 0:
                continue
            ids, dists = rknn._single_query_residual_knn(
                q, tree_indices=np.arange(n, dtype=np.int64), si_cache=np.zeros(n), child_cache=cache,
                root_indices=np.arange(n, dtype=np.int64), k=kk, host_backend=hb, predecessor_mode=pred)
            rows_i[q, :len(ids)] = ids
            rows_d[q, :len(ids)] = dists
        knn[f"X{ci}"] = X
        knn[f"V{ci}"] = hb.v_matrix
        knn[f"p{ci}"] = hb.p_diag
        knn[f"idx{ci}"] = rows_i
        knn[f"dist{ci}"] = rows_d
        knn[f"meta{ci}"] = np.array([kt, ls, k, int(pred)], dtype=np.float64)
    np.savez_compressed(OUT / "residual_knn.npz", **knn)
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/gen_golden.py <path to the covertreex source tree>")
    main(sys.argv[1])
