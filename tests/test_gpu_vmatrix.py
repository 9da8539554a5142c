"""FP64 residual-backend construction on the GPU (ct_vfactor_*) against the oracle's
numpy restatement of build_residual_backend (covertreex/metrics/residual/host_backend.py:165-246),
itself pinned to the reference by tests/golden/residual_backend.npz.

Tolerances.  Both sides compute V in FP64 and round to f32; they differ by the FP64
forward error of the triangular solve, at most c * m * cond(L) * 2^-53 per unit of
|v| <= sqrt(var) (c = 8 here), plus one f32 rounding step (2^-23 relative) where the
two FP64 values straddle an f32 rounding boundary:
    |dV| <= 2^-23 |V| + e64,          e64 = 8 m cond(L) 2^-53 sqrt(var)
    |dp| <= 2^-23 p + 2 sqrt(m var) e64
    |dL| <= 8 m cond(L)^2 2^-53 sqrt(var)     (Cholesky forward error)
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tols(L, m, var):
    cond = float(np.linalg.cond(L))
    e64 = 8.0 * m * cond * 2.0 ** -53 * np.sqrt(var)
    return cond, e64


def _check(X, m, kt, ls, var=1.0, seed=42):
    from covertreex_gb300.device import build_vmatrix_cuda
    from covertreex_gb300.residual import inducing_indices

    Vr, pr, idx, Lr = O.build_residual_backend_np(X, seed=seed, inducing_count=m, variance=var, lengthscale=ls,
                                                  kernel_type=kt)
    assert np.array_equal(idx, inducing_indices(X.shape[0], m, seed))
    V, p, L = build_vmatrix_cuda(X.astype(np.float64), idx, kernel_type=kt, variance=var, lengthscale=ls)
    mm = idx.size
    cond, e64 = _tols(Lr, mm, var)
    assert V.shape == Vr.shape and p.shape == pr.shape and L.shape == (mm, mm)
    assert np.all(np.triu(L, 1) == 0.0)
    dL = np.abs(L - Lr).max()
    assert dL <= 8.0 * mm * cond * cond * 2.0 ** -53 * np.sqrt(var), (dL, cond)
    dV = np.abs(V.astype(np.float64) - Vr.astype(np.float64))
    assert np.all(dV <= 2.0 ** -23 * np.abs(Vr) + e64), (dV.max(), e64, cond)
    dp = np.abs(p.astype(np.float64) - pr.astype(np.float64))
    assert np.all(dp <= 2.0 ** -23 * pr + 2.0 * np.sqrt(mm * var) * e64), (dp.max(), cond)
    if e64 < 2.0 ** -34:
        # FP64 error far below f32 resolution: most entries round to the same f32 value
        assert np.mean(V == Vr) > 0.9
    return V, p


@pytest.mark.parametrize("n,d,m,kt,ls", [
    (4096, 3, 64, 1, 1.0),      # Matern 5/2, plain_small-like
    (3001, 8, 100, 0, 2.0),     # m off the 32-column panel, n off the 64-row tile
    (20000, 8, 512, 0, 2.0),    # precision-like rank
    (200, 2, 200, 1, 0.7),      # inducing set = all points (p at the jitter floor)
    (50, 3, 1, 0, 1.0),         # rank one
])
def test_vmatrix_matches_host_backend(cuda_available, n, d, m, kt, ls):
    X = np.random.default_rng(n + m).standard_normal((n, d)).astype(np.float32)
    _check(X, m, kt, ls)


def test_vmatrix_variance_scaled(cuda_available):
    X = np.random.default_rng(5).uniform(-3, 3, (2048, 4)).astype(np.float32)
    _check(X, 128, 0, 1.5, var=2.5)


def test_embed_new_points(cuda_available):
    """Serving: v_x = L^-1 k(Z, x) for points outside the dataset."""
    from covertreex_gb300.device import CudaVFactor

    X = np.random.default_rng(11).standard_normal((5000, 3)).astype(np.float64)
    _, _, idx, Lr = O.build_residual_backend_np(X, seed=7, inducing_count=96, variance=1.0, lengthscale=1.0,
                                                kernel_type=1)
    Z = X[idx]
    Xn = np.random.default_rng(12).standard_normal((777, 3))
    kz = O.kernel_f64(Xn, Z, 1, 1.0, 1.0)
    vr = np.linalg.solve(Lr, kz.T).T
    pr = np.maximum(1.0 - np.sum(vr * vr, axis=1), 1e-9)
    f = CudaVFactor(Z, kernel_type=1, variance=1.0, lengthscale=1.0)
    try:
        v, p = f.embed(Xn)
        v2, p2 = f.embed(Xn[:5])  # a second, smaller call reuses the scratch
    finally:
        f.free()
    cond, e64 = _tols(Lr, 96, 1.0)
    assert np.all(np.abs(v - vr) <= 2.0 ** -23 * np.abs(vr) + e64 + 2.0 ** -24 * np.abs(vr))
    assert np.all(np.abs(p - pr) <= 2.0 ** -23 * pr + 2.0 * np.sqrt(96) * e64 + 2.0 ** -24 * pr)
    assert np.array_equal(v2, v[:5]) and np.array_equal(p2, p[:5])


def test_not_positive_definite_is_an_error(cuda_available):
    import torch

    from covertreex_gb300 import _lib

    L = _lib.load()
    z = torch.randn(16, 2, dtype=torch.float64, device="cuda")
    h = ctypes.c_void_p()
    rc = L.ct_vfactor_create(ctypes.c_void_p(z.data_ptr()), 16, 2, 0, -1.0, 1.0, None, ctypes.byref(h))
    assert rc == _lib.CT_ERR_ARG and not h.value
    assert b"positive definite" in L.ct_last_error()


def test_cover_tree_with_device_vmatrix(cuda_available):
    from covertreex_gb300 import Matern52, cover_tree

    X = np.random.default_rng(3).standard_normal((3000, 3)).astype(np.float32)
    t_gpu = cover_tree(X, kernel=Matern52(lengthscale=1.0), inducing_count=64, seed=42, vmatrix_device="cuda")
    V, p = _check(X, 64, 1, 1.0)
    idx_gpu = t_gpu.knn(10, queries=np.arange(0, 3000, 7), predecessor_mode=True, form="dense")
    ref = O.brute_knn_f32(V, p, X, 1.0, np.ones(3, np.float32), 1, np.arange(0, 3000, 7), 10, predecessor=True)
    assert np.array_equal(np.asarray(idx_gpu), ref[0])


def test_concurrent_embeds_on_one_factor(cuda_available):
    """Two threads embed through one factor on their own streams, with batch sizes
    that differ call to call: the factor is read-only, each call's scratch is its
    own, and every result equals the single-threaded one."""
    import threading

    import torch

    from covertreex_gb300.device import CudaVFactor

    X = np.random.default_rng(21).standard_normal((4000, 3))
    f = CudaVFactor(X[:256], kernel_type=1, variance=1.0, lengthscale=1.0)
    sizes = [1, 37, 4096, 700, 9000, 5]
    pts = [np.random.default_rng(100 + i).standard_normal((q, 3)) for i, q in enumerate(sizes)]
    ref = [f.embed(p) for p in pts]
    errors = []

    def work(order):
        st = torch.cuda.Stream()
        try:
            for _ in range(3):
                for i in order:
                    with torch.cuda.stream(st):
                        v, p = f.embed_device(pts[i], stream=st)
                        v, p = v.cpu().numpy(), p.cpu().numpy()
                    if not (np.array_equal(v, ref[i][0]) and np.array_equal(p, ref[i][1])):
                        errors.append(i)
        except Exception as exc:  # surfaced below
            errors.append(repr(exc))

    ts = [threading.Thread(target=work, args=(o,)) for o in ([0, 2, 4, 1, 3, 5], [5, 3, 1, 4, 2, 0])]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    f.free()
    assert not errors, errors
