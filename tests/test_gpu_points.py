"""kNN of NEW points against a resident tree (the serving queries): the dense form
bit-exact to the f32 oracle, the screened form against FP64 brute force (distance
error <= 1e-5, neighbour sets equal except listed near-ties with FP64 gap < 1e-6),
and each point's result identical alone and inside a larger call."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # n, d, m, kernel_type, lengthscale, k, nq
    (20000, 3, 256, 1, 1.0, 50, 300),
    (8192, 8, 128, 0, 2.0, 30, 257),
    (3000, 2, 64, 1, 0.7, 10, 5000),  # more points than the initial query slab: the slab grows
]


def _embed(Xq, X, idx, L, kt, ls):
    kz = O.kernel_f64(Xq.astype(np.float64), X[idx].astype(np.float64), kt, 1.0, ls)
    vq = np.linalg.solve(L, kz.T).T
    pq = np.maximum(1.0 - np.sum(vq * vq, axis=1), 1e-9)
    return vq.astype(np.float32), pq.astype(np.float32)


def _case(n, d, m, kt, ls, nq, seed):
    X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
    V, p, idx, L = O.build_residual_backend_np(X, seed=seed + 1, inducing_count=m, variance=1.0, lengthscale=ls,
                                               kernel_type=kt)
    Xq = np.random.default_rng(seed + 2).standard_normal((nq, d)).astype(np.float32)
    qv, qp = _embed(Xq, X, idx, L, kt, ls)
    return X, V, p, Xq, qv, qp


def _check_screened_vs_fp64(V, p, X, Xq, qv, qp, si, sd, kt, lsv, k, limit=400):
    n, nq = X.shape[0], Xq.shape[0]
    Va, pa, Xa = np.vstack([V, qv]), np.concatenate([p, qp]), np.vstack([X, Xq])
    rows = np.arange(n, n + nq)
    check = rows if nq <= limit else rows[:: nq // limit]
    sel = check - n
    ri, rd = O.brute_knn_f64(Va, pa, Xa, 1.0, lsv, kt, check, k, False, cand_limit=n)
    got_d64 = np.array([O.residual_dist_f64(Va, pa, Xa, 1.0, lsv, kt, [q], si[r])[0] for q, r in zip(check, sel)])
    assert np.max(np.abs(sd[sel].astype(np.float64) - got_d64)) <= 1e-5
    assert np.max(np.abs(sd[sel].astype(np.float64) - rd)) <= 1e-5
    exact, mism = O.near_tie_mismatches(si[sel], ri, lambda r, ids: O.residual_dist_f64(Va, pa, Xa, 1.0, lsv, kt,
                                                                                       [check[r]], ids)[0])
    assert all(g < 1e-6 for *_, g in mism), mism[:3]


@pytest.mark.parametrize("case", CASES)
def test_new_points_dense_and_screened(cuda_available, case):
    from covertreex_gb300.device import CudaResidualIndex

    n, d, m, kt, ls, k, nq = case
    X, V, p, Xq, qv, qp = _case(n, d, m, kt, ls, nq, seed=n + d)
    lsv = np.full(d, ls, np.float32)
    # the largest case starts from a reserved 4096-row query slab and outgrows it
    index = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=ls, kernel_type=kt, build_tree=False,
                              query_slab=nq > 4096)
    # dense: bit-exact against the f32 oracle of new points
    di, dd = index.knn_points_device(qv, qp, Xq, k, form="dense")
    ref = O.brute_knn_points_f32(V, p, X, 1.0, lsv, kt, qv, qp, Xq, k)
    assert np.array_equal(di.cpu().numpy(), ref[0]) and np.array_equal(dd.cpu().numpy(), ref[1])
    # screened: FP64 ground truth over the same stored f32 inputs
    si, sd = index.knn_points_device(qv, qp, Xq, k, form="screened")
    si, sd = si.cpu().numpy(), sd.cpu().numpy()
    _check_screened_vs_fp64(V, p, X, Xq, qv, qp, si, sd, kt, lsv, k)
    # the same points alone (a prefix and a strided subset) give the same rows, bit for bit
    for sub in (np.arange(17), np.arange(1, nq, 7)):
        ai, ad = index.knn_points_device(qv[sub], qp[sub], Xq[sub], k, form="screened")
        assert np.array_equal(ai.cpu().numpy(), si[sub]) and np.array_equal(ad.cpu().numpy(), sd[sub])
        bi, bd = index.knn_points_device(qv[sub], qp[sub], Xq[sub], k, form="dense")
        assert np.array_equal(bi.cpu().numpy(), ref[0][sub]) and np.array_equal(bd.cpu().numpy(), ref[1][sub])


def test_new_points_scattered_with_tiny_p(cuda_available):
    """A few scattered new points: one query tile spans the whole space, so the
    candidates are split into parts and each query's threshold is seeded from its
    Hilbert neighbours.  Some points sit on inducing points (p ~ 1e-6): their
    certified bounds cannot exclude candidates, their part slots overflow and are
    rescored over that part's candidates only.  Against FP64, and the same rows
    alone and in the mix."""
    from covertreex_gb300.device import CudaResidualIndex

    n, d, m, kt, ls, k = 30000, 3, 256, 1, 1.0, 50
    X = np.random.default_rng(31).standard_normal((n, d)).astype(np.float32)
    V, p, idx, L = O.build_residual_backend_np(X, seed=32, inducing_count=m, variance=1.0, lengthscale=ls,
                                               kernel_type=kt)
    r = np.random.default_rng(33)
    Xq = np.vstack([r.standard_normal((40, d)),
                    X[idx[:8]] + 1e-5 * r.standard_normal((8, d))]).astype(np.float32)
    qv, qp = _embed(Xq, X, idx, L, kt, ls)
    assert np.min(qp) < 1e-4
    lsv = np.full(d, ls, np.float32)
    index = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=ls, kernel_type=kt, build_tree=False)
    si, sd = index.knn_points_device(qv, qp, Xq, k, form="screened")
    assert index.last_stats["overflow_queries"] > 0  # the part-restricted exhaustive pass ran
    si, sd = si.cpu().numpy(), sd.cpu().numpy()
    _check_screened_vs_fp64(V, p, X, Xq, qv, qp, si, sd, kt, lsv, k)
    for sub in (np.arange(5), np.array([3, 41, 44, 47])):
        ai, ad = index.knn_points_device(qv[sub], qp[sub], Xq[sub], k, form="screened")
        assert np.array_equal(ai.cpu().numpy(), si[sub]) and np.array_equal(ad.cpu().numpy(), sd[sub])


def test_new_points_forced_exhaustive_pass(cuda_available, monkeypatch):
    """Smooth tree (Matern l=2) and a survivor cap of 32 per column half: most new
    points' slots overflow into the exhaustive pass and its certified FP32 filter;
    against FP64, bit-identical to the rows of the survivor pass, and each row
    against FP64 alone and in the mix."""
    from covertreex_gb300.device import CudaResidualIndex

    n, d, m, kt, ls, k, nq = 16384, 3, 128, 1, 2.0, 40, 600
    X, V, p, Xq, qv, qp = _case(n, d, m, kt, ls, nq, seed=77)
    lsv = np.full(d, ls, np.float32)
    index = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=ls, kernel_type=kt, build_tree=False)
    ri, rd = index.knn_points_device(qv, qp, Xq, k, form="screened")
    monkeypatch.setenv("CT_SCREEN_SURVIVOR_CAP", "64")
    si, sd = index.knn_points_device(qv, qp, Xq, k, form="screened")
    assert index.last_stats["overflow_queries"] > 100
    si, sd = si.cpu().numpy(), sd.cpu().numpy()
    _check_screened_vs_fp64(V, p, X, Xq, qv, qp, si, sd, kt, lsv, k)
    # the same rows as through the survivor pass, bit for bit
    assert np.array_equal(ri.cpu().numpy(), si) and np.array_equal(rd.cpu().numpy().view(np.uint32), sd.view(np.uint32))
    for sub in (np.arange(9), np.arange(2, nq, 11)):
        ai, ad = index.knn_points_device(qv[sub], qp[sub], Xq[sub], k, form="screened")
        ai, ad = ai.cpu().numpy(), ad.cpu().numpy()
        _check_screened_vs_fp64(V, p, X, Xq[sub], qv[sub], qp[sub], ai, ad, kt, lsv, k)
