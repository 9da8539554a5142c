"""CoverTree(runtime).fit / insert / delete / knn on the GPU, used as the reference's own
tests use it (tests/test_predecessor_mode.py: configure_residual_correlation, then
CoverTree(Runtime(metric="residual_correlation", ...)).fit(points, mis_seed=7).knn(ids))."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _backend(n, d, m, seed, kt=1):
    from covertreex_gb300 import build_residual_backend

    X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
    hb = build_residual_backend(X, seed=99, inducing_count=m, variance=1.0, lengthscale=1.0, kernel_type=kt)
    return X, hb


def _runtime(**kw):
    from covertreex_gb300 import Runtime

    return Runtime(backend="numpy", precision="float32", metric="residual_correlation", enable_rust=True,
                   engine="rust-natural", residual_use_static_euclidean_tree=True, **kw)


def test_fit_knn_predecessor_and_parity(cuda_available):
    from covertreex_gb300 import CoverTree, configure_residual_correlation

    X, hb = _backend(1500, 2, 128, 42)
    configure_residual_correlation(hb)
    tree = CoverTree(_runtime()).fit(X, mis_seed=7)
    assert tree.num_points == 1500
    q = np.arange(1500, dtype=np.int64).reshape(-1, 1)
    nb = np.asarray(tree.knn(q, k=10, predecessor_mode=True))
    for i in range(1500):
        valid = nb[i][nb[i] >= 0]
        assert np.all(valid < i) and valid.size == min(10, i)
    ls = np.ones(2, np.float32)
    dense = tree.knn(q, k=10, predecessor_mode=True, form="dense")
    ref = O.brute_knn_f32(hb.v_matrix, hb.p_diag, X, 1.0, ls, 1, np.arange(1500), 10, True)
    assert np.array_equal(dense, ref[0])
    idx, dist = tree.knn(q[100:400], k=10, predecessor_mode=False, return_distances=True)
    fi, fd = O.brute_knn_f64(hb.v_matrix, hb.p_diag, X, 1.0, ls, 1, np.arange(100, 400), 10, False)
    assert np.abs(dist.astype(np.float64) - fd).max() < 1e-5
    single = tree.nearest(np.array([[7]]))
    assert int(single) == 7  # a dataset row is its own nearest neighbour (distance 0)


def test_insert_then_delete_keep_dataset_numbering(cuda_available):
    from covertreex_gb300 import CoverTree, configure_residual_correlation

    X, hb = _backend(1200, 3, 64, 5, kt=0)
    configure_residual_correlation(hb)
    rt = _runtime()
    full = CoverTree(rt).fit(X, mis_seed=3)
    first = CoverTree(rt).fit(X[:700], mis_seed=3)
    part = first.insert(X[700:])  # a handle grown on the device from first's
    assert part.num_points == 1200 and first.num_points == 700
    q = np.arange(0, 1200, 7, dtype=np.int64)
    for pred in (False, True):
        a = full.knn(q, k=8, predecessor_mode=pred, form="dense")
        for form in ("dense", "tree", "screened"):
            b = part.knn(q, k=8, predecessor_mode=pred, form=form)
            assert np.array_equal(a, b) if form != "screened" else np.array_equal(
                b, full.knn(q, k=8, predecessor_mode=pred, form="screened")), form
    # trees are immutable: the tree inserted into still answers over its 700 rows
    q7 = np.arange(0, 700, 9, dtype=np.int64)
    ref7, _ = O.brute_knn_f32(hb.v_matrix[:700], hb.p_diag[:700], X[:700], 1.0, np.ones(3, np.float32), 0, q7, 8,
                              True)
    assert np.array_equal(first.knn(q7, k=8, predecessor_mode=True, form="tree"), ref7)
    gone = np.array([0, 5, 17, 333, 1199])
    smaller = full.delete(gone)
    assert smaller.num_points == 1200 - gone.size
    keep = np.setdiff1d(np.arange(1200), gone)
    qk = keep[::11]
    got = smaller.knn(qk, k=8, predecessor_mode=True, form="dense")
    assert not np.isin(got, gone).any()
    ls = np.ones(3, np.float32)
    ref_i, _ = O.brute_knn_f32(hb.v_matrix[keep], hb.p_diag[keep], X[keep], 1.0, ls, 0,
                               np.searchsorted(keep, qk), 8, True)
    ref = np.where(ref_i >= 0, keep[np.maximum(ref_i, 0)], -1)
    assert np.array_equal(got, ref)
    with pytest.raises(ValueError):
        smaller.knn(np.array([5]), k=3)  # deleted id


def test_euclidean_runtime(cuda_available):
    from covertreex_gb300 import CoverTree, Runtime

    X = np.random.default_rng(8).standard_normal((2000, 3)).astype(np.float32)
    tree = CoverTree(Runtime(metric="euclidean")).fit(X)
    idx, dist = tree.knn(X[:50], k=5, return_distances=True)
    d2 = ((X[:50, None, :].astype(np.float64) - X[None, :, :]) ** 2).sum(-1)
    ref = np.argsort(d2, axis=1, kind="stable")[:, :5]
    assert np.array_equal(np.sort(idx, axis=1), np.sort(ref, axis=1))
