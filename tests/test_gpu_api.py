"""The reference-facing API (cover_tree / BuiltCoverTree.knn / engine "cuda") on the GPU."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_cover_tree_kernel_path_matches_fp64(cuda_available):
    from covertreex_gb300 import Matern52, cover_tree

    X = np.random.default_rng(0).standard_normal((3000, 3)).astype(np.float32)
    tree = cover_tree(X, kernel=Matern52(lengthscale=1.0), inducing_count=64, seed=42)
    idx, dist = tree.knn(k=10, predecessor_mode=True, return_distances=True)
    assert idx.shape == (3000, 10) and idx.dtype == np.int64 and dist.dtype == np.float32
    for i in range(3000):
        valid = idx[i][idx[i] >= 0]
        assert np.all(valid < i) and len(valid) == min(10, i)
    V, p, _, _ = O.build_residual_backend_np(X, seed=42, inducing_count=64, variance=1.0, lengthscale=1.0,
                                             kernel_type=1)
    q = np.arange(100, 3000, 29)
    fi, fd = O.brute_knn_f64(V, p, X, 1.0, [1.0] * 3, 1, q, 10, True)
    assert np.abs(dist[q].astype(np.float64) - fd).max() < 1e-5


def test_cover_tree_v_matrix_path(cuda_available):
    from covertreex_gb300 import cover_tree

    X = np.random.default_rng(1).standard_normal((800, 2)).astype(np.float32)
    V, p, _, _ = O.build_residual_backend_np(X, seed=3, inducing_count=32, variance=1.0, lengthscale=1.0,
                                             kernel_type=0)
    tree = cover_tree(X, v_matrix=V, p_diag=p)
    idx = tree.knn(k=5, queries=[10, 20, 30])
    assert idx.shape == (3, 5)
    dense = tree.knn(k=5, queries=[10, 20, 30], form="dense")
    oi, _ = O.brute_knn_f32(V, p, X, 1.0, [1.0, 1.0], 0, np.array([10, 20, 30]), 5, False)
    assert np.array_equal(dense, oi)


def test_single_query_is_squeezed_like_the_reference(cuda_available):
    from covertreex_gb300 import RBF, cover_tree

    X = np.random.default_rng(2).standard_normal((300, 3)).astype(np.float32)
    tree = cover_tree(X, kernel=RBF(), inducing_count=32)
    one = tree.knn(k=4, queries=[7])
    assert one.shape == (4,)
    i1, d1 = tree.knn(k=1, queries=[7], return_distances=True)
    assert int(i1) == 7 and float(d1) == 0.0


def test_residual_engine_rejects_point_payloads(cuda_available):
    from covertreex_gb300 import RBF, cover_tree

    X = np.random.default_rng(3).standard_normal((100, 3)).astype(np.float32)
    tree = cover_tree(X, kernel=RBF(), inducing_count=16)
    with pytest.raises(ValueError):
        tree.knn(k=3, queries=X[:2])
    with pytest.raises(ValueError):
        tree.knn(k=0)
    with pytest.raises(ValueError):
        tree.knn(k=3, queries=[100])


@pytest.mark.parametrize("predecessor", [False, True])
def test_euclidean_cover_tree_exact(cuda_available, predecessor):
    from covertreex_gb300 import cover_tree

    X = np.random.default_rng(4).standard_normal((2000, 3)).astype(np.float32)
    tree = cover_tree(X)
    idx, dist = tree.knn(k=10, queries=X, return_distances=True, predecessor_mode=predecessor)
    fi, fd = O.brute_knn_euclidean_f64(X, X, 10, predecessor=predecessor)
    assert np.abs(np.where(fi >= 0, dist, 0) - np.where(fi >= 0, fd, 0)).max() < 1e-5
    mism = [r for r in range(2000) if set(idx[r]) != set(fi[r])]
    for r in mism:  # only swaps at exact float ties are allowed
        a = np.setdiff1d(idx[r], fi[r])
        b = np.setdiff1d(fi[r], idx[r])
        da = np.sqrt(((X[r].astype(np.float64) - X[a].astype(np.float64)) ** 2).sum(-1))
        db = np.sqrt(((X[r].astype(np.float64) - X[b].astype(np.float64)) ** 2).sum(-1))
        assert np.abs(np.sort(da) - np.sort(db)).max() < 1e-6
