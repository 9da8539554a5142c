"""GPU parity at the full benchmark shapes.

* Precision workload: N=262144, D=8, m=512, RBF l=2 over a seeded mixture of 16
  Gaussians, k=50, predecessor mode.  The screened form is run over ALL N queries (the
  benchmark's call) and 4096 rows sampled by ``default_rng(4).choice(N, 4096, False)``
  are checked against the FP64 brute force: neighbour sets equal except swaps between
  candidates whose FP64 distances differ by < 1e-6 (listed near-ties), distances within
  1e-5, and the predecessor constraint j < i exact with min(k, i) neighbours per row.
  The plain FP32 dense form is checked bit for bit (indices and float bits) against the
  oracle's f32 brute force on the same 4096 ids.
* README shape: N=32768, D=3, m=256, Matern 5/2 l=1, k=50, in both predecessor modes:
  the screened form over all N queries against FP64 on 4096 sampled rows, and the dense
  form over all N queries bit for bit against the f32 oracle.  The Euclidean run on the
  same coordinates (k=10, queries = coords) is checked against the FP64 brute force.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NEAR_TIE = 1e-6
DIST_TOL = 1e-5
SAMPLE = 4096


def _index(wl):
    from covertreex_gb300.device import CudaResidualIndex

    return CudaResidualIndex(wl.v, wl.p, wl.coords, variance=wl.variance, lengthscale=[wl.lengthscale] * wl.d,
                             kernel_type=wl.kernel_type, build_tree=False)


def _sample(n):
    return np.random.default_rng(4).choice(n, min(SAMPLE, n), replace=False)


def _check_fp64(wl, q, k, predecessor, gi, gd):
    """Screened rows gi/gd (for query ids q) against the FP64 brute force."""
    ls = [wl.lengthscale] * wl.d
    fi, fd = O.brute_knn_f64_c(wl.v, wl.p, wl.coords, wl.variance, ls, wl.kernel_type, q, k, predecessor)
    valid = fi >= 0
    assert np.array_equal(gi >= 0, valid), "number of neighbours differs from FP64"
    err = np.abs(gd.astype(np.float64) - np.where(valid, fd, 0.0))[valid]
    assert err.max() <= DIST_TOL, float(err.max())

    def dist_fn(r, ids):
        return O.residual_dist_f64(wl.v, wl.p, wl.coords, wl.variance, ls, wl.kernel_type, np.array([q[r]]), ids)[0]

    exact, mism = O.near_tie_mismatches(gi, fi, dist_fn)
    bad = [t for t in mism if t[3] >= NEAR_TIE]
    assert not bad, bad[:5]
    if predecessor:
        assert np.all(np.where(gi >= 0, gi, -1) < q[:, None])
        assert np.array_equal((gi >= 0).sum(1), np.minimum(k, q))
    return exact, mism, float(err.max())


@pytest.fixture(scope="module")
def precision():
    from covertreex_gb300 import synthetic

    wl = synthetic.make("precision")
    idx = _index(wl)
    yield wl, idx
    idx.free()


def test_precision_screened_all_queries_vs_fp64(cuda_available, precision):
    wl, idx = precision
    assert (wl.n, wl.d, wl.m, wl.k, wl.predecessor, wl.kernel_type) == (262144, 8, 512, 50, True, 0)
    gi, gd = idx.knn(np.arange(wl.n), wl.k, predecessor=True, form="screened")
    q = _sample(wl.n)
    exact, mism, err = _check_fp64(wl, q, wl.k, True, gi[q], gd[q])
    print(f"precision workload: {exact}/{q.size} rows identical to FP64, {len(mism)} near-tie rows, "
          f"max |d - d64| {err:.2e}")


def test_precision_dense_bit_exact_sampled(cuda_available, precision):
    wl, idx = precision
    q = np.sort(_sample(wl.n))
    gi, gd = idx.knn(q, wl.k, predecessor=True, form="dense")
    oi, od = O.brute_knn_f32(wl.v, wl.p, wl.coords, wl.variance, [wl.lengthscale] * wl.d, wl.kernel_type, q, wl.k,
                             True)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))


@pytest.fixture(scope="module")
def readme():
    from covertreex_gb300 import synthetic

    wl = synthetic.make("readme")
    idx = _index(wl)
    yield wl, idx
    idx.free()


@pytest.mark.parametrize("predecessor", [True, False])
def test_readme_screened_all_queries_vs_fp64(cuda_available, readme, predecessor):
    wl, idx = readme
    assert (wl.n, wl.d, wl.m, wl.k, wl.kernel_type) == (32768, 3, 256, 50, 1)
    gi, gd = idx.knn(np.arange(wl.n), wl.k, predecessor=predecessor, form="screened")
    q = _sample(wl.n)
    _check_fp64(wl, q, wl.k, predecessor, gi[q], gd[q])


@pytest.mark.parametrize("predecessor", [True, False])
def test_readme_dense_bit_exact_all_queries(cuda_available, readme, predecessor):
    wl, idx = readme
    q = np.arange(wl.n)
    gi, gd = idx.knn(q, wl.k, predecessor=predecessor, form="dense")
    oi, od = O.brute_knn_f32(wl.v, wl.p, wl.coords, wl.variance, [wl.lengthscale] * wl.d, wl.kernel_type, q, wl.k,
                             predecessor)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))


def test_readme_euclidean_k10_vs_fp64(cuda_available, readme):
    """The README shape's Euclidean run: k=10, queries = the 32768 coordinates."""
    from covertreex_gb300 import cover_tree

    wl, _ = readme
    X = wl.coords
    tree = cover_tree(X)
    idx, dist = tree.knn(k=10, queries=X, return_distances=True)
    fi, fd = O.brute_knn_euclidean_f64(X, X, 10)
    assert np.abs(dist.astype(np.float64) - fd).max() < 1e-5
    X64 = X.astype(np.float64)
    for r in np.nonzero(np.any(np.sort(idx, 1) != np.sort(fi, 1), axis=1))[0]:
        a = np.setdiff1d(idx[r], fi[r])
        b = np.setdiff1d(fi[r], idx[r])
        da = np.sqrt(((X64[r] - X64[a]) ** 2).sum(-1))
        db = np.sqrt(((X64[r] - X64[b]) ** 2).sum(-1))
        # only swaps at float32 ties of the squared distance are allowed
        assert np.abs(np.sort(da) - np.sort(db)).max() < 1e-6, (r, a, b)
