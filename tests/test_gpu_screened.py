"""GPU checks of the precision form: the tcgen05 BF16 screening pass and the
screened kNN against the FP64 brute-force oracle.

Tolerance (the precision form's contract): neighbour index sets equal to the FP64 answer
with ties broken by lower index, except swaps between candidates whose FP64
distances differ by < 1e-6 (listed near-ties); distances within 1e-5 of FP64.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

pytestmark = pytest.mark.gpu

NEAR_TIE = 1e-6
DIST_TOL = 1e-5


def _index(case, build_tree=False):
    from covertreex_gb300.device import CudaResidualIndex

    return CudaResidualIndex(case["V"], case["p"], case["X"], variance=case["var"], lengthscale=case["ls"],
                             kernel_type=case["kt"], build_tree=build_tree)


def test_screen_dots_within_certified_bound(cuda_available):
    case = mixture_case(4000, 8, 512, 2.0)
    idx = _index(case)
    r = np.random.default_rng(0)
    ra = r.choice(4000, 128, replace=False)
    rb = r.choice(4000, 256, replace=False)
    got = idx.debug_screen_dots(ra, rb).astype(np.float64)
    V = case["V"].astype(np.float64)
    exact = V[ra] @ V[rb].T
    nrm = np.linalg.norm(V, axis=1)
    scale = nrm[ra][:, None] * nrm[rb][None, :]
    m = 512
    c_split = 3.1 * 2.0 ** -16 + (3 * m / 16 + 17) * 2.0 ** -22
    err = np.abs(got - exact)
    assert np.all(err <= c_split * scale), float((err / scale).max())
    # the hi/lo split is far more accurate than a single bf16 product
    assert (err / scale).max() < 0.25 * c_split


def test_screen_dots_padding_rows_are_zero(cuda_available):
    case = gaussian_case(600, 3, 64, 1, 1.0, seed=2)
    idx = _index(case)
    got = idx.debug_screen_dots(np.arange(100), np.arange(200))
    assert np.all(got[100:, :] == 0) and np.all(got[:, 200:] == 0)
    V = case["V"].astype(np.float64)
    nrm = np.linalg.norm(V, axis=1)
    c_split = 3.1 * 2.0 ** -16 + (3 * 64 / 16 + 17) * 2.0 ** -22
    err = np.abs(got[:100, :200] - V[:100] @ V[:200].T)
    assert np.all(err <= c_split * nrm[:100, None] * nrm[None, :200])


def _check_against_fp64(case, q, k, predecessor, gi, gd):
    fi, fd = O.brute_knn_f64(case["V"], case["p"], case["X"], case["var"], case["ls"], case["kt"], q, k, predecessor)
    valid = fi >= 0
    assert np.array_equal(gi >= 0, valid)
    err = np.abs(gd.astype(np.float64) - np.where(valid, fd, 0.0))[valid]
    assert err.max() <= DIST_TOL, float(err.max())

    def dist_fn(r, ids):
        return O.residual_dist_f64(case["V"], case["p"], case["X"], case["var"], case["ls"], case["kt"],
                                   np.array([q[r]]), ids)[0]

    exact, mism = O.near_tie_mismatches(gi, fi, dist_fn)
    bad = [t for t in mism if t[3] >= NEAR_TIE]
    assert not bad, bad[:5]
    return exact, mism, float(err.max())


@pytest.mark.parametrize("predecessor", [False, True])
def test_screened_cfg0_shape_vs_fp64(cuda_available, predecessor):
    """N=8192, D=3, m=64, Matern 5/2 l=1, k=50."""
    case = gaussian_case(8192, 3, 64, 1, 1.0, seed=0)
    idx = _index(case)
    q = np.arange(8192)
    gi, gd = idx.knn(q, 50, predecessor=predecessor, form="screened")
    sub = np.random.default_rng(1).choice(8192, 600, replace=False)
    _check_against_fp64(case, q[sub], 50, predecessor, gi[sub], gd[sub])


def test_screened_mixture_d8_subset(cuda_available):
    """D=8 mixture of Gaussians, RBF l=2, m=512; query subset in predecessor mode."""
    case = mixture_case(20000, 8, 512, 2.0)
    idx = _index(case)
    q = np.sort(np.random.default_rng(4).choice(20000, 700, replace=False))
    gi, gd = idx.knn(q, 50, predecessor=True, form="screened")
    _check_against_fp64(case, q, 50, True, gi, gd)
    gi2, gd2 = idx.knn(q[::-1].copy(), 50, predecessor=True, form="screened")  # unsorted query order
    assert np.array_equal(gi2[::-1], gi)


@pytest.mark.parametrize("predecessor", [False, True])
def test_screened_scattered_small_id_set(cuda_available, predecessor):
    """A few scattered query ids (candidate parts, seeded thresholds) including
    inducing rows (p ~ 1e-6: overflowed part slots rescored over their part's
    candidates only), against FP64."""
    case = gaussian_case(30000, 3, 256, 1, 1.0, seed=11)
    idx = _index(case)
    r = np.random.default_rng(12)
    q = np.concatenate([r.choice(30000, 40, replace=False), case["inducing"][:8]]).astype(np.int64)
    gi, gd = idx.knn(q, 50, predecessor=predecessor, form="screened")
    if not predecessor:  # every candidate is eligible: the inducing rows' part slots overflow
        assert idx.last_stats["overflow_queries"] > 0
    _check_against_fp64(case, q, 50, predecessor, gi, gd)


def test_screened_predecessor_invariants(cuda_available):
    case = gaussian_case(300, 2, 32, 0, 1.0, seed=42)
    idx = _index(case)
    gi, gd = idx.knn(np.arange(300), 10, predecessor=True, form="screened")
    for i in range(300):
        valid = gi[i][gi[i] >= 0]
        assert np.all(valid < i) and len(valid) == min(10, i)
    assert np.all(gi[0] == -1)


def test_screened_matches_dense_where_well_conditioned(cuda_available):
    """Plain FP32 (dense) and screened forms agree on rows whose residual variance is not tiny."""
    case = gaussian_case(4000, 3, 64, 1, 1.0, seed=7)
    idx = _index(case)
    q = np.arange(4000)
    di, dd = idx.knn(q, 20, predecessor=True, form="dense")
    si, sd = idx.knn(q, 20, predecessor=True, form="screened")
    good = case["p"] >= 0.05
    agree = np.mean([set(a) == set(b) for a, b, g in zip(di, si, good) if g])
    assert agree > 0.99


@pytest.mark.parametrize("predecessor", [False, True])
def test_screened_forced_exhaustive_pass_vs_fp64(cuda_available, monkeypatch, predecessor):
    """A survivor cap of 32 per column half overflows most query slots of a smooth
    Matern l=2 case, so the exhaustive pass runs over well-conditioned queries: its
    certified FP32 filter (exact distances only where the lower bound reaches the
    query's threshold) must leave the answer equal to FP64.  Every pass computes a pair's
    exact distance from the same double-float dot, so the rows equal those of the
    survivor pass bit for bit."""
    case = gaussian_case(12000, 3, 128, 1, 2.0, seed=21)
    idx = _index(case)
    q = np.random.default_rng(22).choice(12000, 500, replace=False).astype(np.int64)
    monkeypatch.setenv("CT_SCREEN_SURVIVOR_CAP", "64")
    gi, gd = idx.knn(q, 40, predecessor=predecessor, form="screened")
    st = idx.last_stats
    assert st["overflow_queries"] > 100
    _check_against_fp64(case, q, 40, predecessor, gi, gd)
    # the same queries through the survivor pass
    monkeypatch.delenv("CT_SCREEN_SURVIVOR_CAP")
    hi, hd = idx.knn(q, 40, predecessor=predecessor, form="screened")
    assert idx.last_stats["overflow_queries"] < st["overflow_queries"]
    assert np.array_equal(hi, gi) and np.array_equal(hd.view(np.uint32), gd.view(np.uint32))
