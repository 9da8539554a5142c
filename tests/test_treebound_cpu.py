"""CPU check of the certified error model of the tree form's prune (the FP32 restatement
of ct_treebound.cuh): for random, near and tiny-p pairs of both kernels, the squared
FP32 distance (the oracle's bit-exact batch-path value) lies within delta of the squared
FP64 distance over the same stored inputs, and delta is not vacuous on well-conditioned
pairs.  (delta also covers the f32 rounding of V and the FP64 construction error, which
the FP64-over-stored-inputs value does not see.)"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

U = 2.0 ** -24
ETA = 2.0 ** -28
F = np.float32


def bound_model(m, d, kt, var, vmax, nmax):
    kc = 1.0 if kt == 0 else 2.0
    return dict(ck=F(var * kc * (d + 8) * U * 1.01), ck0=F(var * 16.0 * U),
                cdot=F(((m / 8.0 + 12.0) * U + 2.0 * ETA) * 1.01), cvar=F(var * U * 2.0),
                cpa=F((m + 2) * 1.2e-16), cpb=F(2.0 * ETA), var=F(var), vmax=F(vmax), nmax=F(nmax))


def pair_delta(B, nq, nx, vq, vx, isq, isx):
    """ct_treebound.cuh pair_delta, operation by operation in float32."""
    a = (B["ck"] * (nq + nx) + B["ck0"] + B["cdot"] * vq * vx + B["cvar"]) * isq * isx
    rq = F(6.0e-8) + (B["cpa"] * (B["var"] + vq * vq) + B["cpb"] * vq * vq) * isq * isq
    rx = F(6.0e-8) + (B["cpa"] * (B["var"] + vx * vx) + B["cpb"] * vx * vx) * isx * isx
    return (a + F(0.55) * (rq + rx)) * F(1.0001) + F(5.0e-7)


@pytest.mark.parametrize("kind", ["rbf_d8", "matern_d3", "matern_d3_long"])
def test_fp32_distance_within_certified_delta(kind):
    if kind == "rbf_d8":
        case = mixture_case(3000, 8, 128, 2.0)
    elif kind == "matern_d3":
        case = gaussian_case(3000, 3, 64, 1, 1.0, seed=3)
    else:
        case = gaussian_case(3000, 3, 96, 1, 2.5, seed=4)
    V, p, X = case["V"], case["p"], case["X"]
    n, m = V.shape
    d = X.shape[1]
    xs = (X * (F(1.0) / case["ls"].astype(F))).astype(F)
    norms = np.einsum("ij,ij->i", xs.astype(np.float64), xs.astype(np.float64)).astype(F)
    vn = (np.sqrt((V.astype(np.float64) ** 2).sum(1)) * (1 + 1e-6)).astype(F)
    isp = (1.0 / np.sqrt(p.astype(np.float64)) * (1 + 1e-6)).astype(F)
    B = bound_model(m, d, case["kt"], 1.0, vn.max(), norms.max())
    r = np.random.default_rng(11)
    qi = np.concatenate([r.integers(0, n, 4000), np.repeat(case["inducing"][:8], 50)])
    cj = np.concatenate([r.integers(0, n, 4000), r.integers(0, n, 400)])
    # near pairs: each query with its 5 nearest FP64 neighbours
    near_q = r.choice(n, 200, replace=False)
    fi, _ = O.brute_knn_f64(V, p, X, 1.0, case["ls"], case["kt"], near_q, 6, False)
    qi = np.concatenate([qi, np.repeat(near_q, 6)])
    cj = np.concatenate([cj, fi.reshape(-1)])
    keep = cj >= 0
    qi, cj = qi[keep], cj[keep]
    d32 = O.pair_dist_f32(V, p, X, 1.0, case["ls"], case["kt"], qi, cj).astype(np.float64)
    d64 = np.array([O.residual_dist_f64(V, p, X, 1.0, case["ls"], case["kt"], [a], [b])[0, 0]
                    for a, b in zip(qi, cj)])
    delta = pair_delta(B, norms[qi], norms[cj], vn[qi], vn[cj], isp[qi], isp[cj]).astype(np.float64)
    err = np.abs(d32 ** 2 - d64 ** 2)
    assert np.all(err <= delta), float((err / delta).max())
    well = (isp[qi] < 8) & (isp[cj] < 8)
    assert np.median(delta[well]) < 1e-3
