"""GPU parity of the integer kernels against vectors produced by the reference's own
Python code (tests/golden, made by gen_golden.py) and against the oracle:

* device Hilbert keys + radix sort == _hilbert_permutation
  (covertreex/algo/order/strategy.py:38-100) for D = 2, 3, 5, 8, bit for bit;
* device Morton order == the restated hilbert_like_order (src/pcct.rs:27-67);
* device Luby MIS == _run_mis_numba_impl (covertreex/algo/_mis_numba.py:64-131) on the
  golden graphs (indicator and iteration count), and == the oracle's restatement on
  larger random graphs.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_device_hilbert_order_matches_reference_golden(cuda_available):
    from covertreex_gb300.device import batch_order

    g = np.load(GOLDEN / "hilbert.npz")
    for i in range(4):
        P = g[f"P{i}"]
        perm = batch_order(P.astype(np.float32), mode="hilbert")
        assert np.array_equal(perm, g[f"perm{i}"]), f"case {i} (D={P.shape[1]})"


@pytest.mark.parametrize("n,d,seed", [(20000, 3, 1), (4099, 8, 2), (70001, 2, 3)])
def test_device_hilbert_order_matches_oracle(cuda_available, n, d, seed):
    from covertreex_gb300.device import batch_order

    X = np.random.default_rng(seed).standard_normal((n, d)).astype(np.float32)
    X[::97] = X[1]  # duplicated points: equal keys keep the lower row first
    perm = batch_order(X, mode="hilbert")
    ref, _ = O.hilbert_order(X.astype(np.float64))
    assert np.array_equal(perm, ref)


def test_device_morton_order_matches_oracle(cuda_available):
    from covertreex_gb300.device import batch_order

    X = np.random.default_rng(5).standard_normal((30000, 3)).astype(np.float32)
    ref, _ = O.morton_order(X)
    assert np.array_equal(batch_order(X, mode="morton"), ref)
    Y = X[:, :2].copy()
    assert np.array_equal(batch_order(Y, mode="morton"), np.arange(30000))  # identity for D != 3


def test_device_luby_mis_matches_reference_golden(cuda_available):
    from covertreex_gb300.device import luby_mis

    g = np.load(GOLDEN / "mis.npz")
    for i in range(4):
        sel, it = luby_mis(g[f"indptr{i}"], g[f"indices{i}"], int(g[f"seed{i}"]))
        assert np.array_equal(sel, g[f"sel{i}"]), f"graph {i}"
        assert it == int(g[f"iters{i}"]), f"graph {i}"


def _random_graph(n, avg_deg, seed):
    r = np.random.default_rng(seed)
    m = n * avg_deg // 2
    a = r.integers(0, n, m)
    b = r.integers(0, n, m)
    keep = a != b
    a, b = a[keep], b[keep]
    u = np.concatenate([a, b])
    v = np.concatenate([b, a])
    key = np.unique(u * n + v)
    u, v = key // n, key % n
    indptr = np.zeros(n + 1, np.int64)
    np.add.at(indptr, u + 1, 1)
    return np.cumsum(indptr), v.astype(np.int64)


@pytest.mark.parametrize("n,deg,seed", [(5000, 3, 1), (20000, 12, 2), (3000, 60, 3)])
def test_device_luby_mis_matches_oracle(cuda_available, n, deg, seed):
    from covertreex_gb300.device import luby_mis

    indptr, indices = _random_graph(n, deg, seed)
    sel, it = luby_mis(indptr, indices, seed * 7 + 1)
    ref, rit = O.luby_mis(indptr, indices, seed * 7 + 1)
    assert np.array_equal(sel, ref)
    assert it == rit
    # independent and maximal
    s = sel.astype(bool)
    for v in range(n):
        nb = indices[indptr[v]:indptr[v + 1]]
        assert not (s[v] and s[nb].any())
        assert s[v] or s[nb].any()


def test_device_luby_mis_rejects_malformed_graph(cuda_available):
    from covertreex_gb300 import _lib
    from covertreex_gb300.device import luby_mis

    with pytest.raises(_lib.EngineError):
        luby_mis(np.array([0, 1, 2]), np.array([1, 5]), 3)  # neighbour index 5 outside [0, 2)
    with pytest.raises(_lib.EngineError):
        luby_mis(np.array([0, 2, 1]), np.array([1, 0]), 3)  # decreasing indptr
