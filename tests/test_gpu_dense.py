"""GPU parity of the plain FP32 dense form against the CPU oracle.

The dense form must reproduce the oracle's batch-path f32 residual distance
(src/metric.rs:376-487 restated in oracle/ct_oracle.c) bit for bit, and hence
the exact same neighbour lists in (distance, index) order.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

pytestmark = pytest.mark.gpu


def _run(case, k, predecessor, queries=None, form="dense"):
    from covertreex_gb300.device import CudaResidualIndex

    n = case["V"].shape[0]
    q = np.arange(n) if queries is None else np.asarray(queries)
    idx = CudaResidualIndex(case["V"], case["p"], case["X"], variance=case["var"], lengthscale=case["ls"],
                            kernel_type=case["kt"], build_tree=False)
    gi, gd = idx.knn(q, k, predecessor=predecessor, form=form)
    oi, od = O.brute_knn_f32(case["V"], case["p"], case["X"], case["var"], case["ls"], case["kt"], q, k, predecessor)
    return gi, gd, oi, od


@pytest.mark.parametrize("kt", [0, 1])
@pytest.mark.parametrize("predecessor", [False, True])
def test_dense_bit_exact_small(cuda_available, kt, predecessor):
    case = gaussian_case(1500, 3, 64, kt, 1.0, seed=11)
    gi, gd, oi, od = _run(case, 20, predecessor)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))


def test_dense_cfg0_shape(cuda_available):
    """N=8192, D=3, m=64, Matern 5/2 l=1, k=50 (both modes)."""
    case = gaussian_case(8192, 3, 64, 1, 1.0, seed=0)
    for pred in (False, True):
        gi, gd, oi, od = _run(case, 50, pred)
        assert np.array_equal(gi, oi)
        assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))


def test_dense_d8_rbf_subset(cuda_available):
    """D=8 mixture, RBF l=2, m=128; a query subset in both modes."""
    case = mixture_case(6000, 8, 128, 2.0)
    q = np.random.default_rng(4).choice(6000, 700, replace=False)
    for pred in (False, True):
        gi, gd, oi, od = _run(case, 50, pred, queries=q)
        assert np.array_equal(gi, oi)
        assert np.array_equal(gd.view(np.uint32), od.view(np.uint32))


def test_dense_predecessor_invariants(cuda_available):
    """tests/test_predecessor_mode.py:26-120 invariants: j < i, query 0 empty, query 1 -> [0]."""
    case = gaussian_case(100, 2, 32, 0, 1.0, seed=42)
    gi, gd, _, _ = _run(case, 10, True)
    for i in range(100):
        valid = gi[i][gi[i] >= 0]
        assert np.all(valid < i)
        assert len(valid) == min(10, i)
    assert np.all(gi[0] == -1) and np.all(gd[0] == np.float32(3.402823466e38))
    assert list(gi[1][gi[1] >= 0]) == [0]


def test_dense_k_larger_than_n(cuda_available):
    case = gaussian_case(40, 3, 16, 1, 1.0, seed=5)
    gi, gd, oi, od = _run(case, 64, False)
    assert np.array_equal(gi, oi)
    assert (gi[:, 40:] == -1).all()
