"""Device cover-tree build and the plain FP32 traversal form.

Structure: every non-root node has a parent chain ending at a root; the cover
radius si[a] bounds d(a, x) for every descendant x (checked with the oracle's
bit-exact f32 distance); subtree_min matches the reference's relaxation
(src/tree.rs:144-185).  Search: the traversal scores pairs bit-identically to
the dense form, so on well-conditioned queries (p_q >= 0.05, where the f32
metric obeys the triangle inequality to rounding) its neighbour lists equal the
dense form's exactly.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

pytestmark = pytest.mark.gpu


def _tree_index(case):
    from covertreex_gb300.device import CudaResidualIndex

    return CudaResidualIndex(case["V"], case["p"], case["X"], variance=case["var"], lengthscale=case["ls"],
                             kernel_type=case["kt"], build_tree=True)


def test_tree_structure_and_radii(cuda_available):
    case = gaussian_case(4000, 3, 64, 1, 1.0, seed=8)
    idx = _tree_index(case)
    t = idx.tree_arrays()
    par, order, si = t["parents"], t["node_to_dataset"], t["si"]
    n = 4000
    assert np.array_equal(np.sort(order), np.arange(n))
    roots = np.nonzero(par < 0)[0]
    assert 1 <= roots.size <= 64
    # every chain ends at a root within n steps; collect ancestor pairs
    anc_pairs = []
    for x in range(n):
        a, steps = par[x], 0
        while a >= 0:
            anc_pairs.append((a, x))
            a = par[a]
            steps += 1
            assert steps < n
    A = np.array(anc_pairs)
    d = O.pair_dist_f32(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, order[A[:, 0]], order[A[:, 1]])
    assert np.all(d <= si[A[:, 0]]), "cover radius below a descendant distance"
    mn, _ = O.subtree_bounds(par, order)
    assert np.array_equal(mn, t["subtree_min"])


@pytest.mark.parametrize("predecessor", [False, True])
def test_traversal_matches_dense_on_well_conditioned_rows(cuda_available, predecessor):
    case = gaussian_case(8192, 3, 64, 1, 1.0, seed=0)
    idx = _tree_index(case)
    q = np.arange(8192)
    ti, td = idx.knn(q, 50, predecessor=predecessor, form="tree")
    di, dd = idx.knn(q, 50, predecessor=predecessor, form="dense")
    well = case["p"] >= 0.05
    assert np.array_equal(ti[well], di[well])
    assert np.array_equal(td[well].view(np.uint32), dd[well].view(np.uint32))
    assert np.mean(np.all(ti == di, axis=1)) > 0.97


def test_traversal_d8_mixture(cuda_available):
    case = mixture_case(6000, 8, 128, 2.0)
    idx = _tree_index(case)
    q = np.random.default_rng(4).choice(6000, 600, replace=False)
    ti, td = idx.knn(q, 30, predecessor=True, form="tree")
    di, dd = idx.knn(q, 30, predecessor=True, form="dense")
    well = case["p"][q] >= 0.05
    assert np.array_equal(ti[well], di[well])
    for i in range(q.size):
        valid = ti[i][ti[i] >= 0]
        assert np.all(valid < q[i]) and len(valid) == min(30, q[i])
