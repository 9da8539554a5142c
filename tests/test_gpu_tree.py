"""Device cover-tree build and the exact plain FP32 traversal form.

Structure: every non-root node has a parent chain ending at a root, levels fall
strictly along it (down to the floor level), the FP32 cover radius si[a] bounds
d32(a, x) for every descendant x (checked with the oracle's bit-exact f32
distance), and subtree_min matches the reference's relaxation
(src/tree.rs:144-185).  Rows of tiny residual variance are roots without children.

Search: the traversal scores pairs bit-identically to the dense form and prunes
only on certified bounds, so its neighbour lists equal the dense form's on EVERY
row (indices and float bits), tiny-p rows included.  The reference's parity-mode
distance evaluations per query are reported beside the device's.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

pytestmark = pytest.mark.gpu


def _tree_index(case, **kw):
    from covertreex_gb300.device import CudaResidualIndex

    return CudaResidualIndex(case["V"], case["p"], case["X"], variance=case["var"], lengthscale=case["ls"],
                             kernel_type=case["kt"], build_tree=True, **kw)


def test_tree_structure_and_radii(cuda_available):
    case = gaussian_case(4000, 3, 64, 1, 1.0, seed=8)
    idx = _tree_index(case)
    t = idx.tree_arrays()
    info = idx.build_info()
    par, order, si, lev = t["parents"], t["node_to_dataset"], t["si"], t["levels"]
    n = 4000
    assert np.array_equal(np.sort(order), np.arange(n))
    roots = np.nonzero(par < 0)[0]
    side = case["p"][order] < 1.0 / 1024
    assert info["side_rows"] == side.sum() and info["roots"] == roots.size == 1 + side.sum()
    assert np.all(par[side] < 0)                      # side rows are roots
    assert not np.isin(np.nonzero(side)[0], par).any()  # ... without children
    assert info["groups"] == len(O.prefix_slices(n - side.sum() - 1))
    # chains end at a root, levels fall strictly (the floor level -30 may repeat)
    anc_pairs = []
    for x in range(n):
        a, steps = par[x], 0
        while a >= 0:
            assert lev[a] > lev[x] or lev[a] == lev[x] == -30
            anc_pairs.append((a, x))
            a = par[a]
            steps += 1
            assert steps < 64
    A = np.array(anc_pairs)
    d = O.pair_dist_f32(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, order[A[:, 0]], order[A[:, 1]])
    assert np.all(d <= si[A[:, 0]]), "cover radius below a descendant distance"
    mn, _ = O.subtree_bounds(par, order)
    assert np.array_equal(mn, t["subtree_min"])


@pytest.mark.parametrize("predecessor", [False, True])
def test_traversal_equals_dense_on_every_row(cuda_available, predecessor):
    case = gaussian_case(8192, 3, 64, 1, 1.0, seed=0)
    idx = _tree_index(case)
    q = np.arange(8192)
    ti, td = idx.knn(q, 50, predecessor=predecessor, form="tree")
    evals = idx.last_stats["distance_evals"]
    di, dd = idx.knn(q, 50, predecessor=predecessor, form="dense")
    assert np.array_equal(ti, di)
    assert np.array_equal(td.view(np.uint32), dd.view(np.uint32))
    # the reference's parity mode on the same inputs (oracle restatement), for scale
    ref = O.OracleResidualTree(case["V"], case["p"], case["X"], 1.0, case["ls"], kernel_type=1, parity=True)
    ref.knn(q[::16], 50, predecessor=predecessor, parity=True)
    nq_ref = q[::16].size
    print(f"N=8192 predecessor={predecessor}: device tree {evals / q.size:.0f} distance evaluations per query; "
          f"reference parity mode {ref.last_evals / nq_ref:.0f} child evaluations + "
          f"{ref.last_root_evals / nq_ref:.0f} root distances per query; build {idx.build_info()}")


def test_traversal_d8_mixture_equals_dense(cuda_available):
    case = mixture_case(6000, 8, 128, 2.0)
    idx = _tree_index(case)
    q = np.random.default_rng(4).choice(6000, 600, replace=False)
    ti, td = idx.knn(q, 30, predecessor=True, form="tree")
    di, dd = idx.knn(q, 30, predecessor=True, form="dense")
    assert np.array_equal(ti, di)
    assert np.array_equal(td.view(np.uint32), dd.view(np.uint32))
    for i in range(q.size):
        valid = ti[i][ti[i] >= 0]
        assert np.all(valid < q[i]) and len(valid) == min(30, q[i])


def test_traversal_natural_order_and_duplicates(cuda_available):
    """Natural build order, exact duplicate points (distance 0 pairs, floor level) and a
    long lengthscale (few tiny-p rows): still the dense form's lists."""
    case = gaussian_case(3000, 2, 32, 0, 3.0, seed=9)
    X = case["X"].copy()
    X[1000:1100] = X[0]
    case2 = dict(case)
    case2["X"] = X
    V, p, _, _ = O.build_residual_backend_np(X, seed=42, inducing_count=32, variance=1.0, lengthscale=3.0,
                                             kernel_type=0)
    case2["V"], case2["p"] = V, p
    idx = _tree_index(case2, order="natural")
    q = np.arange(3000)
    for pred in (False, True):
        ti, td = idx.knn(q, 20, predecessor=pred, form="tree")
        di, dd = idx.knn(q, 20, predecessor=pred, form="dense")
        assert np.array_equal(ti, di)
        assert np.array_equal(td.view(np.uint32), dd.view(np.uint32))


def test_extend_grows_the_tree_and_answers_as_a_fresh_build(cuda_available):
    """ct_tree_extend (CoverTree.insert): a handle over the base's 3000 rows plus 1000
    new ones (some of them tiny-p inducing rows, which join the side rows).  The base's
    nodes keep their parents and levels; every form on the grown handle returns the
    fresh build's rows bit for bit (the tree form through its certified prune); the base
    still answers as before."""
    case = gaussian_case(4000, 3, 64, 1, 1.0, seed=18)
    n0 = 3000
    base_case = dict(case, V=case["V"][:n0], p=case["p"][:n0], X=case["X"][:n0])
    base = _tree_index(base_case)
    fresh = _tree_index(case)
    grown = base.extend(case["V"][n0:], case["p"][n0:], case["X"][n0:])
    assert grown.n == 4000 and base.n == n0
    tb, tg = base.tree_arrays(), grown.tree_arrays()
    nt0 = n0 - base.build_info()["side_rows"]
    assert np.array_equal(tg["node_to_dataset"][:nt0], tb["node_to_dataset"][:nt0])
    assert np.array_equal(tg["parents"][:nt0], tb["parents"][:nt0])
    assert np.array_equal(tg["levels"][:nt0], tb["levels"][:nt0])
    assert np.array_equal(np.sort(tg["node_to_dataset"]), np.arange(4000))
    side = case["p"][tg["node_to_dataset"]] < 1.0 / 1024
    assert grown.build_info()["side_rows"] == side.sum()
    assert np.all(tg["parents"][side] < 0)
    q = np.arange(4000)
    for pred in (True, False):
        fi, fd = fresh.knn(q, 30, predecessor=pred, form="dense")
        for form in ("dense", "tree", "screened"):
            gi, gd = grown.knn(q, 30, predecessor=pred, form=form)
            ri, rd = (fi, fd) if form != "screened" else fresh.knn(q, 30, predecessor=pred, form="screened")
            assert np.array_equal(gi, ri), form
            assert np.array_equal(gd.view(np.uint32), rd.view(np.uint32)), form
    bi, bd = base.knn(np.arange(n0), 30, predecessor=True, form="tree")
    oi, od = O.brute_knn_f32(base_case["V"], base_case["p"], base_case["X"], 1.0, base_case["ls"], 1,
                             np.arange(n0), 30, True)
    assert np.array_equal(bi, oi) and np.array_equal(bd.view(np.uint32), od.view(np.uint32))
    for ix in (base, fresh, grown):
        ix.free()


def test_subset_answers_as_a_fresh_build(cuda_available):
    """ct_tree_subset (CoverTree.delete): rows gathered on the device give a handle whose
    every form returns the rows of a fresh build over the same rows, bit for bit; bad
    row lists are rejected."""
    from covertreex_gb300.device import CudaResidualIndex

    case = gaussian_case(3000, 3, 64, 0, 1.5, seed=27)
    base = _tree_index(case)
    keep = np.setdiff1d(np.arange(3000), np.random.default_rng(28).choice(3000, 400, replace=False))
    sub = base.subset(keep)
    fresh = _tree_index(dict(case, V=case["V"][keep], p=case["p"][keep], X=case["X"][keep]))
    q = np.arange(keep.size)
    for form in ("dense", "tree", "screened"):
        a, ad = sub.knn(q, 20, predecessor=True, form=form)
        b, bd = fresh.knn(q, 20, predecessor=True, form=form)
        assert np.array_equal(a, b) and np.array_equal(ad.view(np.uint32), bd.view(np.uint32)), form
    with pytest.raises(Exception):
        base.subset(np.array([5, 3]))          # not ascending
    with pytest.raises(Exception):
        base.subset(np.array([0, 3000]))       # out of range
    for ix in (base, sub, fresh):
        ix.free()
