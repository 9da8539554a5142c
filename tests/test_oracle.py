"""CPU tests of the oracle (no GPU): golden vectors produced by the reference's
own Python code (tests/golden/gen_golden.py) and the reference's test
assertions restated for the C restatement of the Rust crate."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case, mixture_case

GOLD = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def test_residual_backend_matches_reference_python():
    g = np.load(GOLD / "residual_backend.npz")
    for i, (kt, ls, m) in enumerate(g["meta"]):
        X = g[f"X{i}"]
        V, p, _, _ = O.build_residual_backend_np(X, seed=42, inducing_count=int(m), variance=1.0,
                                                 lengthscale=float(ls), kernel_type=int(kt))
        assert V.shape == g[f"V{i}"].shape
        np.testing.assert_allclose(V, g[f"V{i}"], rtol=0, atol=2e-6)
        np.testing.assert_allclose(p, g[f"p{i}"], rtol=1e-5, atol=1e-7)


def test_product_host_backend_matches_reference_python():
    from covertreex_gb300.residual import build_residual_backend

    g = np.load(GOLD / "residual_backend.npz")
    for i, (kt, ls, m) in enumerate(g["meta"]):
        hb = build_residual_backend(g[f"X{i}"], seed=42, inducing_count=int(m), variance=1.0, lengthscale=float(ls),
                                    kernel_type=int(kt), device="host")
        np.testing.assert_allclose(hb.v_matrix, g[f"V{i}"], rtol=0, atol=2e-6)
        np.testing.assert_allclose(hb.p_diag, g[f"p{i}"], rtol=1e-5, atol=1e-7)


def test_luby_mis_matches_reference_python():
    g = np.load(GOLD / "mis.npz")
    for i in range(4):
        sel, it = O.luby_mis(g[f"indptr{i}"], g[f"indices{i}"], int(g[f"seed{i}"]))
        assert np.array_equal(sel, g[f"sel{i}"]), i
        assert it == int(g[f"iters{i}"])


def test_mis_is_maximal_independent():
    g = np.load(GOLD / "mis.npz")
    for i in range(4):
        ip, ix = g[f"indptr{i}"], g[f"indices{i}"]
        sel, _ = O.luby_mis(ip, ix, 3)
        n = ip.size - 1
        for v in range(n):
            nb = ix[ip[v]:ip[v + 1]]
            if sel[v]:
                assert not sel[nb].any()
            else:
                assert sel[nb].any() or nb.size == 0 and False


def test_hilbert_order_matches_reference_python():
    g = np.load(GOLD / "hilbert.npz")
    for i in range(4):
        perm, _ = O.hilbert_order(g[f"P{i}"])
        assert np.array_equal(perm, g[f"perm{i}"]), i


def test_prefix_slices_match_reference_python():
    g = np.load(GOLD / "prefix.npz")
    for i in range(9):
        assert [tuple(s) for s in g[f"slices{i}"].tolist()] == O.prefix_slices(int(g[f"len{i}"]))


def test_distance_formula_matches_reference_python():
    """Oracle f32 distance vs the reference's f64 formula (compute_distance_chunk) fed with
    its own f32 SGEMM kernel values.  The tolerance scales with 1/sqrt(p_q p_c): both sides
    round K and the dot product to f32 before the p-normalisation."""
    g = np.load(GOLD / "distance.npz")
    X, V, p, ref = g["X"], g["V"], g["p"], g["dist"]
    qi = np.repeat(np.arange(20), 150)
    cj = np.tile(np.arange(150), 20)
    got = O.pair_dist_f32(V, p, X, 1.0, [1.0] * 3, 0, qi, cj).reshape(20, 150)
    scale = 1.0 / np.sqrt(np.maximum(p[:20, None].astype(np.float64) * p[None, :].astype(np.float64), 1e-18))
    dref = ref.copy()
    for q in range(20):
        dref[q, q] = 0.0  # the f32 batch path returns 0 for the query itself
    err = np.abs(got - dref)
    tol = 2e-3 + 1e-6 * scale
    assert np.all(err <= tol), float((err - tol).max())
    good = scale < 1e3
    assert np.abs(got - dref)[good].max() < 1e-3


def test_expf_within_one_ulp():
    L = O.lib()
    xs = np.concatenate([np.linspace(-86.9, 88.0, 20001), np.linspace(-1, 1, 4001)]).astype(np.float32)
    got = np.array([L.ct_expf(float(x)) for x in xs], dtype=np.float32)
    ref = np.exp(xs.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(got - ref) <= 1.0 * ulp)


def test_dot_order_restatement():
    """dot_f32_simd_inline order: 16 lane sums, lane combine, fixed horizontal tree."""
    L = O.lib()
    r = np.random.default_rng(0)
    for m in (16, 48, 64, 100, 256):
        a = r.standard_normal(m).astype(np.float32)
        b = r.standard_normal(m).astype(np.float32)
        ch = m // 8
        acc0 = np.zeros(8, np.float32)
        acc1 = np.zeros(8, np.float32)
        i = 0
        for _ in range(ch // 2):
            acc0 = (a[i:i + 8] * b[i:i + 8]) + acc0
            acc1 = (a[i + 8:i + 16] * b[i + 8:i + 16]) + acc1
            i += 16
        if ch % 2:
            acc0 = (a[i:i + 8] * b[i:i + 8]) + acc0
        c = acc0 + acc1
        s = c[:4] + c[4:]
        res = (s[0] + s[2]) + (s[1] + s[3])
        for j in range(ch * 8, m):
            res = np.float32(res + a[j] * b[j])
        got = L.ct_dot_simd_inline(a.ctypes.data_as(O._f32p), b.ctypes.data_as(O._f32p), m)
        assert np.float32(got) == np.float32(res)


def test_morton_known_answer():
    L = O.lib()

    def interleave(x, y, z):
        code = 0
        for bit in range(21):
            code |= ((x >> bit) & 1) << (3 * bit)
            code |= ((y >> bit) & 1) << (3 * bit + 1)
            code |= ((z >> bit) & 1) << (3 * bit + 2)
        return code

    r = np.random.default_rng(1)
    for _ in range(200):
        x, y, z = (int(v) for v in r.integers(0, 1 << 21, 3))
        assert L.ct_morton3(x, y, z) == interleave(x, y, z)


def test_morton_order_is_stable_sort_of_codes():
    X = np.random.default_rng(2).standard_normal((1000, 3)).astype(np.float32)
    order, codes = O.morton_order(X)
    assert np.array_equal(order, np.lexsort((np.arange(1000), codes)))
    X2 = np.random.default_rng(2).standard_normal((100, 5)).astype(np.float32)
    o2, _ = O.morton_order(X2)
    assert np.array_equal(o2, np.arange(100))  # D != 3 -> natural order (src/pcct.rs:33-35)


def test_subtree_bounds_relaxation():
    parents = np.array([-1, 0, 0, 1, 1, 2, -1], np.int64)
    n2d = np.array([5, 3, 9, 1, 7, 0, 4], np.int64)
    mn, mx = O.subtree_bounds(parents, n2d)
    assert mn.tolist() == [0, 1, 0, 1, 7, 0, 4]
    assert mx.tolist() == [9, 7, 9, 1, 7, 0, 4]


@pytest.fixture(scope="module")
def small_tree():
    case = gaussian_case(600, 3, 32, 1, 1.0, seed=3)
    T = O.OracleResidualTree(case["V"], case["p"], case["X"], 1.0, case["ls"], kernel_type=1, chunk=128, parity=True)
    return case, T


def test_oracle_predecessor_invariants(small_tree):
    """tests/test_predecessor_mode.py:26-120 of the reference, on the restated Rust path."""
    case, T = small_tree
    q = np.arange(600)
    oi, od = T.knn(q, 10, predecessor=True)
    for i in range(600):
        valid = oi[i][oi[i] >= 0]
        assert np.all(valid < i)
        assert len(valid) == min(10, i)
    assert np.all(oi[0] == -1)
    assert list(oi[1][oi[1] >= 0]) == [0]


def test_oracle_output_contract(small_tree):
    """Shape/dtype/padding contract (reference tests/test_rust_residual_dtype.py:10-64, src/lib.rs:907-938)."""
    case, T = small_tree
    oi, od = T.knn(np.array([0, 1, 2]), 700, predecessor=False)
    assert oi.shape == (3, 700) and oi.dtype == np.int64 and od.dtype == np.float32
    assert (oi[:, 600:] == -1).all() and (od[:, 600:] == np.float32(3.402823466e38)).all()
    assert np.all(np.diff(od[:, :600], axis=1) >= 0)


def test_oracle_parity_traversal_agrees_with_brute(small_tree):
    """Parity-mode traversal vs exhaustive f32 brute force.  The traversal scores roots
    with the scalar path (f64-accumulated dot in parity mode, src/metric.rs:489-563), the
    brute force with the batch path.  Disagreements are confined to queries whose residual
    variance p_q is tiny (the inducing rows, p ~ 1e-6), where 1-|rho| cancels in f32 and
    the two paths round differently; well-conditioned rows agree up to boundary swaps."""
    case, T = small_tree
    q = np.arange(600)
    p = case["p"]
    for pred in (False, True):
        oi, od = T.knn(q, 10, predecessor=pred)
        bi, bd = O.brute_knn_f32(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, q, 10, pred)
        bad = [r for r in range(600) if set(oi[r]) != set(bi[r])]
        well = [r for r in bad if p[r] >= 1e-3]
        for r in well:
            kth = bd[r][bi[r] >= 0].max()
            extra = np.setdiff1d(oi[r], bi[r])
            dd = O.pair_dist_f32(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, np.full(extra.size, r), extra)
            assert np.all(dd - kth < 1e-3)
        assert len(well) <= 3


def test_oracle_default_mode_runs(small_tree):
    case, T = small_tree
    oi, od = T.knn(np.arange(50), 10, predecessor=False, parity=False)
    assert oi.shape == (50, 10) and (oi[:, 0] >= 0).all()


def test_oracle_f32_brute_matches_fp64_when_well_conditioned():
    case = gaussian_case(400, 3, 16, 1, 1.0, seed=4)
    q = np.arange(400)
    bi, bd = O.brute_knn_f32(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, q, 8, False)
    fi, fd = O.brute_knn_f64(case["V"], case["p"], case["X"], 1.0, case["ls"], 1, q, 8, False)
    # rows with p_q >= 0.05 are well conditioned: f32 within 5e-5 of FP64 and identical sets;
    # the inducing rows (p ~ 1e-6) cancel catastrophically in f32 (1 - |rho|).
    good = case["p"] >= 0.05
    assert good.mean() > 0.9
    assert np.abs(bd.astype(np.float64) - fd)[good].max() < 5e-5
    assert all(set(a) == set(b) for a, b, g in zip(bi, fi, good) if g)


def test_euclidean_oracle_restatement():
    """Euclidean batch insert + best-first kNN (src/algo.rs:179-323).  The reference prunes
    with 2^(level+1), which its greedy batch insert does not guarantee as a cover radius, so
    the search is approximate: returned distances are exact for the returned ids, recall
    is high but below 1.  The engine's Euclidean kNN is exact and is checked against FP64."""
    X = np.random.default_rng(6).standard_normal((700, 3)).astype(np.float32)
    T = O.OracleEuclideanTree(X, chunk=128)
    oi, od = T.knn(X, 10)
    fi, fd = O.brute_knn_euclidean_f64(X, X, 10)
    recall = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(oi, fi)])
    assert recall > 0.95
    true_d = np.sqrt(((X[:, None, :].astype(np.float64) - X[oi].astype(np.float64)) ** 2).sum(-1))
    assert np.abs(od - true_d).max() < 1e-5


@pytest.mark.parametrize("predecessor", [False, True])
def test_fp64_brute_c_matches_numpy(predecessor):
    """The blocked C FP64 brute force (used at the full benchmark shapes) returns the
    numpy FP64 brute force's rows: same ids, distances within FP64 summation-order noise
    (the inducing rows divide by sqrt(p_q p_c) ~ 1e-6, which scales that noise up)."""
    case = mixture_case(3000, 8, 128, 2.0)
    q = np.random.default_rng(7).choice(3000, 333, replace=False)
    a_i, a_d = O.brute_knn_f64(case["V"], case["p"], case["X"], 1.0, case["ls"], 0, q, 30, predecessor)
    b_i, b_d = O.brute_knn_f64_c(case["V"], case["p"], case["X"], 1.0, case["ls"], 0, q, 30, predecessor)
    assert np.array_equal(a_i, b_i)
    fin = np.isfinite(a_d)
    assert np.array_equal(fin, np.isfinite(b_d))
    assert np.abs(a_d[fin] - b_d[fin]).max() < 1e-9


def _reference_knn_cases():
    g = np.load(Path(__file__).resolve().parent / "golden" / "residual_knn.npz")
    for ci in range(4):
        kt, ls, k, pred = g[f"meta{ci}"]
        yield dict(X=g[f"X{ci}"], V=g[f"V{ci}"], p=g[f"p{ci}"], kt=int(kt), ls=float(ls), k=int(k),
                   pred=bool(pred), idx=g[f"idx{ci}"], dist=g[f"dist{ci}"])


def test_oracle_brute_forces_match_reference_knn():
    """Neighbour sets of the reference's own Python residual kNN
    (covertreex/queries/residual_knn.py:249-386, exhaustive on a flat tree; golden vectors).
    Where the query's residual variance is not tiny (p >= 1e-3) the FP64 and f32 brute
    forces return exactly the reference's sets.  On the inducing rows (p ~ 1e-6) the
    reference's f32 kernel provider decides 1 - |rho| by rounding noise (its distances
    there are off by up to 0.3), so only the number of neighbours is compared."""
    for c in _reference_knn_cases():
        n, d = c["X"].shape
        q = np.arange(n)
        good = c["p"] >= 1e-3
        assert good.mean() > 0.75
        for fn in (O.brute_knn_f64, O.brute_knn_f32):
            gi, _ = fn(c["V"], c["p"], c["X"], 1.0, [c["ls"]] * d, c["kt"], q, c["k"], c["pred"])
            assert np.array_equal(gi >= 0, c["idx"] >= 0)
            same = np.array([set(a[a >= 0]) == set(b[b >= 0]) for a, b in zip(gi, c["idx"])])
            assert same[good].all()
        # the reference's distances agree with FP64 to its own f32 rounding on those rows
        fi, fd = O.brute_knn_f64(c["V"], c["p"], c["X"], 1.0, [c["ls"]] * d, c["kt"], q, c["k"], c["pred"])
        v = (c["idx"] >= 0) & good[:, None]
        assert np.abs(np.sort(np.where(v, c["dist"], 0), 1) - np.sort(np.where(v, fd, 0), 1)).max() < 5e-3
