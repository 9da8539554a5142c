"""Serving form (covertreex_gb300.serving): resident trees, HBM-budget admission,
continuous batching of new-point query requests.  Every query result must be the
same whether the request ran in the mix or alone, and correct against the oracle:
dense-form requests bit-exact to the f32 oracle, screened-form requests within
1e-5 of FP64 brute force with only listed near-ties (FP64 gap < 1e-6)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _stream(n_queries=40, seed=9):
    from covertreex_gb300.serving import BuildRequest, QueryRequest

    r = np.random.default_rng(seed)
    pre = []
    for j, n in enumerate((3000, 12000, 40000)):
        X = np.random.default_rng(50 + j).standard_normal((n, 3)).astype(np.float32)
        pre.append(BuildRequest(rid=j, arrival=0.0, coords=X, kernel_type=1, lengthscale=0.5 + 0.6 * j,
                                inducing_count=256, seed=17 + j))
    qs = []
    for i in range(n_queries):
        q = int(r.choice([1, 3, 17, 64, 300, 1500]))
        qs.append(QueryRequest(rid=10 + i, arrival=0.0005 * i, tree=int(r.integers(0, 3)),
                               points=r.standard_normal((q, 3)).astype(np.float32), k=int(r.choice([30, 50, 60]))))
    return pre, qs


def test_serving_mix_equals_alone_and_oracle(cuda_available):
    from covertreex_gb300.serving import ServingEngine, latency_summary

    pre, qs = _stream()
    eng = ServingEngine(hbm_budget_bytes=8e9, dense_pair_limit=2e8)
    try:
        eng.preload(pre)
        recs = eng.serve(qs, realtime=False)  # everything admitted at once: large mixed steps
        assert all(r.status == "ok" for r in recs)
        forms = {r.form for r in recs}
        assert forms == {"dense", "screened"}
        s = latency_summary(recs)
        assert s["count"] == len(qs) and s["dropped"] == 0
        by = {q.rid: q for q in qs}
        for rec in recs[::3]:
            alone = eng.serve([by[rec.rid]], realtime=False)[0]
            assert alone.form == rec.form
            assert np.array_equal(alone.result[0], rec.result[0]) and np.array_equal(alone.result[1], rec.result[1])
        # correctness of a few requests of each form against the oracle
        trees = {b.rid: b for b in pre}
        checked = {"dense": 0, "screened": 0}
        for rec in recs:
            if checked[rec.form] >= 3:
                continue
            q = by[rec.rid]
            b = trees[q.tree]
            t = eng.trees[q.tree]
            V, p = t.factor.embed(b.coords.astype(np.float64))
            qv, qp = t.factor.embed(q.points.astype(np.float64))
            ls = np.full(3, b.lengthscale, np.float32)
            if rec.form == "dense":
                ref = O.brute_knn_points_f32(V, p, b.coords, 1.0, ls, 1, qv, qp, q.points, q.k)
                assert np.array_equal(rec.result[0], ref[0]) and np.array_equal(rec.result[1], ref[1])
            else:
                n = b.coords.shape[0]
                Va, pa, Xa = np.vstack([V, qv]), np.concatenate([p, qp]), np.vstack([b.coords, q.points])
                rows = np.arange(n, n + min(q.points.shape[0], 64))
                ri, rd = O.brute_knn_f64(Va, pa, Xa, 1.0, ls, 1, rows, q.k, False, cand_limit=n)
                got_i, got_d = rec.result[0][: rows.size], rec.result[1][: rows.size]
                assert np.max(np.abs(got_d.astype(np.float64) - rd)) <= 1e-5
                _, mism = O.near_tie_mismatches(got_i, ri, lambda r_, ids: O.residual_dist_f64(
                    Va, pa, Xa, 1.0, ls, 1, [rows[r_]], ids)[0])
                assert all(g < 1e-6 for *_, g in mism)
            checked[rec.form] += 1
        assert checked["dense"] >= 1 and checked["screened"] >= 1
        # the per-request baseline (dense only) agrees with the dense requests of the mix
        base = eng.serve_per_request([by[r.rid] for r in recs if r.form == "dense"][:5], realtime=False)
        dense_recs = [r for r in recs if r.form == "dense"][:5]
        for a, b_ in zip(base, dense_recs):
            assert np.array_equal(a.result[0], b_.result[0]) and np.array_equal(a.result[1], b_.result[1])
    finally:
        eng.close()


def test_serving_budget_admission_and_eviction(cuda_available):
    from covertreex_gb300.serving import BuildRequest, QueryRequest, ServingEngine, estimate_tree_bytes

    X = [np.random.default_rng(70 + j).standard_normal((n, 3)).astype(np.float32)
         for j, n in enumerate((4000, 4000, 4000, 200000))]
    est = estimate_tree_bytes(4000, 3, 256)
    eng = ServingEngine(hbm_budget_bytes=2.0 * est, dense_pair_limit=1e12)
    try:
        eng.preload([BuildRequest(rid=0, arrival=0.0, coords=X[0], seed=1)])
        pts = np.random.default_rng(1).standard_normal((8, 3)).astype(np.float32)
        reqs = [
            BuildRequest(rid=1, arrival=0.000, coords=X[1], seed=2),
            QueryRequest(rid=2, arrival=0.001, tree=0, points=pts, k=30),
            BuildRequest(rid=3, arrival=0.002, coords=X[2], seed=3),     # over budget: evicts the LRU idle tree
            BuildRequest(rid=4, arrival=0.003, coords=X[3], seed=4),     # larger than the whole budget: rejected
            QueryRequest(rid=5, arrival=0.004, tree=3, points=pts, k=30),
            QueryRequest(rid=6, arrival=0.005, tree=4, points=pts, k=30),
        ]
        recs = {r.rid: r for r in eng.serve(reqs, realtime=True)}
        assert recs[1].status == "ok" and recs[3].status == "ok"
        assert recs[4].status == "rejected"
        assert recs[2].status == "ok" and recs[5].status == "ok"
        assert recs[6].status != "ok"
        assert eng.peak_bytes <= eng.budget
        assert len(eng.evicted) >= 1
    finally:
        eng.close()
