"""Batching form (ct_batch_*): many trees and query sets of uneven N, D, m and k in
one persistent launch.  Every query set must come out bit-identical to the oracle's
f32 brute force (the reference's batch-path arithmetic, ties to the lower index),
whatever the launch shape, the candidate split, the graph replay or the other query
sets in the batch."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (n, d, m, kernel_type, lengthscale, k, predecessor)
TREES = [
    (700, 2, 64, 1, 0.8, 10, False),
    (2048, 3, 128, 0, 1.3, 30, True),
    (3001, 5, 64, 1, 1.0, 50, False),
    (5000, 3, 128, 0, 0.6, 50, True),
    (1500, 2, 128, 1, 2.0, 30, True),
]


def _trees():
    from covertreex_gb300.device import CudaResidualIndex

    out = []
    for t, (n, d, m, kt, ls, k, pred) in enumerate(TREES):
        X = np.random.default_rng(100 + t).standard_normal((n, d)).astype(np.float32)
        V, p, _, _ = O.build_residual_backend_np(X, seed=7 + t, inducing_count=m, variance=1.0, lengthscale=ls,
                                                 kernel_type=kt)
        idx = CudaResidualIndex(V, p, X, variance=1.0, lengthscale=ls, kernel_type=kt, build_tree=False)
        r = np.random.default_rng(200 + t)
        q = np.concatenate([[0, 1, n - 1], r.choice(n, size=min(n - 3, 257), replace=False)]).astype(np.int64)
        ref = O.brute_knn_f32(V, p, X, 1.0, np.full(d, ls, np.float32), kt, q, k, pred)
        out.append(dict(X=X, V=V, p=p, ls=ls, kt=kt, k=k, pred=pred, index=idx, q=q, ref=ref))
    return out


@pytest.fixture(scope="module")
def trees(cuda_available):
    return _trees()


def _run(trees, shape=None, use_graph=False, reps=1, batch=None):
    from covertreex_gb300.device import CudaBatch

    b = batch or CudaBatch()
    b.clear()
    if shape:
        b.set_shape(*shape)
    outs = [b.add_ids(t["index"], t["q"], t["k"], predecessor=t["pred"]) for t in trees]
    for _ in range(reps):
        b.run(use_graph=use_graph)
    return b, [(i.cpu().numpy(), d.cpu().numpy()) for i, d in outs]


def _assert_exact(trees, res):
    for t, (i, d) in zip(trees, res):
        assert np.array_equal(i, t["ref"][0])
        assert np.array_equal(d, t["ref"][1])


def test_batch_matches_oracle(trees):
    b, res = _run(trees)
    _assert_exact(trees, res)
    assert b.last_stats["kernel_launches"] == 1


def test_batch_matches_single_tree_dense(trees):
    _, res = _run(trees)
    for t, (i, d) in zip(trees, res):
        si, sd = t["index"].knn(t["q"], t["k"], predecessor=t["pred"], form="dense")
        assert np.array_equal(i, si) and np.array_equal(d, sd)


@pytest.mark.parametrize("shape", [(64, 1, 1), (32, 1, 4), (16, 1, 16), (16, 2, 64), (64, 1, 64)])
def test_batch_shapes_and_candidate_split(trees, shape):
    b, res = _run(trees, shape=shape)
    _assert_exact(trees, res)
    sh = b.shape()
    assert sh["qt"] == shape[0] and sh["items"] >= sum((len(t["q"]) + shape[0] - 1) // shape[0] for t in trees)


def test_batch_graph_replay_and_reuse(trees):
    # replays of one graph: the queue and tile counters must return to zero each time
    b, res = _run(trees, shape=(16, 1, 16), use_graph=True, reps=3)
    _assert_exact(trees, res)
    # the same graph serves a different batch (fewer query sets, other outputs)
    _, res2 = _run(trees[::-1][:3], shape=(16, 1, 16), use_graph=True, reps=2, batch=b)
    _assert_exact(trees[::-1][:3], res2)


def test_batch_edge_queries(trees):
    from covertreex_gb300.device import CudaBatch

    t = trees[1]
    n = t["X"].shape[0]
    b = CudaBatch()
    q_bad = np.array([-1, n, n + 100], dtype=np.int64)
    i0, d0 = b.add_ids(t["index"], q_bad, 5)
    i1, d1 = b.add_ids(t["index"], np.zeros(0, np.int64), 5)  # empty query set
    i2, d2 = b.add_ids(t["index"], np.array([0, 1], np.int64), 5, predecessor=True)
    b.set_shape(16, 1, 32)
    b.run()
    assert np.all(i0.cpu().numpy() == -1) and np.all(d0.cpu().numpy() == np.float32(3.402823466e38))
    assert i1.shape == (0, 5)
    r2 = i2.cpu().numpy()
    assert np.all(r2[0] == -1)  # query 0 has no predecessors
    assert r2[1, 0] == 0 and np.all(r2[1, 1:] == -1)


def test_batch_autotune_keeps_results(trees):
    from covertreex_gb300.device import CudaBatch

    b = CudaBatch()
    outs = [b.add_ids(t["index"], t["q"], t["k"], predecessor=t["pred"]) for t in trees]
    shape = b.autotune(reps=1)
    assert shape["qt"] in (16, 32, 64) and shape["ctas_per_sm"] in (1, 2) and shape["items_per_slot"] > 0
    b.run(use_graph=True)
    _assert_exact(trees, [(i.cpu().numpy(), d.cpu().numpy()) for i, d in outs])


def test_new_points_alone_and_in_the_mix(trees):
    """Serving queries: new points against resident trees, bit-exact to the oracle,
    and identical whether a query set runs alone or batched with others."""
    from covertreex_gb300.device import CudaBatch, CudaVFactor

    pts = []
    for j, t in enumerate(trees[:3]):
        n, d = t["X"].shape
        _, _, ind, _ = O.build_residual_backend_np(t["X"], seed=7 + j, inducing_count=t["V"].shape[1],
                                                   variance=1.0, lengthscale=t["ls"], kernel_type=t["kt"])
        f = CudaVFactor(t["X"][ind].astype(np.float64), kernel_type=t["kt"], variance=1.0, lengthscale=t["ls"])
        Xq = np.random.default_rng(300 + j).standard_normal((37 + 50 * j, d)).astype(np.float32)
        qv, qp = f.embed(Xq.astype(np.float64))
        f.free()
        ref = O.brute_knn_points_f32(t["V"], t["p"], t["X"], 1.0, np.full(d, t["ls"], np.float32), t["kt"],
                                     qv, qp, Xq, t["k"])
        pts.append((t, qv, qp, Xq, ref))
    alone = []
    for t, qv, qp, Xq, ref in pts:
        i, d = t["index"].knn_points_device(qv, qp, Xq, t["k"])
        i, d = i.cpu().numpy(), d.cpu().numpy()
        assert np.array_equal(i, ref[0]) and np.array_equal(d, ref[1])
        alone.append((i, d))
    b = CudaBatch()
    b.set_shape(16, 1, 16)
    mixed = [b.add_points(t["index"], qv, qp, Xq, t["k"]) for t, qv, qp, Xq, _ in pts]
    ids = [b.add_ids(t["index"], t["q"], t["k"], predecessor=t["pred"]) for t in trees]
    b.run(use_graph=True)
    for (i, d), (ai, ad) in zip(mixed, alone):
        assert np.array_equal(i.cpu().numpy(), ai) and np.array_equal(d.cpu().numpy(), ad)
    _assert_exact(trees, [(i.cpu().numpy(), d.cpu().numpy()) for i, d in ids])
