"""Host-side API logic that needs no GPU."""
import numpy as np
import pytest


def test_engine_registry():
    from covertreex_gb300 import engine

    assert engine.get_engine("cuda").name == "cuda"
    assert "cuda" in engine.SUPPORTED_ENGINES
    with pytest.raises(ValueError):
        engine.get_engine("rust-hilbert")


def test_format_knn_output_mirrors_reference():
    from covertreex_gb300.engine import _format_knn_output

    idx = np.arange(6).reshape(2, 3)
    dist = np.ones((2, 3), np.float32)
    assert _format_knn_output(idx, dist, return_distances=False) is idx
    one = _format_knn_output(idx[:1], dist[:1], return_distances=False)
    assert one.shape == (3,)
    a, b = _format_knn_output(idx[:1, :1], dist[:1, :1], return_distances=True)
    assert a == 0 and b == 1.0


def test_kernels_match_reference_formulas():
    from covertreex_gb300.kernels import RBF, Matern52

    x = np.array([[0.0, 0.0]])
    y = np.array([[1.0, 2.0]])
    r2 = 5.0
    assert np.isclose(RBF(lengthscale=2.0, variance=3.0)(x, y)[0, 0], 3.0 * np.exp(-0.5 * r2 / 4.0))
    a = np.sqrt(5.0) * np.sqrt(r2) / 1.5
    assert np.isclose(Matern52(lengthscale=1.5)(x, y)[0, 0], (1 + a + a * a / 3) * np.exp(-a))
    assert RBF().kernel_type == 0 and Matern52().kernel_type == 1


def test_residual_host_data_validation():
    from covertreex_gb300.residual import ResidualCorrHostData

    with pytest.raises(ValueError):
        ResidualCorrHostData(v_matrix=np.zeros((4, 2)), p_diag=np.ones(3), kernel_diag=np.ones(4))


def test_query_sharding_covers_every_query_once():
    import importlib.util
    import pathlib

    spec = importlib.util.spec_from_file_location("bench", pathlib.Path(__file__).resolve().parent.parent / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    for world in (1, 2, 3, 8):
        parts = [bench.shard_queries(1001, world, r) for r in range(world)]
        allq = np.sort(np.concatenate(parts))
        assert np.array_equal(allq, np.arange(1001))


def test_serving_stream_is_seeded_and_shaped():
    from covertreex_gb300.synthetic import serving_stream

    pre, s1 = serving_stream(500.0, 0.2, seed=6, preload=2)
    _, s2 = serving_stream(500.0, 0.2, seed=6, preload=2)
    assert [r.rid for r in s1] == [r.rid for r in s2]
    assert all(a.arrival <= b.arrival for a, b in zip(s1, s1[1:]))
    builds = [r for r in s1 if hasattr(r, "coords")]
    queries = [r for r in s1 if hasattr(r, "points")]
    assert len(pre) == 2 and len(queries) > len(builds)
    for b in pre + builds:
        assert 1024 <= b.coords.shape[0] <= 131072 and b.coords.shape[1] == 3 and b.inducing_count == 256
        assert 0.5 <= b.lengthscale <= 2.0 and b.kernel_type == 1
    known = {b.rid for b in pre + builds}
    for q in queries:
        assert 1 <= q.points.shape[0] <= 4096 and q.k in (30, 50, 60) and q.tree in known


def test_batch_trees_shapes():
    from covertreex_gb300.synthetic import batch_trees

    trees = batch_trees()
    assert len(trees) == 64
    assert all(2048 <= t.n <= 65536 and t.d in (2, 3, 5) and t.m == 128 and t.k in (10, 30, 50) for t in trees)
    assert {t.kernel_type for t in trees} == {0, 1} and {t.predecessor for t in trees} == {False, True}


def test_serving_estimates_and_summary():
    from covertreex_gb300.serving import RequestRecord, estimate_tree_bytes, latency_summary

    assert estimate_tree_bytes(1000, 3, 256) < estimate_tree_bytes(2000, 3, 256) < estimate_tree_bytes(2000, 3, 512)
    recs = [RequestRecord(rid=i, kind="query", arrival=0.001 * i, size=10, done=0.001 * i + 0.002, status="ok",
                          form="dense") for i in range(100)]
    recs.append(RequestRecord(rid=100, kind="query", arrival=0.0, size=5, status="evicted"))
    s = latency_summary(recs)
    assert s["count"] == 100 and s["dropped"] == 1
    assert abs(s["p50_ms"] - 2.0) < 1e-6 and abs(s["p99_ms"] - 2.0) < 1e-6


def test_serving_latency_by_size():
    from covertreex_gb300.serving import RequestRecord, latency_by_size

    recs = [RequestRecord(rid=i, kind="query", arrival=0.0, size=size, done=ms / 1e3, status="ok", form="dense")
            for i, (size, ms) in enumerate([(1, 1.0), (8, 2.0), (300, 5.0), (4096, 9.0), (2000, 7.0)])]
    recs.append(RequestRecord(rid=9, kind="query", arrival=0.0, size=20, status="evicted"))
    recs.append(RequestRecord(rid=10, kind="build", arrival=0.0, size=5000, done=0.5, status="ok"))
    b = latency_by_size(recs)
    assert [x["size"] for x in b] == ["1-15", "256-1023", "1024-4096"]  # the evicted 20-point request is not counted
    assert [x["count"] for x in b] == [2, 1, 2]
    assert abs(b[0]["max_ms"] - 2.0) < 1e-9 and abs(b[2]["p50_ms"] - 8.0) < 1e-9 and abs(b[2]["max_ms"] - 9.0) < 1e-9


def test_runtime_api_host_checks():
    import pytest as _pytest

    from covertreex_gb300 import CoverTree, Residual, Runtime, api

    rt = Runtime(backend="numpy", precision="float32", metric="residual_correlation", enable_rust=True,
                 engine="rust-natural", residual_use_static_euclidean_tree=True, residual=Residual(radius_floor=1e-3))
    assert rt.is_residual and rt.with_updates(metric="euclidean").is_residual is False
    with _pytest.raises(RuntimeError):
        CoverTree(rt).knn(np.array([[0]]), k=1)       # not fitted
    with _pytest.raises(ValueError):
        CoverTree(rt).fit(np.zeros((0, 2)))           # no points
    with _pytest.raises(ValueError):
        CoverTree(Runtime(engine="no-such-engine")).fit(np.zeros((4, 2), np.float32))
    api.reset_residual_correlation()
    with _pytest.raises(RuntimeError):
        api.get_residual_backend()
    with _pytest.raises(ValueError):
        api.configure_residual_correlation(None)


def test_telemetry_formats(tmp_path):
    import json as _json

    from covertreex_gb300.telemetry import (BENCHMARK_BATCH_REQUIRED, BENCHMARK_BATCH_SCHEMA_ID,
                                            BatchTelemetryWriter, query_telemetry)

    # the field names of ResidualQueryTelemetry (src/telemetry.rs)
    fields = ["frontier_levels", "frontier_expanded", "yields", "caps_applied", "prunes_lower_bound",
              "prunes_lower_bound_chunks", "prunes_cap", "masked_dedup", "distance_evals", "budget_escalations",
              "budget_early_terminate", "level_cache_hits", "level_cache_misses", "block_sizes",
              "predecessor_filtered", "subtrees_pruned"]
    t = query_telemetry({"distance_evals": 42, "pairs_screened": 7, "device_ms": 1.5}, "screened")
    assert all(f in t for f in fields) and t["distance_evals"] == 42 and t["gpu"]["pairs_screened"] == 7
    w = BatchTelemetryWriter(tmp_path / "t.jsonl", runtime={"engine": "cuda", "metric": "residual_correlation"})
    w.record(batch_index=0, batch_size=512, measurements={"build_seconds": 0.01}, metadata={"n": 4096})
    w.record(batch_index=1, batch_size=100, measurements={"queries_per_s": 1e6})
    rows = [_json.loads(x) for x in (tmp_path / "t.jsonl").read_text().splitlines()]
    assert [r["batch_event_index"] for r in rows] == [0, 1]
    for r in rows:
        assert all(k in r for k in BENCHMARK_BATCH_REQUIRED) and r["schema_id"] == BENCHMARK_BATCH_SCHEMA_ID
    assert rows[0]["build_seconds"] == 0.01 and rows[1]["queries_per_s"] == 1e6
