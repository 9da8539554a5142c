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
