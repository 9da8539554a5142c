"""Tree persistence and query telemetry of the GPU index."""
import numpy as np
import pytest

from tests._data import gaussian_case

pytestmark = pytest.mark.gpu


def test_save_load_roundtrip(cuda_available, tmp_path):
    from covertreex_gb300.device import CudaResidualIndex

    c = gaussian_case(3000, 3, 64, 1, 1.0, seed=12)
    a = CudaResidualIndex(c["V"], c["p"], c["X"], variance=1.0, lengthscale=1.0, kernel_type=1, seed=5,
                          build_tree=True)
    path = tmp_path / "tree.ctx"
    a.save(path)
    b = CudaResidualIndex.load(path)
    ta, tb = a.tree_arrays(), b.tree_arrays()
    for key in ta:
        assert np.array_equal(ta[key], tb[key]), key
    q = np.arange(0, 3000, 13)
    for form in ("dense", "tree", "screened"):
        ia, da = a.knn(q, 20, predecessor=True, form=form)
        ib, db = b.knn(q, 20, predecessor=True, form=form)
        assert np.array_equal(ia, ib) and np.array_equal(da, db), form


def test_query_telemetry_fields(cuda_available):
    from covertreex_gb300.device import CudaResidualIndex

    c = gaussian_case(2000, 3, 64, 1, 1.0, seed=3)
    a = CudaResidualIndex(c["V"], c["p"], c["X"], variance=1.0, lengthscale=1.0, kernel_type=1, build_tree=True)
    assert a.last_query_telemetry() is None
    a.knn(np.arange(100), 10, predecessor=False, form="tree")
    t = a.last_query_telemetry()
    assert t["distance_evals"] > 0 and t["gpu"]["form"] == "tree"
    a.knn(np.arange(100), 10, predecessor=False, form="screened")
    t = a.last_query_telemetry()
    assert t["gpu"]["pairs_screened"] > 0 and t["gpu"]["form"] == "screened"
    a.clear_last_query_telemetry()
    assert a.last_query_telemetry() is None
