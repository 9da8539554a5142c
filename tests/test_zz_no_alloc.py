"""The allocation-free entry point ct_knn_residual_dense_noalloc.

It serves callers that cannot allocate device memory (their framework owns all
GPU memory, or their loop cannot afford cudaMalloc's synchronisation): its
scratch is a fixed 64 MiB array inside the library.  This file runs last so a
stop-at-first-failure run has already exercised everything else; it must pass
both alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests._data import gaussian_case

pytestmark = pytest.mark.gpu


def _noalloc(L, case, q, k, predecessor, torch, stream):
    dev = torch.device("cuda")
    v = torch.as_tensor(case["V"], device=dev)
    p = torch.as_tensor(case["p"], device=dev)
    c = torch.as_tensor(case["X"], device=dev)
    qd = torch.as_tensor(np.asarray(q, np.int64), device=dev)
    oi = torch.empty((qd.numel(), k), dtype=torch.int64, device=dev)
    od = torch.empty((qd.numel(), k), dtype=torch.float32, device=dev)
    ls = (ctypes.c_float * len(case["ls"]))(*[float(x) for x in case["ls"]])
    n, m = case["V"].shape
    rc = L.ct_knn_residual_dense_noalloc(v.data_ptr(), p.data_ptr(), c.data_ptr(), n, m, case["X"].shape[1],
                                         float(case["var"]), ls, len(case["ls"]), int(case["kt"]), qd.data_ptr(),
                                         qd.numel(), k, 1 if predecessor else 0, oi.data_ptr(), od.data_ptr(),
                                         ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return rc, oi.cpu().numpy(), od.cpu().numpy()


def _reference_call(case, q, k, predecessor):
    from covertreex_gb300.device import CudaResidualIndex

    idx = CudaResidualIndex(case["V"], case["p"], case["X"], variance=case["var"], lengthscale=case["ls"],
                            kernel_type=case["kt"], build_tree=False)
    return idx.knn(q, k, predecessor=predecessor, form="dense")


def test_noalloc_matches_dense_entry_point_twice_in_a_row(cuda_available):
    import torch

    from covertreex_gb300 import _lib

    L = _lib.load()
    stream = torch.cuda.current_stream()
    a = gaussian_case(3000, 3, 64, 1, 1.0, seed=21)
    b = gaussian_case(2500, 2, 32, 0, 0.8, seed=22)
    qa = np.arange(3000)
    qb = np.random.default_rng(5).choice(2500, 700, replace=False)
    rc, ia, da = _noalloc(L, a, qa, 20, True, torch, stream)
    assert rc == 0, L.ct_last_error()
    rc, ib, db = _noalloc(L, b, qb, 16, False, torch, stream)
    assert rc == 0, L.ct_last_error()
    ra_i, ra_d = _reference_call(a, qa, 20, True)
    rb_i, rb_d = _reference_call(b, qb, 16, False)
    # same kernel, same arithmetic: bit-exact (tolerance 0)
    assert np.array_equal(ia, ra_i) and np.array_equal(da.view(np.uint32), ra_d.view(np.uint32))
    assert np.array_equal(ib, rb_i) and np.array_equal(db.view(np.uint32), rb_d.view(np.uint32))
    # and, independently of the dense entry point, bit-exact against the CPU oracle's
    # f32 brute force (the reference's batch-path distance)
    for case, q, k, pred, gi, gd in ((a, qa, 20, True, ia, da), (b, qb, 16, False, ib, db)):
        oi, od = O.brute_knn_f32(case["V"], case["p"], case["X"], case["var"], case["ls"], case["kt"], q, k, pred)
        assert np.array_equal(gi, oi) and np.array_equal(gd.view(np.uint32), od.view(np.uint32))


def _bytes_needed(n, m, d):
    """The documented scratch rule: five pieces, each rounded up to 256 bytes."""
    a = lambda x: (x + 255) // 256 * 256  # noqa: E731
    return a(4 * n * m) + a(4 * n * d) + a(4 * n) + a(4 * n) + 256


def test_noalloc_accepts_the_largest_input_and_rejects_one_row_more(cuda_available):
    import torch

    from covertreex_gb300 import _lib

    L = _lib.load()
    m, d = 64, 3
    n = 243145
    assert _bytes_needed(n, m, d) == _lib.CT_NOALLOC_SCRATCH_BYTES < _bytes_needed(n + 1, m, d)
    r = np.random.default_rng(9)
    case = {"V": (0.1 * r.standard_normal((n + 1, m))).astype(np.float32),
            "p": r.uniform(0.05, 1.0, n + 1).astype(np.float32),
            "X": r.standard_normal((n + 1, d)).astype(np.float32),
            "ls": np.ones(d, np.float32), "var": 1.0, "kt": 0}
    at_limit = {key: (val[:n] if key in ("V", "p", "X") else val) for key, val in case.items()}
    q = r.choice(n, 64, replace=False)
    stream = torch.cuda.current_stream()
    rc, gi, gd = _noalloc(L, at_limit, q, 10, False, torch, stream)
    assert rc == 0, L.ct_last_error()
    ri, rd = _reference_call(at_limit, q, 10, False)
    assert np.array_equal(gi, ri) and np.array_equal(gd.view(np.uint32), rd.view(np.uint32))
    rc, _, _ = _noalloc(L, case, q, 10, False, torch, stream)
    assert rc == _lib.CT_ERR_UNSUPPORTED
    assert b"scratch" in L.ct_last_error()


def test_noalloc_rejects_inputs_beyond_the_scratch(cuda_available):
    import torch

    from covertreex_gb300 import _lib

    L = _lib.load()
    dummy = torch.zeros(16, device="cuda")
    out = torch.zeros(16, device="cuda")
    ls = (ctypes.c_float * 1)(1.0)
    # 70000 x 256 f32 = 71.7 MB > 64 MiB: rejected before any device work
    rc = L.ct_knn_residual_dense_noalloc(dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 70000, 256, 3, 1.0, ls,
                                         1, 0, dummy.data_ptr(), 1, 5, 0, out.data_ptr(), out.data_ptr(), None)
    assert rc == _lib.CT_ERR_UNSUPPORTED
    assert b"scratch" in L.ct_last_error()
