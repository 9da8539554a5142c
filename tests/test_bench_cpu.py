"""CPU checks of bench.py's host-side logic: the FP64 check of the timed output
(run here with torch on the CPU) against the oracle's FP64 brute force."""
import numpy as np

import bench
from covertreex_gb300 import synthetic
from oracle import oracle as O


def _small_workload():
    return synthetic.make("plain_small", n=1500)


def test_fp64_check_accepts_oracle_rows():
    import torch

    wl = _small_workload()
    rows = np.random.default_rng(4).choice(wl.n, 300, replace=False)
    fi, fd = O.brute_knn_f64(wl.v, wl.p, wl.coords, wl.variance, [wl.lengthscale] * wl.d, wl.kernel_type, rows,
                             wl.k, wl.predecessor)
    got_d = np.where(fi >= 0, fd, np.float32(3.402823466e38)).astype(np.float32)
    st = bench.fp64_check(wl, torch.device("cpu"), rows, fi, got_d, block=64)
    assert st["rows_identical"] == rows.size
    assert st["mismatches_beyond_near_tie"] == 0 and st["count_mismatches"] == 0
    assert st["predecessor_violations"] == 0
    assert st["max_abs_err"] < 1e-6


def test_fp64_check_flags_planted_mistakes():
    import torch

    wl = _small_workload()
    rows = np.sort(np.random.default_rng(5).choice(np.arange(200, wl.n), 100, replace=False))
    fi, fd = O.brute_knn_f64(wl.v, wl.p, wl.coords, wl.variance, [wl.lengthscale] * wl.d, wl.kernel_type, rows,
                             wl.k, wl.predecessor)
    gi = fi.copy()
    gd = fd.astype(np.float32)
    gi[3, 0] = rows[3] + 1          # a successor: breaks the predecessor constraint and the set
    gi[7, -1] = np.setdiff1d(np.arange(rows[7]), fi[7])[-1]   # a far candidate instead of the k-th
    gd[11, 2] += 1e-3               # a distance error
    st = bench.fp64_check(wl, torch.device("cpu"), rows, gi, gd, block=32)
    assert st["predecessor_violations"] == 1
    assert st["mismatches_beyond_near_tie"] == 2
    assert st["max_abs_err"] >= 1e-3 * 0.99
