"""The N>1 path of bench.py on CPU: two gloo ranks shard the queries exactly as the
GPU ranks do (interleaved, no data-path collective), each answers its shard with the
oracle standing in for the device, and rank 0 checks that the gathered rows equal the
single-process answer and that the time reduction is the max over ranks."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_path):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch

    import bench
    from oracle import oracle as O
    from tests._data import gaussian_case

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    assert bench.dist_env() == (world, rank, rank)
    d = bench.dist_init(world, "gloo")
    c = gaussian_case(700, 3, 64, 1, 1.0, seed=4)
    q = bench.shard_queries(700, world, rank)
    idx, _ = O.brute_knn_f32(c["V"], c["p"], c["X"], 1.0, c["ls"], 1, q, 7, True)
    # rows of every rank, as the ranks' results would be concatenated on the host
    rows = [torch.zeros((len(bench.shard_queries(700, world, r)), 7), dtype=torch.int64) for r in range(world)]
    d.all_gather(rows, torch.as_tensor(idx))
    t = torch.tensor([10.0 + rank], dtype=torch.float64)  # per-rank timed region
    d.all_reduce(t, op=d.ReduceOp.MAX)
    if rank == 0:
        full = np.empty((700, 7), np.int64)
        for r in range(world):
            full[bench.shard_queries(700, world, r)] = rows[r].numpy()
        ref, _ = O.brute_knn_f32(c["V"], c["p"], c["X"], 1.0, c["ls"], 1, np.arange(700), 7, True)
        np.save(out_path, np.array([float(np.array_equal(full, ref)), float(t.item())]))
    d.barrier()
    d.destroy_process_group()


def test_two_rank_query_sharding(tmp_path):
    import bench

    # interleaved shards cover every query exactly once
    parts = [bench.shard_queries(1001, 3, r) for r in range(3)]
    allq = np.sort(np.concatenate(parts))
    assert np.array_equal(allq, np.arange(1001))
    out = str(tmp_path / "res.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    same, tmax = np.load(out)
    assert same == 1.0 and tmax == 11.0
