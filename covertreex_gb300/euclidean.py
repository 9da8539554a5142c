"""Euclidean kNN on the GPU (the reference's ``cover_tree(coords)`` path,
covertreex/api/factory.py:284-296 -> CoverTreeWrapper.insert / knn_query).

The reference answers with a best-first search whose pruning radius its batch
insert does not guarantee (approximate); this engine returns the exact k
nearest points (ties by lower index) through ``ct_knn_euclidean``.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .device import _as_device, _stream_ptr, _torch
from .engine import _format_knn_output


class EuclideanTree:
    def __init__(self, coords: np.ndarray, device=None):
        torch = _torch()
        self.device = torch.device(device if device is not None else "cuda")
        self.points = _as_device(np.asarray(coords, dtype=np.float32), torch.float32, self.device)
        if self.points.dim() == 1:
            self.points = self.points.reshape(-1, 1)
        self.n, self.d = int(self.points.shape[0]), int(self.points.shape[1])
        self.build_seconds = 0.0

    def knn_device(self, queries, k: int, predecessor: bool = False):
        torch = _torch()
        q = _as_device(queries, torch.float32, self.device)
        if q.dim() == 1:
            q = q.reshape(1, -1)
        if q.shape[1] != self.d:
            raise ValueError(f"queries must have {self.d} columns")
        nq = int(q.shape[0])
        idx = torch.empty((nq, k), dtype=torch.int64, device=self.device)
        dist = torch.empty((nq, k), dtype=torch.float32, device=self.device)
        rc = _lib.load().ct_knn_euclidean(self.points.data_ptr(), self.n, self.d, q.data_ptr(), nq, int(k),
                                          1 if predecessor else 0, idx.data_ptr(), dist.data_ptr(), _stream_ptr(None))
        _lib.check(rc)
        return idx, dist

    def knn(self, query_points, *, k: int, return_distances: bool = False, predecessor_mode: bool = False, **_):
        if int(k) <= 0:
            raise ValueError("k must be positive")
        qp = np.asarray(query_points, dtype=np.float32)
        if qp.ndim == 2 and qp.shape[1] == 1 and self.d != 1:
            raise ValueError("Euclidean queries are points; pass queries=coords (integer ids are not points)")
        idx, dist = self.knn_device(qp, int(k), predecessor=predecessor_mode)
        return _format_knn_output(idx.cpu().numpy(), dist.cpu().numpy(), return_distances=return_distances)
