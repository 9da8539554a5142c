"""Tree persistence (not in the reference, which keeps trees in memory only).

File layout: one JSON header line (magic, version, shapes, metric parameters and
build parameters), then V [n, m], p [n] and the raw coordinates [n, d] as
little-endian f32.  Loading rebuilds the device layouts and the cover tree with
the saved parameters; the device build is deterministic for a given seed and
order, so the loaded index is the saved one.
"""
from __future__ import annotations

import json

import numpy as np

MAGIC = "covertreex_gb300.index"
VERSION = 1


def save_index(index, path) -> None:
    v, p, c = index.inputs_device()
    header = {"magic": MAGIC, "version": VERSION, "n": index.n, "m": index.m, "d": index.d,
              "variance": index.variance, "lengthscale": [float(x) for x in np.atleast_1d(index.lengthscale)],
              "kernel_type": index.kernel_type, **index.build_params}
    with open(path, "wb") as fh:
        fh.write((json.dumps(header) + "\n").encode())
        for a in (v, p, c):
            fh.write(np.ascontiguousarray(a.cpu().numpy(), dtype="<f4").tobytes())


def load_index(path, *, device=None, stream=None):
    from .device import CudaResidualIndex

    with open(path, "rb") as fh:
        header = json.loads(fh.readline().decode())
        if header.get("magic") != MAGIC or int(header.get("version", 0)) != VERSION:
            raise ValueError(f"{path}: not a covertreex_gb300 index file (version {VERSION})")
        n, m, d = int(header["n"]), int(header["m"]), int(header["d"])
        raw = [fh.read(4 * n * m), fh.read(4 * n), fh.read(4 * n * d)]
        if [len(b) for b in raw] != [4 * n * m, 4 * n, 4 * n * d]:
            raise ValueError(f"{path}: truncated index file")
        v = np.frombuffer(raw[0], dtype="<f4").reshape(n, m).astype(np.float32)
        p = np.frombuffer(raw[1], dtype="<f4").astype(np.float32)
        c = np.frombuffer(raw[2], dtype="<f4").reshape(n, d).astype(np.float32)
    return CudaResidualIndex(v, p, c, variance=header["variance"], lengthscale=header["lengthscale"],
                             kernel_type=header["kernel_type"], chunk_size=header["chunk_size"],
                             order=header["order"], seed=header["seed"], build_tree=header["build_tree"],
                             query_slab=header["query_slab"], device=device, stream=stream)


__all__ = ["save_index", "load_index", "MAGIC", "VERSION"]
