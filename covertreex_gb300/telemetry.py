"""Telemetry in the reference's formats.

* ``query_telemetry`` — the per-query counters of ``ResidualQueryTelemetry``
  (src/telemetry.rs:1-19) as the reference's PyO3 layer hands them to Python
  (``CoverTreeWrapper.last_query_telemetry``, src/lib.rs:357-363): the same keys,
  with the GPU forms' counters under ``"gpu"``.  The GPU searches have no
  frontier, budget ladder or level cache, so those entries are empty / zero.
* ``BatchTelemetryWriter`` — JSONL rows of the ``covertreex.benchmark_batch.v2``
  schema (covertreex/telemetry/schemas.py:6-43): the required keys, ``runtime``,
  ``metadata`` and ``seed_pack`` objects, and the measurements as extra keys, so
  the reference's tooling (``BenchmarkBatchRecord.from_payload``) reads GPU runs.
"""
from __future__ import annotations

import hashlib
import json
import time
import uuid
from typing import Any, Mapping, Optional

BENCHMARK_BATCH_SCHEMA_VERSION = 2
BENCHMARK_BATCH_SCHEMA_ID = f"covertreex.benchmark_batch.v{BENCHMARK_BATCH_SCHEMA_VERSION}"
BENCHMARK_BATCH_REQUIRED = ("schema_id", "schema_version", "run_id", "run_hash", "timestamp", "batch_event_index",
                            "batch_index", "batch_size", "runtime", "metadata")


def query_telemetry(stats: Mapping[str, Any], form: str = "") -> dict:
    evals = int(stats.get("distance_evals", 0) or 0)
    return {
        "frontier_levels": [], "frontier_expanded": [], "yields": [], "caps_applied": 0,
        "prunes_lower_bound": 0, "prunes_lower_bound_chunks": 0, "prunes_cap": 0, "masked_dedup": 0,
        "distance_evals": max(evals, 0), "budget_escalations": 0, "budget_early_terminate": 0,
        "level_cache_hits": 0, "level_cache_misses": 0, "block_sizes": [], "predecessor_filtered": 0,
        "subtrees_pruned": 0,
        "gpu": {"form": form, **{k: stats[k] for k in ("pairs_screened", "pairs_rescored", "kernel_launches",
                                                      "device_ms", "screen_ms", "threshold_ms", "rescore_ms",
                                                      "screen_pairs_main", "overflow_queries", "pairs_exhaustive")
                                   if k in stats}},
    }


def _digest(obj: Any) -> str:
    return hashlib.sha256(json.dumps(obj, sort_keys=True, default=str).encode()).hexdigest()[:16]


class BatchTelemetryWriter:
    """Append ``covertreex.benchmark_batch.v2`` rows to a JSONL file."""

    def __init__(self, path, *, runtime: Optional[Mapping[str, Any]] = None, run_id: Optional[str] = None,
                 seed_pack: Optional[Mapping[str, Any]] = None):
        self.path = str(path)
        self.runtime = dict(runtime or {"engine": "cuda"})
        self.run_id = run_id or uuid.uuid4().hex[:12]
        self.run_hash = _digest({"run_id": self.run_id, "runtime": self.runtime})
        self.runtime_digest = _digest(self.runtime)
        self.seed_pack = dict(seed_pack or {})
        self.events = 0

    def record(self, *, batch_index: int, batch_size: int, measurements: Optional[Mapping[str, Any]] = None,
               metadata: Optional[Mapping[str, Any]] = None) -> dict:
        row = {
            "schema_id": BENCHMARK_BATCH_SCHEMA_ID, "schema_version": BENCHMARK_BATCH_SCHEMA_VERSION,
            "run_id": self.run_id, "run_hash": self.run_hash, "runtime_digest": self.runtime_digest,
            "timestamp": time.time(), "batch_event_index": self.events, "batch_index": int(batch_index),
            "batch_size": int(batch_size), "runtime": self.runtime, "metadata": dict(metadata or {}),
            "seed_pack": self.seed_pack,
        }
        for k, v in (measurements or {}).items():
            if k not in row:
                row[k] = v
        with open(self.path, "a") as fh:
            fh.write(json.dumps(row, default=float) + "\n")
        self.events += 1
        return row


__all__ = ["query_telemetry", "BatchTelemetryWriter", "BENCHMARK_BATCH_SCHEMA_ID", "BENCHMARK_BATCH_REQUIRED"]
