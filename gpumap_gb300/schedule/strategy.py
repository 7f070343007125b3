"""Latency-budget strategies: how many ops of each operation one cycle runs.

A strategy owns one cost model per operation (insertion, update,
embedding), learns from every cycle's result, tracks the three progress
fractions, and turns a target latency into an (insertion, update, embedding)
op triple.  The interface (``allocate``, ``update``, ``on_operation_complete``,
``get_progress``) and the allocations are those of the reference's
python/gpumap/schedule/strategy.py:41-160, checked against its own outputs in
tests/golden/schedule_golden.json.

Rules shared by the strategies:

* The budget is split in proportion to the operation weights, with a
  ``reserved`` fraction held back: share_i = total * w_i / (sum(w) * (1 + reserved)).
  A finished operation's weight drops to zero.
* A share becomes ops through the operation's estimator.  While the estimator
  cannot answer (too few samples) or answers 0 for a positive share, the
  strategy proposes ``default_n_ops`` with +-10 % uniform jitter
  (numpy's global generator), so every cycle makes progress.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import numpy as np

from .estimator import Estimator, MeanRateEstimator

OPERATIONS = ("insertion", "update", "embedding")
UINT32_MAX = 2**32 - 1


def clip_ops(n_ops: int, ops_range: tuple[int, int]) -> int:
    """n_ops limited to [ops_range[0], ops_range[1]]."""
    lo, hi = ops_range
    return max(lo, min(n_ops, hi))


def jittered(n_ops: int) -> int:
    """n_ops moved by a uniform integer in [-max(1, n_ops // 10), that bound)."""
    spread = max(1, n_ops // 10)
    return n_ops + int(np.random.randint(-spread, spread))


def ops_for_budget(estimator: Estimator, seconds: float, confidence: float, default_ops: int) -> int:
    """Ops that fit ``seconds``; 0 for no budget; the jittered default while
    the estimator has no usable answer."""
    if seconds <= 0.0:
        return 0
    try:
        ops = max(0, int(estimator.estimate_ops(seconds, confidence)))
    except ValueError:
        ops = 0
    return ops if ops > 0 else jittered(default_ops)


class BaseStrategy(ABC):
    """Budget splitting, estimators and progress; subclasses decide the
    allocation.  ``min_insertion_ops`` defaults to 1 % of the dataset."""

    def __init__(
        self,
        weights: tuple[float, float, float] = (1.0, 1.0, 1.0),
        reserved: float = 0.2,
        insertion_estimator: Optional[Estimator] = None,
        update_estimator: Optional[Estimator] = None,
        embedding_estimator: Optional[Estimator] = None,
        n_instances: int = 0,
        n_neighbors: int = 15,
        default_n_ops: int = 100,
        confidence: float = 0.95,
        min_insertion_ops: Optional[int] = None,
    ):
        given = (insertion_estimator, update_estimator, embedding_estimator)
        self._estimators = {op: est or MeanRateEstimator() for op, est in zip(OPERATIONS, given)}
        self._weights = {op: float(w) for op, w in zip(OPERATIONS, weights)}
        self._done = dict.fromkeys(OPERATIONS, False)
        self._reserved = reserved
        self._n_instances = n_instances
        self._n_neighbors = n_neighbors
        self.default_n_ops = default_n_ops
        self.confidence = confidence
        self.min_insertion_ops = min_insertion_ops or int(0.01 * n_instances)
        self.max_uint32 = UINT32_MAX
        self._history: list = []
        self._progress = {op: 0.0 for op in OPERATIONS}

    # -- estimators and state ------------------------------------------------
    @property
    def insertion_estimator(self) -> Estimator:
        return self._estimators["insertion"]

    @property
    def update_estimator(self) -> Estimator:
        return self._estimators["update"]

    @property
    def embedding_estimator(self) -> Estimator:
        return self._estimators["embedding"]

    @property
    def completeness(self) -> list[bool]:
        """[insertion, update, embedding] finished flags."""
        return [self._done[op] for op in OPERATIONS]

    @property
    def insertion_progress(self) -> float:
        return self._progress["insertion"]

    @property
    def update_progress(self) -> float:
        return self._progress["update"]

    @property
    def embedding_progress(self) -> float:
        return self._progress["embedding"]

    # -- the cycle interface -------------------------------------------------
    @abstractmethod
    def allocate(self, target_latency: float) -> tuple[int, int, int]: ...

    def update(self, result) -> None:
        """Learns from one cycle's result (op counts and phase seconds); a
        finished insertion stops contributing samples."""
        self._history.append(result)
        observed = (
            ("insertion", result.n_insertion_ops, result.insertion_time),
            ("update", result.n_update_ops, result.update_time),
            ("embedding", result.n_embedding_ops, result.embedding_time),
        )
        for op, ops, secs in observed:
            if ops > 0 and not (op == "insertion" and self._done[op]):
                self._estimators[op].add_sample(ops, secs)
        self._record_progress(result)

    def on_operation_complete(self, operation: str) -> None:
        if operation not in self._done:
            raise ValueError(f"Unknown operation: {operation}")
        self._done[operation] = True
        self._weights[operation] = 0.0

    def get_progress(self) -> tuple[float, float, float]:
        return tuple(self._progress[op] for op in OPERATIONS)

    # -- helpers -------------------------------------------------------------
    def _record_progress(self, result) -> None:
        def frac_left(left, total):
            return 1.0 - (left / total) if total > 0 else 0.0

        inserted = result.n_inserted_instances
        self._progress["insertion"] = inserted / self._n_instances if self._n_instances > 0 else 0.0
        self._progress["update"] = frac_left(result.update_queue_size, inserted)
        self._progress["embedding"] = frac_left(result.embedding_queue_size, result.embedding_pending_edges)

    def _split(self, total: float) -> tuple[float, float, float]:
        denom = sum(self._weights.values()) * (1 + self._reserved)
        if denom <= 0:
            return (0.0, 0.0, 0.0)
        return tuple(total * self._weights[op] / denom for op in OPERATIONS)
