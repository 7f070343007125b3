"""Budget allocation between the insertion, update and embedding operations.

Restates python/gpumap/schedule/strategy.py of the reference: progress
tracking, weighted splitting of a time budget and the estimate-or-default
rule (a default op count with +-10% jitter while estimators warm up).
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import numpy as np

from .estimator import Estimator, MeanRateEstimator

_OPS = {"insertion": 0, "update": 1, "embedding": 2}


def _jitter(base: int) -> int:
    lo = max(1, base // 10)
    return base + int(np.random.randint(-lo, lo))


def _estimate_or_fallback(estimator: Estimator, budget_sec: float, confidence: float, default_ops: int) -> int:
    """Ops from the estimator, or the jittered default when it cannot answer
    or answers 0 for a positive budget (so a cycle always makes progress)."""
    if budget_sec <= 0.0:
        return 0
    try:
        ops = max(0, int(estimator.estimate_ops(budget_sec, confidence)))
    except ValueError:
        return _jitter(default_ops)
    return ops if ops > 0 else _jitter(default_ops)


def clip_ops(n_ops: int, ops_range: tuple[int, int]) -> int:
    return max(ops_range[0], min(n_ops, ops_range[1]))


class BaseStrategy(ABC):
    """Tracks progress and splits a budget by weights; subclasses allocate.

    Progress in [0, 1]: insertion = inserted / total; update = 1 - queue /
    inserted; embedding = 1 - queue / pending.  ``reserved`` is idle headroom.
    """

    insertion_ops_range: tuple[int, int] = (0, 0)
    update_ops_range: tuple[int, int] = (0, 0)
    embedding_ops_range: tuple[int, int] = (0, 0)
    _n_instances: int = 0
    _n_inserted: int = 0
    insertion_progress: float = 0.0
    update_progress: float = 0.0
    embedding_progress: float = 0.0

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
        self._weights = list(weights)
        self._reserved = reserved
        self.insertion_estimator = insertion_estimator or MeanRateEstimator()
        self.update_estimator = update_estimator or MeanRateEstimator()
        self.embedding_estimator = embedding_estimator or MeanRateEstimator()
        self._n_instances = n_instances
        self._n_neighbors = n_neighbors
        self.default_n_ops = default_n_ops
        self.confidence = confidence
        self.min_insertion_ops = min_insertion_ops or int(0.01 * n_instances)
        self.max_uint32 = 2**32 - 1
        self._result_history: list = []
        self.completeness = [False, False, False]

    @abstractmethod
    def allocate(self, target_latency: float) -> tuple[int, int, int]: ...

    def update(self, result) -> None:
        self._result_history.append(result)
        if not self.completeness[0] and result.n_insertion_ops > 0:
            self.insertion_estimator.add_sample(result.n_insertion_ops, result.insertion_time)
        if result.n_update_ops > 0:
            self.update_estimator.add_sample(result.n_update_ops, result.update_time)
        if result.n_embedding_ops > 0:
            self.embedding_estimator.add_sample(result.n_embedding_ops, result.embedding_time)
        self._track_progress(result)

    def on_operation_complete(self, operation: str) -> None:
        if operation not in _OPS:
            raise ValueError(f"Unknown operation: {operation}")
        i = _OPS[operation]
        self.completeness[i] = True
        self._weights[i] = 0.0

    def _track_progress(self, result) -> None:
        self._n_inserted = result.n_inserted_instances
        self.insertion_progress = self._n_inserted / self._n_instances if self._n_instances > 0 else 0.0
        self.update_progress = (
            1.0 - result.update_queue_size / self._n_inserted if self._n_inserted > 0 else 0.0
        )
        pending = result.embedding_pending_edges
        self.embedding_progress = 1.0 - result.embedding_queue_size / pending if pending > 0 else 0.0

    def get_progress(self) -> tuple[float, float, float]:
        return (self.insertion_progress, self.update_progress, self.embedding_progress)

    def _split(self, total: float) -> tuple[float, float, float]:
        denom = sum(self._weights) * (1 + self._reserved)
        if denom <= 0:
            return (0.0, 0.0, 0.0)
        a, b, c = (total * w / denom for w in self._weights)
        return (a, b, c)
