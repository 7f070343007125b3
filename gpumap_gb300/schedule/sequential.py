"""Insertion, then update, then embedding: the whole budget goes to the first
unfinished operation (reference: python/gpumap/schedule/sequential.py)."""
from __future__ import annotations

from typing import Optional

from .estimator import Estimator, MeanRateEstimator
from .strategy import BaseStrategy


class SequentialPriorityStrategy(BaseStrategy):
    def __init__(
        self,
        n_instances: int,
        n_neighbors: int = 15,
        insertion_estimator: Optional[Estimator] = None,
        update_estimator: Optional[Estimator] = None,
        embedding_estimator: Optional[Estimator] = None,
        default_n_ops: int = 100,
        confidence: float = 0.95,
        min_insertion_ops: int = 500,
    ):
        super().__init__(
            weights=(1.0, 1.0, 1.0),
            reserved=0.1,
            insertion_estimator=insertion_estimator or MeanRateEstimator(),
            update_estimator=update_estimator or MeanRateEstimator(),
            embedding_estimator=embedding_estimator or MeanRateEstimator(),
            n_instances=n_instances,
            n_neighbors=n_neighbors,
            default_n_ops=default_n_ops,
            confidence=confidence,
            min_insertion_ops=min_insertion_ops,
        )
        self._update_counter = 0

    def allocate(self, target_latency: float) -> tuple[int, int, int]:
        for i in range(3):
            if not self.completeness[i]:
                out = [0, 0, 0]
                out[i] = self.max_uint32
                return tuple(out)
        return (0, 0, self.max_uint32)
