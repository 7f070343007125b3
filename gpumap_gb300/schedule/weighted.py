"""Default strategy: weighted budget split with a floor on insertion
(reference: python/gpumap/schedule/weighted.py)."""
from __future__ import annotations

from typing import Optional

from .estimator import Estimator, MeanRateEstimator
from .strategy import BaseStrategy, _estimate_or_fallback, clip_ops


class WeightedStrategy(BaseStrategy):
    def __init__(
        self,
        n_instances: int,
        n_neighbors: int = 15,
        weights: tuple[float, float, float] = (1.0, 2.0, 1.0),
        reserved: float = 0.1,
        insertion_estimator: Optional[Estimator] = None,
        update_estimator: Optional[Estimator] = None,
        embedding_estimator: Optional[Estimator] = None,
        default_n_ops: int = 100,
        confidence: float = 0.95,
        min_insertion_ops: int = 500,
    ):
        super().__init__(
            weights=weights,
            reserved=reserved,
            insertion_estimator=insertion_estimator or MeanRateEstimator(),
            update_estimator=update_estimator or MeanRateEstimator(),
            embedding_estimator=embedding_estimator or MeanRateEstimator(),
            n_instances=n_instances,
            n_neighbors=n_neighbors,
            default_n_ops=default_n_ops,
            confidence=confidence,
            min_insertion_ops=min_insertion_ops,
        )

    def allocate(self, target_latency: float) -> tuple[int, int, int]:
        budgets = self._split(max(0.0, target_latency))
        ests = (self.insertion_estimator, self.update_estimator, self.embedding_estimator)
        n_ins, n_upd, n_emb = (
            _estimate_or_fallback(e, t, self.confidence, self.default_n_ops) for e, t in zip(ests, budgets)
        )
        return (
            clip_ops(n_ins, (self.min_insertion_ops, self.max_uint32)),
            clip_ops(n_upd, (0, self.max_uint32)),
            clip_ops(n_emb, (0, self.max_uint32)),
        )
