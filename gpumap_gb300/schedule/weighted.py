"""Weighted split of the cycle budget (the default strategy; reference
python/gpumap/schedule/weighted.py:9-59)."""
from __future__ import annotations

from typing import Optional

from .estimator import Estimator
from .strategy import OPERATIONS, UINT32_MAX, BaseStrategy, clip_ops, ops_for_budget


class WeightedStrategy(BaseStrategy):
    """Every unfinished operation gets its weighted share of the budget
    (default weights insertion 1, update 2, embedding 1, 10 % held back),
    converted to ops by its estimator.  Insertion never gets fewer than
    ``min_insertion_ops`` (500 by default) while it runs, so the dataset keeps
    streaming in."""

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
        super().__init__(weights=weights, reserved=reserved, insertion_estimator=insertion_estimator,
                         update_estimator=update_estimator, embedding_estimator=embedding_estimator,
                         n_instances=n_instances, n_neighbors=n_neighbors, default_n_ops=default_n_ops,
                         confidence=confidence, min_insertion_ops=min_insertion_ops)

    def allocate(self, target_latency: float) -> tuple[int, int, int]:
        shares = self._split(max(0.0, target_latency))
        floors = {"insertion": self.min_insertion_ops, "update": 0, "embedding": 0}
        out = []
        for op, seconds in zip(OPERATIONS, shares):  # in order: the jitter draws are ordered
            ops = ops_for_budget(self._estimators[op], seconds, self.confidence, self.default_n_ops)
            out.append(clip_ops(ops, (floors[op], UINT32_MAX)))
        return tuple(out)
