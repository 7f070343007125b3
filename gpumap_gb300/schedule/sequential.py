"""One operation at a time (reference python/gpumap/schedule/sequential.py:9-52)."""
from __future__ import annotations

from typing import Optional

from .estimator import Estimator
from .strategy import OPERATIONS, UINT32_MAX, BaseStrategy


class SequentialPriorityStrategy(BaseStrategy):
    """Insertion until it finishes, then update until it finishes, then
    embedding: the first unfinished operation gets an unbounded op count (the
    engine stops it when its work runs out) and the other two none.  The
    estimators still learn from every cycle."""

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
        super().__init__(weights=(1.0, 1.0, 1.0), reserved=0.1, insertion_estimator=insertion_estimator,
                         update_estimator=update_estimator, embedding_estimator=embedding_estimator,
                         n_instances=n_instances, n_neighbors=n_neighbors, default_n_ops=default_n_ops,
                         confidence=confidence, min_insertion_ops=min_insertion_ops)

    def allocate(self, target_latency: float) -> tuple[int, int, int]:
        active = next((op for op in OPERATIONS if not self._done[op]), OPERATIONS[-1])
        return tuple(UINT32_MAX if op == active else 0 for op in OPERATIONS)
