from .estimator import (
    DefaultLinearEstimator,
    Estimator,
    FitResult,
    MeanRateEstimator,
    PersistentEstimator,
    RateFitResult,
)
from .sequential import SequentialPriorityStrategy
from .strategy import BaseStrategy, clip_ops
from .weighted import WeightedStrategy

__all__ = [
    "Estimator",
    "FitResult",
    "RateFitResult",
    "MeanRateEstimator",
    "DefaultLinearEstimator",
    "PersistentEstimator",
    "BaseStrategy",
    "clip_ops",
    "WeightedStrategy",
    "SequentialPriorityStrategy",
]
