"""GB300-native progressive UMAP engine with the gpumap Python surface.

``import gpumap_gb300 as gpumap`` gives the reference package's public names
(python/gpumap/__init__.py:16-29).  The engine is the in-tree CUDA library
``_lib/libgpumap_gb300.so`` reached through the pybind11 module ``_core``.
"""
from __future__ import annotations

from ._core import GPUMAPParams
from .gpumap import GPUMAP
from .metric import Metric
from .schedule import (
    BaseStrategy,
    DefaultLinearEstimator,
    Estimator,
    MeanRateEstimator,
    PersistentEstimator,
    SequentialPriorityStrategy,
    WeightedStrategy,
)

__all__ = [
    "GPUMAP",
    "GPUMAPParams",
    "Metric",
    "BaseStrategy",
    "WeightedStrategy",
    "SequentialPriorityStrategy",
    "Estimator",
    "MeanRateEstimator",
    "DefaultLinearEstimator",
    "PersistentEstimator",
]
