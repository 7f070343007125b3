"""GB300-native progressive UMAP engine with the gpumap Python surface.

``import gpumap_gb300 as gpumap`` gives the reference package's public names
(python/gpumap/__init__.py:16-29).  The engine is the in-tree CUDA library
``_lib/libgpumap_gb300.so`` reached through the pybind11 module ``_core``.

The public names resolve on first use, so that importing a pure-Python
submodule (``gpumap_gb300.datasets``, ``gpumap_gb300.schedule``) does not load
the native library.
"""
from __future__ import annotations

import importlib

_EXPORTS = {
    "GPUMAP": ".gpumap",
    "GPUMAPParams": "._core",
    "Metric": ".metric",
    "BaseStrategy": ".schedule",
    "WeightedStrategy": ".schedule",
    "SequentialPriorityStrategy": ".schedule",
    "Estimator": ".schedule",
    "MeanRateEstimator": ".schedule",
    "DefaultLinearEstimator": ".schedule",
    "PersistentEstimator": ".schedule",
}

__all__ = list(_EXPORTS)


def __getattr__(name: str):
    mod = _EXPORTS.get(name)
    if mod is None:
        raise AttributeError(f"module 'gpumap_gb300' has no attribute {name!r}")
    value = getattr(importlib.import_module(mod, __name__), name)
    globals()[name] = value
    return value


def __dir__():
    return sorted(set(globals()) | set(__all__))
