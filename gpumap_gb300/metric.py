"""Distance metric selector for ``GPUMAPParams.metric``.

``params.metric`` takes a name ("euclidean", "cosine"; any case), a plain int
or this enum; the values equal the engine's GM_METRIC_* codes
(reference: python/gpumap/metric.py, cpp/include/gpumap/gpumap.cuh:13).
"""
from __future__ import annotations

import enum


class Metric(enum.IntEnum):
    Euclidean = 0
    Cosine = 1
