"""Array helpers (reference: python/gpumap/utils/as_f32_c_contig_2d.py)."""
from __future__ import annotations

import numpy as np


def _as_f32_c_contig_2d(x: np.ndarray) -> np.ndarray:
    """Returns ``x`` as a C-contiguous float32 2-D array (copying only if needed)."""
    if np.ndim(x) != 2:
        raise ValueError("Input array must be 2D")
    if x.dtype != np.float32 or not x.flags["C_CONTIGUOUS"]:
        x = np.ascontiguousarray(x, dtype=np.float32)
    return x


__all__ = ["_as_f32_c_contig_2d"]
