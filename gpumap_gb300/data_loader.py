"""Chunked data feeds for the progressive engine (reference: python/gpumap/data_loader.py).

``get_next_chunk(n)`` hands out the next ``n`` rows (fewer at the end).  The
named preload datasets of the reference are not shipped; asking for one
whose files are absent raises ``ValueError`` as the reference does.
"""
from __future__ import annotations

import os

import numpy as np


class DataLoader:
    n_instances: int
    n_features: int
    X: np.ndarray
    y: np.ndarray | None = None
    _current_index: int = 0

    def __init__(self):
        raise NotImplementedError("init not implemented")

    def get_next_chunk(self, chunk_size: int) -> np.ndarray:
        start = self._current_index
        stop = min(start + max(0, int(chunk_size)), self.n_instances)
        self._current_index = stop
        return self.X[start:stop]


def load_numpy_data(file_path: str) -> np.ndarray:
    if not os.path.exists(file_path):
        raise ValueError(f"File not found: {file_path}")
    return np.load(file_path)


PRELOAD_DATASETS = ["mnist", "fashion_mnist", "wine_reviews", "svhn"]


class PreloadDataLoader(DataLoader):
    def __init__(self, dataset_name: str):
        if dataset_name not in PRELOAD_DATASETS:
            raise ValueError(f"Unsupported dataset name: {dataset_name}")
        base = os.path.join(os.path.dirname(os.path.realpath(__file__)), "data", dataset_name)
        x_path = os.path.join(base, f"{dataset_name}_X.npy")
        y_path = os.path.join(base, f"{dataset_name}_y.npy")
        self.X = load_numpy_data(x_path)
        self.y = load_numpy_data(y_path) if os.path.exists(y_path) else None
        self.n_instances = len(self.X)
        self.n_features = self.X.shape[1]
        self._current_index = 0


class NumpyDataLoader(DataLoader):
    def __init__(self, dataset_name: str, npy_path: str, label_npy_path: str | None = None):
        self.dataset_name = dataset_name
        self.X = load_numpy_data(npy_path)
        self.y = load_numpy_data(label_npy_path) if label_npy_path else None
        self.n_instances = len(self.X)
        self.n_features = self.X.shape[1]
        self._current_index = 0


class ArrayDataLoader(DataLoader):
    """Feeds an in-memory array (a convenience the reference lacks)."""

    def __init__(self, X: np.ndarray, y: np.ndarray | None = None, dataset_name: str = "array"):
        self.dataset_name = dataset_name
        self.X = X
        self.y = y
        self.n_instances = len(X)
        self.n_features = X.shape[1]
        self._current_index = 0
