"""Drives the reference's own Python API (``gpumap.GPUMAP`` over its compiled
``_core``) on a seeded in-memory workload.  Test and benchmark infrastructure
only; nothing in the product imports it.

The reference ships loaders only for ``.npy`` files and downloadable
datasets (python/gpumap/data_loader.py:7-62); ``array_loader`` subclasses its
``DataLoader`` base class over an array already in memory, as a user of the
reference would.
"""
from __future__ import annotations

import time

import numpy as np

from . import refpkg


def array_loader(X: np.ndarray):
    gp = refpkg.load()
    from gpumap.data_loader import DataLoader

    class ArrayLoader(DataLoader):
        def __init__(self, X):
            self.X = np.ascontiguousarray(X, dtype=np.float32)
            self.y = None
            self.n_instances = len(self.X)
            self.n_features = self.X.shape[1]
            self._current_index = 0

    del gp
    return ArrayLoader(X)


def make_model(X: np.ndarray, k: int = 15, metric: str = "euclidean", max_epoch: int = 200,
               negative_sample_rate: int = 5, min_dist: float = 0.1):
    """A reference ``gpumap.GPUMAP`` over X (its constructor fits a, b)."""
    gp = refpkg.load()
    p = gp.GPUMAPParams()
    p.n_neighbors = k
    p.n_components = 2
    p.min_dist = min_dist
    p.negative_sample_rate = negative_sample_rate
    p.max_epoch = max_epoch
    p.metric = metric
    p.n_instances = X.shape[0]
    p.n_features = X.shape[1]
    return gp.GPUMAP(array_loader(X), p)


def neighbor_indices(model) -> np.ndarray:
    import torch

    torch.cuda.synchronize()
    return model.get_neighbor_indices().to(torch.int64).cpu().numpy()


def embedding(model) -> np.ndarray:
    import torch

    torch.cuda.synchronize()
    return model.get_embedding().cpu().numpy()


def progressive_build(X, chunk, upd, emb, k=15, metric="euclidean", max_epoch=200, recall_fn=None,
                      target=None, max_final=0, plateau=None):
    """Inserts X in chunks of ``chunk`` rows with run_with_n_ops(chunk, upd,
    emb), then runs full update cycles run_with_n_ops(0, n, 0) while
    ``recall_fn(indices) < target`` (at most ``max_final``; with ``plateau``
    set, also stops once a cycle raises recall by less than it).  Returns
    (model, seconds, recall, final cycles); the clock covers every run call
    and recall check, as points-inserted/s counts every cycle until the
    target is met."""
    import torch

    n = X.shape[0]
    model = make_model(X, k=k, metric=metric, max_epoch=max_epoch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c in range(0, n, chunk):
        model.run_with_n_ops(min(chunk, n - c), upd, emb)
    rec = recall_fn(neighbor_indices(model)) if recall_fn else None
    rounds = 0
    while recall_fn and rec < target and rounds < max_final:
        model.run_with_n_ops(0, n, 0)
        rounds += 1
        prev, rec = rec, recall_fn(neighbor_indices(model))
        if plateau is not None and rec - prev < plateau:
            break
    torch.cuda.synchronize()
    return model, time.perf_counter() - t0, rec, rounds
