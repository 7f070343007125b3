"""User-facing progressive UMAP driver (reference: python/gpumap/gpumap.py).

``GPUMAP(data_loader, params)`` fits the UMAP curve parameters a, b from
``min_dist``, creates the engine and then advances it one cycle per
``run(target_latency)`` (budget split by a strategy) or
``run_with_n_ops(i, u, e)`` (explicit op counts).  Results are zero-copy
device views sliced to the inserted rows: a CuPy array when CuPy is
installed, else a torch tensor (through DLPack, ordered after the session's
queued work on torch's current stream), else the engine's view object.
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import curve_fit

from . import _core
from .data_loader import DataLoader
from .schedule import BaseStrategy, Estimator, WeightedStrategy
from .utils import _as_f32_c_contig_2d
from .validators import validate_data_chunk


def find_ab_params(spread, min_dist):
    """Least-squares fit of 1 / (1 + a x^(2b)) to the UMAP target curve
    (1 below min_dist, exp(-(x - min_dist)/spread) above) on 300 points of [0, 3*spread]."""

    def curve(x, a, b):
        return 1.0 / (1.0 + a * x ** (2 * b))

    xv = np.linspace(0, spread * 3, 300)
    yv = np.where(xv < min_dist, 1.0, np.exp(-(xv - min_dist) / spread))
    params, _ = curve_fit(curve, xv, yv)
    return params[0], params[1]


def _device_array(view):
    """A device array over an engine view: CuPy through the CUDA Array
    Interface when CuPy is installed, else a torch tensor through DLPack (the
    view makes torch's current stream wait for the session's queued work),
    else the view itself.  The memory stays the engine's."""
    try:
        import cupy as cp  # noqa: F401

        return cp.asarray(view)
    except ImportError:
        pass
    try:
        import torch
    except ImportError:
        return view
    return torch.from_dlpack(view)


class GPUMAP:
    def __init__(
        self,
        data_loader: DataLoader,
        params: _core.GPUMAPParams,
        strategy: BaseStrategy | None = None,
        insertion_estimator: Estimator | None = None,
        update_estimator: Estimator | None = None,
        embedding_estimator: Estimator | None = None,
        default_n_ops: int = 100,
    ):
        self.data_loader = data_loader
        self._params = params
        if self.params.min_dist > 1.0:
            raise ValueError("min_dist must be <= 1.0")
        self.params.a, self.params.b = find_ab_params(1.0, self.params.min_dist)
        try:
            self._impl = _core.GPUMAP(self.params)
        except MemoryError:
            # one retry, as the reference does for a transient first allocation
            self._impl = _core.GPUMAP(self.params)
        self._closed = False
        self._strategy = strategy or WeightedStrategy(
            n_instances=data_loader.n_instances,
            n_neighbors=params.n_neighbors,
            insertion_estimator=insertion_estimator,
            update_estimator=update_estimator,
            embedding_estimator=embedding_estimator,
            default_n_ops=default_n_ops,
        )
        self._inserted_instances = 0
        self._impl.initialize(self.data_loader.n_instances, self.data_loader.n_features)

    @property
    def params(self) -> _core.GPUMAPParams:
        return self._params

    @property
    def n_inserted_instances(self) -> int:
        return self._inserted_instances

    @property
    def strategy(self) -> BaseStrategy:
        return self._strategy

    def close(self):
        if not self._closed:
            self._impl.close()
            self._closed = True

    def _feed(self, n_insertion_ops: int) -> None:
        if n_insertion_ops <= 0:
            return
        chunk = self.data_loader.get_next_chunk(n_insertion_ops)
        try:
            validate_data_chunk(chunk, self._params.n_features)
            chunk = _as_f32_c_contig_2d(chunk)
        except ValueError as e:
            print(f"Error validating data chunk: {e}")
        self._impl.append_data(chunk)

    def _after(self, res):
        self._inserted_instances = res.n_inserted_instances
        self._strategy.update(res)
        if res.insertion_completed:
            self._strategy.on_operation_complete("insertion")
        if res.update_completed:
            self._strategy.on_operation_complete("update")
        if res.embedding_completed:
            self._strategy.on_operation_complete("embedding")
        return res

    def run_with_n_ops(self, n_insertion_ops: int, n_update_ops: int, n_embedding_ops: int):
        self._feed(n_insertion_ops)
        return self._after(self._impl.run(n_insertion_ops, n_update_ops, n_embedding_ops))

    def run(self, target_latency: float = 10.0):
        alloc = self._strategy.allocate(target_latency)
        n_ins = min(alloc[0], self.data_loader.n_instances - self._inserted_instances)
        self._feed(n_ins)
        return self._after(self._impl.run(n_ins, alloc[1], alloc[2]))

    def get_embedding(self):
        return _device_array(self._impl.get_embedding())[: self._inserted_instances]

    def get_neighbor_indices(self):
        v = _device_array(self._impl.get_neighbor_indices())
        return v[: self._inserted_instances, : self._params.n_neighbors]

    def get_neighbor_dists(self):
        v = _device_array(self._impl.get_neighbor_dists())
        return v[: self._inserted_instances, : self._params.n_neighbors]
