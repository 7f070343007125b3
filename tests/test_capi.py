"""The C ABI library loads and exports every declared entry point; the
pybind11 module mirrors the reference's Python surface.  No GPU calls."""
import re
from pathlib import Path

import pytest

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(gm_[a-z_]+)\s*\(", text))
    return sorted(names)


def test_all_declared_symbols_exported(native):
    lib = native.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_params_defaults_match_reference(native):
    # reference defaults: cpp/include/gpumap/gpumap.cuh:15-30
    p = native.default_params()
    assert (p.n_neighbors, p.n_components, p.negative_sample_rate, p.max_epoch) == (15, 2, 5, 200)
    assert abs(p.min_dist - 0.1) < 1e-7 and (p.a, p.b, p.alpha) == (1.0, 1.0, 1.0)
    assert p.metric == 0 and p.verbose == 0 and p.n_instances == 0 and p.n_features == 0


def test_pybind_surface(native):
    import gpumap_gb300 as gm
    from gpumap_gb300 import _core

    p = _core.GPUMAPParams()
    for name in ("n_neighbors", "n_components", "min_dist", "negative_sample_rate", "max_epoch", "a", "b",
                 "alpha", "verbose", "metric", "n_instances", "n_features"):
        assert hasattr(p, name)
    assert p.metric == "euclidean"
    p.metric = "CoSiNe"
    assert p.metric == "cosine"
    p.metric = gm.Metric.Euclidean
    assert p.metric == "euclidean"
    with pytest.raises(ValueError):
        p.metric = "manhattan"
    for name in ("n_insertion_ops", "n_update_ops", "n_embedding_ops", "insertion_time", "update_time",
                 "embedding_time", "insertion_completed", "update_completed", "embedding_completed",
                 "n_inserted_instances", "n_update_changed_edges", "embedding_pending_edges",
                 "insertion_queue_size", "update_queue_size", "embedding_queue_size"):
        assert hasattr(_core.GPUMAPResult, name)
    for name in ("initialize", "append_data", "run", "close", "get_embedding", "get_neighbor_indices",
                 "get_neighbor_dists"):
        assert hasattr(_core.GPUMAP, name)


def test_invalid_params_rejected_before_device(native):
    # parameter validation happens before any CUDA call
    for kw in ({"n_components": 3}, {"n_neighbors": 33}, {"n_neighbors": 0}, {"metric": 7}, {"precision": 2},
               {"overlap": 2}):
        p = native.default_params(n_instances=10, n_features=4, **kw)
        with pytest.raises(ValueError):
            native.Session(p)


def test_python_package_exports():
    import gpumap_gb300 as gm

    assert set(gm.__all__) >= {"GPUMAP", "GPUMAPParams", "Metric", "BaseStrategy", "WeightedStrategy",
                               "SequentialPriorityStrategy", "Estimator", "MeanRateEstimator",
                               "DefaultLinearEstimator", "PersistentEstimator"}
