"""The Python surface (gpumap_gb300.GPUMAP over the pybind11 module) on the GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(n=3000, d=16, k=15, seed=0, **kw):
    import gpumap_gb300 as gm
    from gpumap_gb300.data_loader import ArrayDataLoader
    from gpumap_gb300.datasets import gaussian_mixture

    X, _ = gaussian_mixture(n, d, seed=seed)
    p = gm.GPUMAPParams()
    p.n_instances, p.n_features, p.n_neighbors = n, d, k
    p.max_epoch = 50
    for key, v in kw.items():
        setattr(p, key, v)
    return X, gm.GPUMAP(ArrayDataLoader(X), p)


def test_run_with_n_ops_views():
    import torch

    X, m = _model()
    res = None
    for _ in range(6):
        res = m.run_with_n_ops(500, 1500, 800)
    assert res.n_inserted_instances == 3000 and res.insertion_completed
    assert m.n_inserted_instances == 3000
    emb, idx, dst = m.get_embedding(), m.get_neighbor_indices(), m.get_neighbor_dists()
    assert tuple(emb.shape) == (3000, 2) and tuple(idx.shape) == (3000, 15) and tuple(dst.shape) == (3000, 15)
    assert isinstance(emb, torch.Tensor) and emb.is_cuda
    assert torch.isfinite(emb).all()
    i64 = idx.to(torch.int64).cpu().numpy()
    assert np.all((i64 >= 0) & (i64 < 3000))
    # dists are squared L2 of the listed ids; random initial neighbours not yet
    # re-scored stay at FLT_MAX, as in the reference
    d2 = ((X[:, None, :].astype(np.float64) - X[i64].astype(np.float64)) ** 2).sum(-1)
    dn = dst.cpu().numpy()
    real = dn < np.finfo(np.float32).max
    assert real.mean() > 0.9
    assert np.max(np.abs(dn[real] - d2[real]) / np.maximum(d2[real], 1e-3)) < 1e-4
    m.close()


def test_run_with_target_latency_and_strategy():
    import gpumap_gb300 as gm
    from gpumap_gb300.data_loader import ArrayDataLoader
    from gpumap_gb300.datasets import gaussian_mixture

    X, _ = gaussian_mixture(4000, 8, seed=2)
    p = gm.GPUMAPParams()
    p.n_instances, p.n_features = 4000, 8
    p.max_epoch = 20
    m = gm.GPUMAP(ArrayDataLoader(X), p, strategy=gm.SequentialPriorityStrategy(n_instances=4000))
    res = m.run(0.5)
    assert res.n_inserted_instances == 4000 and res.insertion_completed  # whole budget to insertion
    res = m.run(0.5)
    assert res.n_update_ops > 0 and res.n_insertion_ops == 0
    m.close()
    m2 = gm.GPUMAP(ArrayDataLoader(X), p)
    for _ in range(3):
        r = m2.run(0.2)
        assert r.n_insertion_ops >= min(500, 4000)
    assert 0.0 < m2.strategy.get_progress()[0] <= 1.0
    m2.close()


def test_append_validation_errors():
    import gpumap_gb300 as gm

    p = gm.GPUMAPParams()
    p.n_instances, p.n_features = 10, 4
    core = gm._core.GPUMAP(p)
    with pytest.raises(RuntimeError, match="2D"):
        core.append_data(np.zeros(4, np.float32))
    with pytest.raises(RuntimeError, match="float32"):
        core.append_data(np.zeros((2, 4), np.float64))
    with pytest.raises(RuntimeError, match="C-contiguous"):
        core.append_data(np.zeros((4, 8), np.float32)[:, ::2])
    with pytest.raises(RuntimeError, match="n_features"):
        core.append_data(np.zeros((2, 5), np.float32))
    core.append_data(np.zeros((10, 4), np.float32))
    with pytest.raises(RuntimeError, match="Exceeding"):
        core.append_data(np.zeros((1, 4), np.float32))
    from gpumap_gb300.data_loader import ArrayDataLoader

    p2 = gm.GPUMAPParams()
    p2.min_dist = 1.5
    with pytest.raises(ValueError, match="min_dist"):
        gm.GPUMAP(ArrayDataLoader(np.zeros((3, 4), np.float32)), p2)
    cai = core.get_neighbor_indices().__cuda_array_interface__
    assert cai["shape"] == (10, 16) and cai["typestr"] == "<u4" and cai["data"][1] is True


@pytest.mark.parametrize("precision", [0, 1])
def test_overlap_through_python_api(precision):
    # overlap = 1 from Python: the k-NN tables equal the non-overlapped
    # build's, get_embedding waits for the embedding still in flight
    import torch

    X, a = _model(n=2000, d=24, seed=5, precision=precision, overlap=1)
    _, b = _model(n=2000, d=24, seed=5, precision=precision, overlap=0)
    assert a.params.overlap == 1
    for _ in range(4):
        a.run_with_n_ops(500, 300, 600)
        b.run_with_n_ops(500, 300, 600)
    emb = a.get_embedding()
    assert tuple(emb.shape) == (2000, 2) and torch.isfinite(emb).all()
    assert torch.equal(a.get_neighbor_indices(), b.get_neighbor_indices())
    assert torch.equal(a.get_neighbor_dists(), b.get_neighbor_dists())
    a.close()
    b.close()


def test_views_carry_stream_and_dlpack():
    # the views keep the reference's interface (read-only CAI v3, full
    # capacity, k+1 columns) and add the producing stream and DLPack; a
    # consumer on another stream is ordered after the session's work
    import torch

    from gpumap_gb300 import _core
    from gpumap_gb300.datasets import gaussian_mixture

    n, d, k = 2000, 16, 10
    X, _ = gaussian_mixture(n, d, seed=4)
    p = _core.GPUMAPParams()
    p.n_instances, p.n_features, p.n_neighbors, p.max_epoch = n, d, k, 30
    p.precision, p.overlap = 1, 1
    core = _core.GPUMAP(p)
    core.append_data(X)
    core.run(n, 0, n)
    for getter, typestr in ((core.get_neighbor_indices, "<u4"), (core.get_neighbor_dists, "<f4"),
                            (core.get_embedding, "<f4")):
        v = getter()
        cai = v.__cuda_array_interface__
        assert cai["typestr"] == typestr and cai["data"][1] is True and cai["version"] == 3
        assert cai["stream"] not in (0, None)
        assert v.__dlpack_device__() == (2, torch.cuda.current_device())
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            t = torch.from_dlpack(v)
            via_dl = t.clone()
        side.synchronize()
        holder = type("H", (), {})()
        holder.__cuda_array_interface__ = dict(cai, data=(cai["data"][0], False))
        via_cai = torch.as_tensor(holder, device="cuda")
        assert tuple(via_dl.shape) == tuple(cai["shape"])
        assert torch.equal(via_dl.view(torch.int32) if typestr == "<u4" else via_dl,
                           via_cai.view(torch.int32) if typestr == "<u4" else via_cai)
    # the DLPack tensor keeps the model alive
    t = torch.from_dlpack(core.get_embedding())
    del core
    assert torch.isfinite(t[:n]).all()
