"""gm_op_sgd_noalloc: the SGD operator for callers that must not allocate.

Callers inside a framework whose memory pool owns the GPU, or in a loop that
cannot take cudaFree's device-wide synchronisation, call gm_op_sgd_noalloc,
which keeps its scratch in one fixed device array of the library instead of
cudaMalloc'd buffers.  These tests check it against gm_op_sgd, the operator
that allocates, on two calls in a row (the second one reuses the array the
first one left behind), and that it refuses edge lists beyond its array.

The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIG = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float,
       C.c_float, C.c_float, C.c_float, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p]
MAX_EDGES = 1048576  # GM_SGD_NOALLOC_MAX_EDGES


def _fn(lib, name):
    f = getattr(lib, name)
    f.restype = C.c_int
    f.argtypes = SIG
    return f


def _case(seed, n, nnz):
    # disjoint head/tail pairs and no negative samples: each epoch is free of
    # races, so both operators give the same bits
    rng = np.random.default_rng(seed)
    emb = rng.normal(size=(n, 2)).astype(np.float32)
    perm = rng.permutation(n).astype(np.int32)
    head, tail = perm[:nnz].copy(), perm[nnz:2 * nnz].copy()
    eps = rng.uniform(1.0, 6.0, size=nnz).astype(np.float32)
    return emb, head, tail, eps


def _run(fn, emb, head, tail, eps, n_epochs, stream_ptr, neg_rate=0):
    import torch

    dev = torch.device("cuda:0")
    te = torch.from_numpy(emb.copy()).to(dev)
    th, tt, tp = (torch.from_numpy(a).to(dev) for a in (head, tail, eps))
    rc = fn(te.data_ptr(), emb.shape[0], th.data_ptr(), tt.data_ptr(), tp.data_ptr(), head.shape[0],
            4.0, 1.0, 1.0, 1.58, 0.9, n_epochs, neg_rate, 42, stream_ptr)
    torch.cuda.synchronize()
    return rc, te.cpu().numpy()


def test_noalloc_sgd_matches_allocating_operator_twice(native):
    import torch

    lib = native.load()
    ref_fn, na_fn = _fn(lib, "gm_op_sgd"), _fn(lib, "gm_op_sgd_noalloc")
    stream = torch.cuda.current_stream().cuda_stream
    # first call larger than the second: its leftovers sit past the second's edges
    for seed, n, nnz, epochs in ((11, 4096, 1500, 60), (12, 1024, 512, 40)):
        emb, head, tail, eps = _case(seed, n, nnz)
        rc_ref, want = _run(ref_fn, emb, head, tail, eps, epochs, stream)
        rc_na, got = _run(na_fn, emb, head, tail, eps, epochs, stream)
        assert rc_ref == 0 and rc_na == 0, lib.gm_last_error()
        assert not np.array_equal(got, emb)  # the epochs moved the points
        assert np.array_equal(got, want)


def test_noalloc_sgd_single_edge_with_negative_samples(native):
    # one edge, five negative samples per sampling: one thread updates, so
    # both operators run the same sequence of operations and agree bit for bit
    import torch

    lib = native.load()
    ref_fn, na_fn = _fn(lib, "gm_op_sgd"), _fn(lib, "gm_op_sgd_noalloc")
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(21)
    emb = rng.normal(size=(2048, 2)).astype(np.float32)
    head, tail, eps = np.array([3], np.int32), np.array([1500], np.int32), np.array([1.0], np.float32)
    for _ in range(2):
        rc_ref, want = _run(ref_fn, emb, head, tail, eps, 200, stream, neg_rate=5)
        rc_na, got = _run(na_fn, emb, head, tail, eps, 200, stream, neg_rate=5)
        assert rc_ref == 0 and rc_na == 0, lib.gm_last_error()
        assert not np.array_equal(got, emb)
        assert np.array_equal(got, want)


def test_noalloc_sgd_with_races_agrees_statistically(native):
    # the 8-NN graph of a 6-cluster mixture (every row is the head of 8 edges
    # and the tail of others, so edges share rows) with negative samples:
    # Hogwild updates race, and the two operators visit the edges in
    # different orders (gm_op_sgd groups them by sampling period), so the
    # check is statistical: from a random start both reach the same
    # trustworthiness within 0.02, on two calls in a row.  (The sequential
    # oracle reaches 0.955 on this case.)
    import torch

    from gpumap_gb300.datasets import gaussian_mixture
    from oracle.knn import trustworthiness

    lib = native.load()
    ref_fn, na_fn = _fn(lib, "gm_op_sgd"), _fn(lib, "gm_op_sgd_noalloc")
    stream = torch.cuda.current_stream().cuda_stream
    n, deg = 3000, 8
    X, _ = gaussian_mixture(n, 8, n_centers=6, seed=31)
    x = X.astype(np.float64)
    sq = (x * x).sum(1)
    d = sq[:, None] + sq[None, :] - 2.0 * (x @ x.T)
    np.fill_diagonal(d, np.inf)
    nbr = np.argsort(d, axis=1)[:, :deg]
    head = np.repeat(np.arange(n, dtype=np.int32), deg)
    tail = nbr.reshape(-1).astype(np.int32)
    rng = np.random.default_rng(31)
    eps = rng.uniform(1.0, 4.0, size=head.shape[0]).astype(np.float32)
    emb = rng.normal(size=(n, 2)).astype(np.float32)
    sample = np.arange(0, n, 3)
    start = trustworthiness(X, emb, deg, sample=sample)
    for _ in range(2):
        rc_ref, want = _run(ref_fn, emb, head, tail, eps, 100, stream, neg_rate=5)
        rc_na, got = _run(na_fn, emb, head, tail, eps, 100, stream, neg_rate=5)
        assert rc_ref == 0 and rc_na == 0, lib.gm_last_error()
        assert np.all(np.isfinite(got))
        t_ref = trustworthiness(X, want, deg, sample=sample)
        t_na = trustworthiness(X, got, deg, sample=sample)
        assert t_ref > start + 0.3 and t_na > start + 0.3, (start, t_ref, t_na)
        assert abs(t_ref - t_na) <= 0.02, (t_ref, t_na)


def test_noalloc_sgd_rejects_oversized_edge_list(native):
    lib = native.load()
    fn = _fn(lib, "gm_op_sgd_noalloc")
    lib.gm_last_error.restype = C.c_char_p
    rc = fn(None, 10, None, None, None, MAX_EDGES + 1, 4.0, 1.0, 1.0, 1.58, 0.9, 10, 5, 42, None)
    assert rc == native.GM_ERR_INVALID
    assert b"1048576" in lib.gm_last_error()
