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


def _run(fn, emb, head, tail, eps, n_epochs, stream_ptr):
    import torch

    dev = torch.device("cuda:0")
    te = torch.from_numpy(emb.copy()).to(dev)
    th, tt, tp = (torch.from_numpy(a).to(dev) for a in (head, tail, eps))
    rc = fn(te.data_ptr(), emb.shape[0], th.data_ptr(), tt.data_ptr(), tp.data_ptr(), head.shape[0],
            4.0, 1.0, 1.0, 1.58, 0.9, n_epochs, 0, 42, stream_ptr)
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


def test_noalloc_sgd_rejects_oversized_edge_list(native):
    lib = native.load()
    fn = _fn(lib, "gm_op_sgd_noalloc")
    lib.gm_last_error.restype = C.c_char_p
    rc = fn(None, 10, None, None, None, MAX_EDGES + 1, 4.0, 1.0, 1.0, 1.58, 0.9, 10, 5, 42, None)
    assert rc == native.GM_ERR_INVALID
    assert b"1048576" in lib.gm_last_error()
