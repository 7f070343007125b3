"""ctypes wrapper for the oracle library (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import build_oracle, lib_path

_lib = None
_P = C.c_void_p


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        build_oracle()
    lib = C.CDLL(str(p))
    sig = {
        "gmo_create": (_P, [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                            C.c_int]),
        "gmo_destroy": (None, [_P]),
        "gmo_append": (C.c_int, [_P, _P, C.c_uint64, C.c_uint64]),
        "gmo_run": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
        "gmo_copy": (C.c_int, [_P, C.c_int, _P, C.c_uint64]),
        "gmo_size": (C.c_uint64, [_P, C.c_int]),
        "gmo_scalars": (C.c_int, [_P, _P, C.c_int]),
        "gmo_update_queue": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
        "gmo_fuzzy_schedule": (C.c_int, [_P, _P, C.c_int64, C.c_int32, C.c_int32, _P, C.c_int64, C.c_int32,
                                         C.c_float, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
        "gmo_sgd": (C.c_int, [_P, C.c_int64, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float,
                              C.c_float, C.c_float, C.c_int32, C.c_int32, C.c_uint64]),
        "gmo_queue_script": (C.c_int, [C.c_char_p, C.c_uint64]),
        "gmo_expf": (C.c_float, [C.c_float]),
        "gmo_logf": (C.c_float, [C.c_float]),
        "gmo_powf": (C.c_float, [C.c_float, C.c_float]),
        "gmo_philox": (None, [_P, C.c_uint32, C.c_uint32]),
        "gmo_bloom_hash": (C.c_uint32, [C.c_int, C.c_uint32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


RESULT_FIELDS = [
    "n_insertion_ops", "n_update_ops", "n_embedding_ops", "insertion_completed", "update_completed",
    "embedding_completed", "n_inserted_instances", "n_update_changed_edges", "embedding_pending_edges",
    "insertion_queue_size", "update_queue_size", "embedding_queue_size",
]

# Buffer ids shared with include/gpumap_gb300_ops.h, plus oracle-only tables.
BUF = {"graph_ids": 0, "graph_dists": 1, "knn_ids": 2, "knn_dists": 3, "norms": 4, "bloom": 5,
       "sigma": 6, "rho": 7, "coo_row": 8, "coo_col": 9, "coo_val": 10, "sched_row": 11,
       "sched_col": 12, "sched_eps": 13, "x": 14, "pub_idx": 15, "pub_dist": 16, "embedding": 17}


class OracleSession:
    def __init__(self, n_instances, n_features, k=15, metric=0, a=1.0, b=1.0, alpha=1.0,
                 negative_sample_rate=5, max_epoch=200, precision=0):
        self._lib = load()
        self.n_instances, self.n_features, self.k = n_instances, n_features, k
        self._h = self._lib.gmo_create(n_instances, n_features, k, metric, a, b, alpha,
                                       negative_sample_rate, max_epoch, precision)
        if not self._h:
            raise ValueError("bad oracle parameters")
        self.ld = (n_features + 3) // 4 * 4

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gmo_destroy(self._h)
            self._h = None

    def append(self, x):
        a = np.ascontiguousarray(x, dtype=np.float32)
        rc = self._lib.gmo_append(self._h, a.ctypes.data, a.shape[0], a.shape[1])
        if rc:
            raise RuntimeError(f"oracle append failed ({rc})")

    def run(self, ni, nu, ne) -> dict:
        out = np.zeros(15, dtype=np.int64)
        self._lib.gmo_run(self._h, ni, nu, ne, out.ctypes.data)
        return dict(zip(RESULT_FIELDS, out[: len(RESULT_FIELDS)].tolist()))

    def copy(self, which: str, dtype):
        bid = BUF[which]
        N = max(self.n_instances, 1)
        sizes = {0: N * 32, 1: N * 32, 2: N * self.k, 3: N * self.k, 4: N, 5: N * 64, 14: N * self.ld,
                 15: N * (self.k + 1), 16: N * (self.k + 1), 17: N * 2}
        n = sizes[bid] if bid in sizes else self._lib.gmo_size(self._h, bid) // 4
        out = np.empty(n, dtype=dtype)
        rc = self._lib.gmo_copy(self._h, bid, out.ctypes.data, n * 4)
        if rc:
            raise RuntimeError("oracle copy failed")
        return out

    def scalars(self):
        out = np.zeros(11, dtype=np.int64)
        self._lib.gmo_scalars(self._h, out.ctypes.data, 11)
        return out.tolist()

    def update_queue(self):
        n = C.c_uint64()
        self._lib.gmo_update_queue(self._h, None, 0, C.byref(n))
        out = np.empty(n.value, dtype=np.uint32)
        self._lib.gmo_update_queue(self._h, out.ctypes.data, n.value, C.byref(n))
        return out

    def neighbor_indices(self, n):
        return self.copy("pub_idx", np.uint32).reshape(-1, self.k + 1)[:n, : self.k]

    def neighbor_dists(self, n):
        return self.copy("pub_dist", np.float32).reshape(-1, self.k + 1)[:n, : self.k]

    def embedding(self, n):
        return self.copy("embedding", np.float32).reshape(-1, 2)[:n]


def queue_script() -> str:
    buf = C.create_string_buffer(1 << 20)
    n = load().gmo_queue_script(buf, len(buf))
    if n < 0:
        raise RuntimeError("queue script output too large")
    return buf.value.decode()


def fuzzy_schedule(pub_idx, pub_dist, k, euclidean, batch, n_epochs=200, alpha=1.0):
    lib = load()
    pub_idx = np.ascontiguousarray(pub_idx, dtype=np.uint32)
    pub_dist = np.ascontiguousarray(pub_dist, dtype=np.float32)
    batch = np.ascontiguousarray(batch, dtype=np.int32)
    n = pub_idx.shape[0]
    nb = batch.shape[0]
    cap = max(2 * nb * k, 1)
    cr, cc, tr, tc = (np.zeros(cap, np.int32) for _ in range(4))
    cv, te = np.zeros(cap, np.float32), np.zeros(cap, np.float32)
    sg, rh = np.zeros(max(n, 1), np.float32), np.zeros(max(n, 1), np.float32)
    counts = np.zeros(4, np.int64)
    scal = np.zeros(3, np.float32)
    lib.gmo_fuzzy_schedule(pub_idx.ctypes.data, pub_dist.ctypes.data, n, k, 1 if euclidean else 0,
                           batch.ctypes.data, nb, n_epochs, alpha, cr.ctypes.data, cc.ctypes.data,
                           cv.ctypes.data, tr.ctypes.data, tc.ctypes.data, te.ctypes.data, sg.ctypes.data,
                           rh.ctypes.data, counts.ctypes.data, scal.ctypes.data)
    nnz, nnz2 = int(counts[0]), int(counts[2])
    return dict(coo_row=cr[:nnz], coo_col=cc[:nnz], coo_val=cv[:nnz], t_row=tr[:nnz2], t_col=tc[:nnz2],
                t_eps=te[:nnz2], sigma=sg[:n], rho=rh[:n], nnz=nnz, extras=int(counts[1]), nnz2=nnz2,
                max_deg=int(counts[3]), mean=float(scal[0]), max_w=float(scal[1]), rounding=float(scal[2]))


def sgd(emb, head, tail, eps, rounding, alpha0=1.0, gamma=1.0, a=1.0, b=1.0, n_epochs=200,
        negative_sample_rate=5, seed=42):
    lib = load()
    emb = np.ascontiguousarray(emb, dtype=np.float32).copy()
    head = np.ascontiguousarray(head, dtype=np.int32)
    tail = np.ascontiguousarray(tail, dtype=np.int32)
    eps = np.ascontiguousarray(eps, dtype=np.float32)
    lib.gmo_sgd(emb.ctypes.data, emb.shape[0], head.ctypes.data, tail.ctypes.data, eps.ctypes.data,
                head.shape[0], rounding, alpha0, gamma, a, b, n_epochs, negative_sample_rate, seed)
    return emb
