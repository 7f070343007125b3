"""ctypes view of the C ABI (include/gpumap_gb300.h, include/gpumap_gb300_ops.h).

Loads the in-tree ``_lib/libgpumap_gb300.so``.  There is no fallback: if the
library is missing this raises ``ImportError`` telling the caller to build it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgpumap_gb300.so"

GM_OK = 0
GM_ERR_INVALID = -1
GM_ERR_RUNTIME = -2
GM_ERR_CAPACITY = -3
GM_ERR_OOM = -4
GM_ERR_CUDA = -5
GM_ERR_DEVICE = -6
GM_ERR_CLOSED = -7

GM_BUF = {
    "graph_ids": 0, "graph_dists": 1, "knn_ids": 2, "knn_dists": 3, "norms": 4, "bloom": 5,
    "sigma": 6, "rho": 7, "coo_row": 8, "coo_col": 9, "coo_val": 10, "sched_row": 11,
    "sched_col": 12, "sched_eps": 13, "x": 14, "pub_idx": 15, "pub_dist": 16, "embedding": 17, "exact_d": 18,
}


class gm_params(C.Structure):
    _fields_ = [
        ("n_neighbors", C.c_uint64), ("n_components", C.c_uint64), ("min_dist", C.c_float),
        ("negative_sample_rate", C.c_uint64), ("max_epoch", C.c_uint64), ("a", C.c_float),
        ("b", C.c_float), ("alpha", C.c_float), ("verbose", C.c_int32), ("metric", C.c_int32),
        ("n_instances", C.c_uint64), ("n_features", C.c_uint64), ("precision", C.c_int32),
        ("device", C.c_int32), ("overlap", C.c_int32),
    ]


class gm_result(C.Structure):
    _fields_ = [
        ("n_insertion_ops", C.c_uint32), ("n_update_ops", C.c_uint32), ("n_embedding_ops", C.c_uint32),
        ("insertion_time", C.c_float), ("update_time", C.c_float), ("embedding_time", C.c_float),
        ("insertion_completed", C.c_uint8), ("update_completed", C.c_uint8),
        ("embedding_completed", C.c_uint8), ("n_inserted_instances", C.c_uint64),
        ("n_update_changed_edges", C.c_uint64), ("embedding_pending_edges", C.c_uint64),
        ("insertion_queue_size", C.c_uint64), ("update_queue_size", C.c_uint64),
        ("embedding_queue_size", C.c_uint64),
    ]


class gm_view(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("rows", C.c_uint64), ("cols", C.c_uint64),
                ("row_stride_bytes", C.c_uint64), ("dtype", C.c_int32)]


class gm_stats(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_uint64), ("join_launches", C.c_uint64), ("join_ms", C.c_double),
        ("join_nodes", C.c_uint64), ("join_rows", C.c_uint64), ("join_pairs", C.c_uint64),
        ("join_merges", C.c_uint64), ("cand_launches", C.c_uint64), ("cand_ms", C.c_double),
        ("cand_rows", C.c_uint64), ("sgd_launches", C.c_uint64), ("sgd_ms", C.c_double),
        ("sgd_edges", C.c_uint64), ("sgd_negatives", C.c_uint64),
        ("exact_launches", C.c_uint64), ("exact_ms", C.c_double), ("exact_flops", C.c_double),
        ("screen_ms", C.c_double), ("exact_pairs", C.c_uint64), ("exact_rescored", C.c_uint64),
        ("phase_s", C.c_double * 3),
        ("exact_overflow_blocks", C.c_uint64),
    ]


# (name, restype, argtypes) for every exported entry point.
_P = C.c_void_p
_SIGS = [
    ("gm_params_default", C.c_int, [C.POINTER(gm_params)]),
    ("gm_create", C.c_int, [C.POINTER(gm_params), C.POINTER(_P)]),
    ("gm_initialize", C.c_int, [_P, C.c_uint64, C.c_uint64]),
    ("gm_append", C.c_int, [_P, _P, C.c_uint64, C.c_uint64]),
    ("gm_append_device", C.c_int, [_P, _P, C.c_uint64, C.c_uint64]),
    ("gm_run", C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(gm_result)]),
    ("gm_get_embedding", C.c_int, [_P, C.POINTER(gm_view)]),
    ("gm_get_neighbor_indices", C.c_int, [_P, C.POINTER(gm_view)]),
    ("gm_get_neighbor_dists", C.c_int, [_P, C.POINTER(gm_view)]),
    ("gm_get_stream", C.c_int, [_P, C.POINTER(_P)]),
    ("gm_stream_wait", C.c_int, [_P, _P]),
    ("gm_get_device", C.c_int, [_P, C.POINTER(C.c_int32)]),
    ("gm_close", C.c_int, [_P]),
    ("gm_destroy", None, [_P]),
    ("gm_last_error", C.c_char_p, []),
    ("gm_set_stats", C.c_int, [_P, C.c_int]),
    ("gm_get_stats", C.c_int, [_P, C.POINTER(gm_stats)]),
    ("gm_debug_buffer_size", C.c_int, [_P, C.c_int, C.POINTER(C.c_uint64)]),
    ("gm_debug_copy", C.c_int, [_P, C.c_int, _P, C.c_uint64]),
    ("gm_debug_keep_tiles", C.c_int, [_P, C.c_int]),
    ("gm_debug_pre_capacity", C.c_int, [_P, C.c_int]),
    ("gm_debug_scalars", C.c_int, [_P, C.POINTER(C.c_int64), C.c_int]),
    ("gm_debug_update_queue", C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("gm_op_fuzzy_schedule", C.c_int,
     [_P, _P, C.c_int64, C.c_int32, C.c_int32, _P, C.c_int64, C.c_int32, C.c_float, _P, _P, _P,
      _P, _P, _P, _P, _P, C.POINTER(C.c_int64), C.POINTER(C.c_float), _P]),
    ("gm_op_sgd", C.c_int,
     [_P, C.c_int64, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float,
      C.c_float, C.c_int32, C.c_int32, C.c_uint64, _P]),
]

_lib = None


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    """Loads the native library (once) and declares every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise ImportError(
            f"gpumap_gb300 native library not built: {_LIB_PATH} is missing; "
            "run `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(str(_LIB_PATH))
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def check(rc: int) -> None:
    if rc != GM_OK:
        msg = (load().gm_last_error() or b"").decode(errors="replace")
        if rc == GM_ERR_INVALID:
            raise ValueError(msg)
        if rc == GM_ERR_OOM:
            raise MemoryError(msg)
        raise GMError(rc, msg or f"gpumap_gb300 error {rc}")


def default_params(**kw) -> gm_params:
    p = gm_params()
    check(load().gm_params_default(C.byref(p)))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


class Session:
    """Thin owner of a ``gm_session*`` for tests and the benchmark."""

    def __init__(self, params: gm_params):
        self._lib = load()
        self._h = C.c_void_p()
        check(self._lib.gm_create(C.byref(params), C.byref(self._h)))
        self.params = params

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gm_destroy(h)
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def append_host(self, arr) -> None:
        import numpy as np

        a = np.ascontiguousarray(arr, dtype=np.float32)
        check(self._lib.gm_append(self._h, a.ctypes.data, a.shape[0], a.shape[1]))

    def append_device(self, ptr: int, rows: int, cols: int) -> None:
        check(self._lib.gm_append_device(self._h, C.c_void_p(ptr), rows, cols))

    def run(self, ni: int, nu: int, ne: int) -> gm_result:
        r = gm_result()
        check(self._lib.gm_run(self._h, ni, nu, ne, C.byref(r)))
        return r

    def view(self, which: str) -> gm_view:
        v = gm_view()
        fn = {"embedding": self._lib.gm_get_embedding, "indices": self._lib.gm_get_neighbor_indices,
              "dists": self._lib.gm_get_neighbor_dists}[which]
        check(fn(self._h, C.byref(v)))
        return v

    def stream(self) -> int:
        s = C.c_void_p()
        check(self._lib.gm_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def close(self) -> None:
        check(self._lib.gm_close(self._h))

    def keep_tiles(self, on: bool) -> None:
        check(self._lib.gm_debug_keep_tiles(self._h, 1 if on else 0))

    def pre_capacity(self, cap: int) -> None:
        check(self._lib.gm_debug_pre_capacity(self._h, int(cap)))

    def set_stats(self, on: bool) -> None:
        check(self._lib.gm_set_stats(self._h, 1 if on else 0))

    def stats(self) -> gm_stats:
        st = gm_stats()
        check(self._lib.gm_get_stats(self._h, C.byref(st)))
        return st

    def copy(self, which: str, dtype, count: int | None = None):
        import numpy as np

        nbytes = C.c_uint64()
        check(self._lib.gm_debug_buffer_size(self._h, GM_BUF[which], C.byref(nbytes)))
        n = nbytes.value // 4 if count is None else count
        out = np.empty(n, dtype=dtype)
        check(self._lib.gm_debug_copy(self._h, GM_BUF[which], out.ctypes.data, n * 4))
        return out

    def scalars(self):
        out = (C.c_int64 * 11)()
        check(self._lib.gm_debug_scalars(self._h, out, 11))
        return list(out)

    def update_queue(self):
        import numpy as np

        n = C.c_uint64()
        check(self._lib.gm_debug_update_queue(self._h, None, 0, C.byref(n)))
        out = np.empty(n.value, dtype=np.uint32)
        check(self._lib.gm_debug_update_queue(self._h, out.ctypes.data, n.value, C.byref(n)))
        return out
