"""Serving many progressive sessions on one GPU (include/gpumap_gb300_server.h).

``Server`` wraps the C ABI: sessions are opened against a device-memory
budget, insertion requests are queued with ``submit`` and run by ``slots``
worker threads, one request per session at a time, the cycles of different
sessions overlapping on the GPU.  ``replay`` plays a timed request trace
against a server from a submitting thread (each request is submitted at its
arrival time) and returns every request's record.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native


class gm_server_params(C.Structure):
    _fields_ = [("device", C.c_int32), ("slots", C.c_int32), ("hbm_budget", C.c_uint64)]


class gm_request_info(C.Structure):
    _fields_ = [("request", C.c_uint64), ("session", C.c_uint32), ("status", C.c_int32),
                ("rows", C.c_uint64), ("t_arrive", C.c_double), ("t_start", C.c_double),
                ("t_end", C.c_double), ("result", _native.gm_result)]


class gm_server_stats(C.Structure):
    _fields_ = [("finished", C.c_uint64), ("failed", C.c_uint64), ("rows", C.c_uint64),
                ("sessions_open", C.c_uint64), ("bytes_in_use", C.c_uint64),
                ("first_arrive", C.c_double), ("last_end", C.c_double),
                ("latency_p50", C.c_double), ("latency_p99", C.c_double), ("latency_max", C.c_double),
                ("service_p50", C.c_double), ("service_p99", C.c_double)]


_P = C.c_void_p
_SIGS = [
    ("gm_server_create", C.c_int, [C.POINTER(gm_server_params), C.POINTER(_P)]),
    ("gm_server_destroy", None, [_P]),
    ("gm_server_open_session", C.c_int, [_P, C.POINTER(_native.gm_params), C.POINTER(C.c_uint32)]),
    ("gm_server_close_session", C.c_int, [_P, C.c_uint32]),
    ("gm_server_submit", C.c_int, [_P, C.c_uint32, _P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                   C.POINTER(C.c_uint64)]),
    ("gm_server_wait", C.c_int, [_P, C.c_uint64, C.POINTER(gm_request_info)]),
    ("gm_server_drain", C.c_int, [_P]),
    ("gm_server_session_handle", C.c_int, [_P, C.c_uint32, C.POINTER(_P)]),
    ("gm_server_get_stats", C.c_int, [_P, C.POINTER(gm_server_stats)]),
]


def _lib():
    lib = _native.load()
    if not getattr(lib, "_server_sigs", False):
        for name, res, args in _SIGS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._server_sigs = True
    return lib


class BorrowedSession(_native.Session):
    """A server session's engine handle (debug copies, result views); the
    server owns it."""

    def __init__(self, handle: C.c_void_p, params):  # noqa: D107 - no engine of its own
        self._lib = _native.load()
        self._h = handle
        self.params = params

    def __del__(self):
        pass


class Server:
    def __init__(self, slots: int = 4, hbm_budget: int = 150 * 10**9, device: int = 0):
        self._lib = _lib()
        p = gm_server_params(device, slots, hbm_budget)
        self._h = C.c_void_p()
        _native.check(self._lib.gm_server_create(C.byref(p), C.byref(self._h)))
        self._params = {}

    def close(self):
        if self._h is not None and self._h.value:
            self._lib.gm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def open_session(self, params) -> int:
        sid = C.c_uint32()
        _native.check(self._lib.gm_server_open_session(self._h, C.byref(params), C.byref(sid)))
        self._params[sid.value] = params
        return sid.value

    def close_session(self, sid: int) -> None:
        _native.check(self._lib.gm_server_close_session(self._h, sid))
        self._params.pop(sid, None)

    def submit(self, sid: int, rows: np.ndarray, n_update_ops: int, n_embedding_ops: int) -> int:
        a = np.ascontiguousarray(rows, dtype=np.float32)
        rid = C.c_uint64()
        _native.check(self._lib.gm_server_submit(self._h, sid, a.ctypes.data, a.shape[0], a.shape[1],
                                                 n_update_ops, n_embedding_ops, C.byref(rid)))
        return rid.value

    def wait(self, rid: int) -> gm_request_info:
        info = gm_request_info()
        _native.check(self._lib.gm_server_wait(self._h, rid, C.byref(info)))
        return info

    def drain(self) -> None:
        _native.check(self._lib.gm_server_drain(self._h))

    def session(self, sid: int) -> BorrowedSession:
        h = C.c_void_p()
        _native.check(self._lib.gm_server_session_handle(self._h, sid, C.byref(h)))
        return BorrowedSession(h, self._params[sid])

    def stats(self) -> gm_server_stats:
        st = gm_server_stats()
        _native.check(self._lib.gm_server_get_stats(self._h, C.byref(st)))
        return st


@dataclass
class TraceRequest:
    t: float          # arrival, seconds after the start of the replay
    session: int      # index into the trace's sessions
    rows: np.ndarray  # float32 rows to insert
    n_update_ops: int
    n_embedding_ops: int


@dataclass
class RequestRecord:
    session: int
    rows: int
    status: int
    t_arrive: float
    t_start: float
    t_end: float

    @property
    def latency(self) -> float:
        return self.t_end - self.t_arrive


@dataclass
class ReplayResult:
    records: list = field(default_factory=list)
    wall_s: float = 0.0

    def latencies(self) -> np.ndarray:
        return np.array([r.latency for r in self.records if r.status == 0])

    def summary(self) -> dict:
        lat = self.latencies()
        ok = [r for r in self.records if r.status == 0]
        rows = sum(r.rows for r in ok)
        span = (max(r.t_end for r in ok) - min(r.t_arrive for r in ok)) if ok else 0.0
        return {"requests": len(self.records), "failed": len(self.records) - len(ok), "rows": rows,
                "latency_p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
                "latency_p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
                "latency_max_ms": float(lat.max() * 1e3) if len(lat) else None,
                "points_per_s": rows / span if span > 0 else None, "span_s": span}


def replay(server: Server, session_ids: list, trace: list, timed: bool = True) -> ReplayResult:
    """Submits every request of ``trace`` (sorted by arrival) at its arrival
    time (all at once when ``timed`` is false) from this thread, while a
    second thread waits for them in submission order."""
    ids: list = []
    lock = threading.Condition()
    done = {"n": 0}
    out = ReplayResult()

    def waiter():
        i = 0
        while True:
            with lock:
                while i >= len(ids) and done["n"] == 0:
                    lock.wait()
                if i >= len(ids):
                    return
                rid, req = ids[i]
            info = server.wait(rid)
            out.records.append(RequestRecord(req.session, int(info.rows), int(info.status), info.t_arrive,
                                             info.t_start, info.t_end))
            i += 1

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    t0 = time.perf_counter()
    for req in trace:
        if timed:
            delay = req.t - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
        rid = server.submit(session_ids[req.session], req.rows, req.n_update_ops, req.n_embedding_ops)
        with lock:
            ids.append((rid, req))
            lock.notify()
    with lock:
        done["n"] = 1
        lock.notify()
    th.join()
    out.wall_s = time.perf_counter() - t0
    return out
