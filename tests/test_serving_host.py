"""Host-side logic of the served and batched workloads (no GPU): the seeded
workload generators and the trace replayer, the latter against a stand-in
server that records what it is given."""
import threading
import time

import numpy as np

from gpumap_gb300.datasets import mixture_stream, poisson_trace, session_specs
from gpumap_gb300.serving import ReplayResult, RequestRecord, TraceRequest, replay


def test_session_specs_are_seeded_and_in_range():
    a = session_specs(16, 20_000, 500_000, (64, 784), seed=0)
    b = session_specs(16, 20_000, 500_000, (64, 784), seed=0)
    assert a == b
    assert all(20_000 <= s["n"] <= 500_000 and 64 <= s["d"] <= 784 and 5 <= s["centers"] <= 20 for s in a)
    c = session_specs(64, 2_000, 200_000, [32, 128, 784], seed=0)
    assert {s["d"] for s in c} <= {32, 128, 784} and [s["seed"] for s in c] == list(range(64))


def test_poisson_trace_respects_sizes_and_rate():
    specs = session_specs(4, 3_000, 6_000, [16], seed=2)
    tr = poisson_trace(specs, rate=100.0, duration=20.0, rows_lo=500, rows_hi=5000, seed=3)
    per = [0] * len(specs)
    for t, i, r in tr:
        assert 0 < r <= 5000 and 0 <= t <= 20.0
        per[i] += r
    assert all(p <= s["n"] for p, s in zip(per, specs))
    # the sessions fill up long before 20 s at 100 requests per second
    assert sum(per) == sum(s["n"] for s in specs)
    ts = [t for t, _, _ in tr]
    assert ts == sorted(ts)
    big = [{"n": 10**9}]
    tr2 = poisson_trace(big, rate=40.0, duration=50.0, rows_lo=1, rows_hi=1, seed=4)
    assert abs(len(tr2) / 50.0 - 40.0) < 4.0  # Poisson count: mean 2000, sd ~45


def test_mixture_stream_prefix_is_stable():
    full = np.concatenate(list(mixture_stream(20_000, 12, 5, seed=9)))
    again = np.concatenate(list(mixture_stream(20_000, 12, 5, seed=9)))
    np.testing.assert_array_equal(full, again)
    assert full.shape == (20_000, 12) and full.dtype == np.float32


class _FakeServer:
    """Runs each request for a fixed time on one background thread."""

    def __init__(self, service_s):
        self.service_s = service_s
        self.lock = threading.Lock()
        self.submitted = []
        self.done = {}
        self.next = 1
        self.busy_until = 0.0

    def submit(self, sid, rows, n_upd, n_emb):
        with self.lock:
            rid = self.next
            self.next += 1
            now = time.perf_counter()
            start = max(now, self.busy_until)
            self.busy_until = start + self.service_s
            self.submitted.append((sid, len(rows), n_upd, n_emb))
            self.done[rid] = (sid, len(rows), now, start, self.busy_until)
            return rid

    def wait(self, rid):
        sid, rows, ta, ts, te = self.done.pop(rid)
        while time.perf_counter() < te:
            time.sleep(0.001)

        class Info:
            pass

        info = Info()
        info.rows, info.status, info.t_arrive, info.t_start, info.t_end = rows, 0, ta, ts, te
        return info


def test_replay_submits_in_order_and_collects_every_request():
    rows = np.zeros((10, 3), np.float32)
    trace = [TraceRequest(0.01 * i, i % 2, rows[: 1 + i % 3], 7, 9) for i in range(12)]
    srv = _FakeServer(service_s=0.002)
    res = replay(srv, [100, 200], trace, timed=True)
    assert [s for s, *_ in srv.submitted] == [100 if i % 2 == 0 else 200 for i in range(12)]
    assert [r for _, r, _, _ in srv.submitted] == [1 + i % 3 for i in range(12)]
    assert len(res.records) == 12 and all(r.status == 0 for r in res.records)
    assert res.wall_s >= 0.11
    s = res.summary()
    assert s["requests"] == 12 and s["failed"] == 0 and s["rows"] == sum(1 + i % 3 for i in range(12))
    assert s["latency_p99_ms"] >= s["latency_p50_ms"] >= 2.0 * 0.9


def test_replay_summary_percentiles():
    r = ReplayResult(records=[RequestRecord(0, 10, 0, 0.0, 0.0, float(i)) for i in range(1, 101)])
    s = r.summary()
    assert abs(s["latency_p50_ms"] - 50500.0) < 1.0 and s["latency_max_ms"] == 100000.0
