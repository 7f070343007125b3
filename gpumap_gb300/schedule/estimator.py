"""Per-operation cost models for the latency scheduler.

An estimator learns, from (ops, seconds) samples of one engine operation,
how many ops fit a time budget at a given confidence and how long a given
op count will take.  Names, call signatures and results are those of the
reference's python/gpumap/schedule/estimator.py (Estimator :10-22,
FitResult / RateFitResult :25-37, MeanRateEstimator :40-101,
DefaultLinearEstimator :104-227, PersistentEstimator :230-325); the
allocations they lead to are checked against the reference's own outputs in
tests/golden/schedule_golden.json.

Both models keep a bounded window of the most recent valid samples (ops > 0,
seconds >= 0) and cache their fit until the next sample arrives.
"""
from __future__ import annotations

import contextlib
import os
import sqlite3
import time
from collections import deque
from dataclasses import dataclass
from statistics import NormalDist
from typing import Iterable, Optional, Sequence, Tuple

Sample = Tuple[int, float]


def _quantile(q: float) -> float:
    """Standard normal quantile (the safety margin in standard deviations)."""
    return NormalDist().inv_cdf(q)


def _mean_sd(values: Sequence[float]) -> Tuple[float, float]:
    """Mean and sample standard deviation (n - 1 denominator; 0 for one value)."""
    n = len(values)
    mean = sum(values) / n
    if n < 2:
        return mean, 0.0
    return mean, (sum((v - mean) ** 2 for v in values) / (n - 1)) ** 0.5


@dataclass
class RateFitResult:
    mean_rate: float  # seconds per op
    sigma_rate: float  # standard deviation of the per-sample rate
    n_samples: int


@dataclass
class FitResult:
    slope_a: float  # seconds per op
    intercept_b: float  # fixed seconds per call
    sigma: float  # standard deviation of the residuals
    n_samples: int


def fit_rate(samples: Iterable[Sample]) -> Tuple[float, float, int]:
    """(mean, sd, count) of the per-op times seconds / ops."""
    rates = [secs / ops for ops, secs in samples]
    mean, sd = _mean_sd(rates) if rates else (0.0, 0.0)
    return mean, sd, len(rates)


def fit_line(samples: Sequence[Sample]) -> FitResult:
    """Least-squares line seconds = a * ops + b, with the residuals' spread.
    Raises ValueError when every sample has the same op count."""
    xs = [ops for ops, _ in samples]
    ys = [secs for _, secs in samples]
    n = len(xs)
    mx, my = sum(xs) / n, sum(ys) / n
    sxx = sum((x - mx) ** 2 for x in xs)
    if sxx == 0:
        raise ValueError("Degenerate samples.")
    sxy = sum((x - mx) * (y - my) for x, y in zip(xs, ys))
    a = sxy / sxx
    b = my - a * mx
    _, sd = _mean_sd([y - (a * x + b) for x, y in zip(xs, ys)])
    return FitResult(a, b, sd, n)


class Estimator:
    """Interface of a per-operation cost model."""

    def add_sample(self, ops: int, elapsed_sec: float):
        raise NotImplementedError()

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        raise NotImplementedError()

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        raise NotImplementedError()


class _WindowedEstimator(Estimator):
    """The part both models share: the sample window and the cached fit."""

    def __init__(self, window_size: int, min_samples: int):
        self.window_size = window_size
        self.min_samples = min_samples
        self._samples: deque = deque(maxlen=window_size)
        self._fit = None

    def add_sample(self, ops: int, elapsed_sec: float):
        if ops > 0 and elapsed_sec >= 0:
            self._samples.append((ops, elapsed_sec))
            self._fit = None

    def fit(self):
        raise NotImplementedError()

    def fit_result(self):
        if not self._fit:
            self._fit = self.fit()
        return self._fit


class MeanRateEstimator(_WindowedEstimator):
    """Time is proportional to ops: t = rate * ops.  The budget is divided by
    a pessimistic rate, mean + z * sd over the window (z the normal quantile
    of the confidence).  Needs ``min_samples`` samples; ValueError before."""

    def __init__(self, window_size: int = 20, min_samples: int = 3):
        super().__init__(window_size, min_samples)

    def fit(self) -> RateFitResult:
        mean, sd, n = fit_rate(self._samples)
        if n < self.min_samples:
            raise ValueError("Not enough samples.")
        if mean <= 0:
            raise ValueError("Non-positive mean rate.")
        return RateFitResult(mean, sd, n)

    def _pessimistic_rate(self, q: float) -> float:
        f = self.fit_result()
        return f.mean_rate + _quantile(q) * f.sigma_rate

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        if time_budget_sec <= 0:
            return 0
        rate = self._pessimistic_rate(confidence)
        return max(0, int(time_budget_sec / rate)) if rate > 0 else 0

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        if ops <= 0:
            return 0.0
        return ops * max(0.0, self._pessimistic_rate(quantile))


class DefaultLinearEstimator(_WindowedEstimator):
    """Time is affine in ops: t = a * ops + b + noise.  The op count keeps
    t within the budget at the requested confidence.  Before ``min_samples``
    samples it proposes the fixed warm-up sizes ``cold_start_ops`` in turn
    (then the last one again); when the fit is unusable (slope <= 0, or the
    intercept and margin exceed the budget) it falls back to the slowest
    per-op time among the recent samples of at least 1 % of the largest
    op count."""

    def __init__(self, window_size: int = 10, min_samples: int = 3):
        super().__init__(window_size, min_samples)
        self.cold_start_ops = [1000, 2000, 3000]
        self.cold_cnt = 0

    def fit(self) -> Optional[FitResult]:
        if len(self._samples) < self.min_samples:
            return None
        return fit_line(list(self._samples))

    def _next_cold_start_ops(self) -> int:
        step = min(self.cold_cnt, len(self.cold_start_ops) - 1)
        self.cold_cnt = min(self.cold_cnt + 1, len(self.cold_start_ops))
        return self.cold_start_ops[step]

    def _fallback_ops_from_recent_rates(self, time_budget_sec: float) -> int:
        if time_budget_sec <= 0:
            return 0
        floor = max((ops for ops, _ in self._samples), default=0) * 0.01
        rates = [secs / ops for ops, secs in self._samples if ops >= floor and secs > 0]
        if not rates:
            return self._next_cold_start_ops()
        return max(1, int(time_budget_sec / max(rates)))

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        f = self.fit_result()
        if f is None:
            return self._next_cold_start_ops()
        if f.slope_a <= 0:
            return self._fallback_ops_from_recent_rates(time_budget_sec)
        room = time_budget_sec - f.intercept_b - _quantile(confidence) * f.sigma
        ops = room / f.slope_a if room > 0 else 0.0
        return int(ops) if ops > 0 else self._fallback_ops_from_recent_rates(time_budget_sec)

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        f = self.fit_result()
        if f is None:
            return float("inf")
        return f.slope_a * ops + f.intercept_b + _quantile(quantile) * f.sigma


# On-disk format of the timing history (shared with the reference's files,
# so a history written by either can be read by the other).
_SCHEMA = (
    "CREATE TABLE IF NOT EXISTS samples (id INTEGER PRIMARY KEY AUTOINCREMENT, "
    "kind TEXT NOT NULL, ops INTEGER NOT NULL, elapsed REAL NOT NULL, ts REAL NOT NULL)",
    "CREATE INDEX IF NOT EXISTS idx_kind_ts ON samples(kind, ts)",
    "CREATE TABLE IF NOT EXISTS runs (id INTEGER PRIMARY KEY AUTOINCREMENT, "
    "kind TEXT NOT NULL, data_name TEXT NOT NULL, n_features INTEGER NOT NULL, "
    "n_inserted_instances INTEGER NOT NULL, ts REAL NOT NULL)",
)


class PersistentEstimator(Estimator):
    """Any estimator with its samples kept in an SQLite file, so a new
    process starts from the recent history instead of a cold start.

    ``kind`` names the operation (rows of several kinds share one file); the
    newest ``load_limit`` samples of that kind are replayed into ``base``,
    oldest first, when the estimator is created.  The file's directory is
    created if needed.
    """

    def __init__(self, base: Estimator, db_path: str, kind: str, load_limit: int = 100):
        self._base = base
        self._kind = kind
        path = os.path.abspath(db_path)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        self._conn = sqlite3.connect(path, check_same_thread=False)
        with self._conn:
            for stmt in _SCHEMA:
                self._conn.execute(stmt)
        for ops, secs in self._recent(load_limit):
            base.add_sample(int(ops), float(secs))

    def _recent(self, limit: int):
        newest_first = self._conn.execute(
            "SELECT ops, elapsed FROM samples WHERE kind = ? ORDER BY ts DESC LIMIT ?",
            (self._kind, limit)).fetchall()
        return newest_first[::-1]

    def add_sample(self, ops: int, elapsed_sec: float) -> None:
        if ops <= 0 or elapsed_sec < 0:
            return
        self._base.add_sample(ops, elapsed_sec)
        with self._conn:
            self._conn.execute("INSERT INTO samples (kind, ops, elapsed, ts) VALUES (?, ?, ?, ?)",
                               (self._kind, ops, elapsed_sec, time.time()))

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        return self._base.estimate_ops(time_budget_sec, confidence)

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        return self._base.predict_time(ops, quantile)

    def log_run(self, data_name: str, n_features: int, n_inserted_instances: int) -> None:
        """Records one run (dataset name, width, rows inserted) for this kind."""
        with self._conn:
            self._conn.execute(
                "INSERT INTO runs (kind, data_name, n_features, n_inserted_instances, ts) "
                "VALUES (?, ?, ?, ?, ?)",
                (self._kind, data_name, n_features, n_inserted_instances, time.time()))

    def close(self) -> None:
        with contextlib.suppress(Exception):
            self._conn.close()
