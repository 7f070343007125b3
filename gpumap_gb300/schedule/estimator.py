"""Per-operation cost models used to turn a time budget into op counts.

Restates python/gpumap/schedule/estimator.py of the reference:
``MeanRateEstimator`` (rolling mean/std of seconds-per-op), the
``DefaultLinearEstimator`` (least-squares t = a*ops + b with cold-start and
rate fallbacks) and ``PersistentEstimator`` (SQLite-backed sample history).
"""
from __future__ import annotations

import os
import sqlite3
import time as _time
from collections import deque
from dataclasses import dataclass
from statistics import NormalDist
from typing import Deque, Optional, Tuple


class Estimator:
    """Estimates how many operations fit in a time budget."""

    def add_sample(self, ops: int, elapsed_sec: float):
        raise NotImplementedError()

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        raise NotImplementedError()

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        raise NotImplementedError()


@dataclass
class FitResult:
    slope_a: float  # seconds per op
    intercept_b: float  # fixed overhead in seconds
    sigma: float  # residual standard deviation
    n_samples: int


@dataclass
class RateFitResult:
    mean_rate: float  # seconds per op
    sigma_rate: float  # standard deviation of seconds per op
    n_samples: int


def _sample_std(values, mean: float) -> float:
    n = len(values)
    if n < 2:
        return 0.0
    return (sum((v - mean) ** 2 for v in values) / (n - 1)) ** 0.5


class MeanRateEstimator(Estimator):
    """t ~ rate * ops, rate from a rolling window; conservative by a normal quantile."""

    def __init__(self, window_size: int = 20, min_samples: int = 3):
        self.window_size = window_size
        self.min_samples = min_samples
        self._samples: Deque[Tuple[int, float]] = deque(maxlen=window_size)
        self._fit: Optional[RateFitResult] = None

    def add_sample(self, ops: int, elapsed_sec: float):
        if ops <= 0 or elapsed_sec < 0:
            return
        self._samples.append((ops, elapsed_sec))
        self._fit = None

    def fit(self) -> RateFitResult:
        rates = [t / o for o, t in self._samples if o > 0]
        if len(rates) < self.min_samples:
            raise ValueError("Not enough samples.")
        mean = sum(rates) / len(rates)
        if mean <= 0:
            raise ValueError("Non-positive mean rate.")
        self._fit = RateFitResult(mean, _sample_std(rates, mean), len(rates))
        return self._fit

    def fit_result(self) -> RateFitResult:
        return self._fit if self._fit else self.fit()

    def _safe_rate(self, q: float) -> float:
        fr = self.fit_result()
        return fr.mean_rate + NormalDist().inv_cdf(q) * fr.sigma_rate

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        if time_budget_sec <= 0:
            return 0
        rate = self._safe_rate(confidence)
        if rate <= 0:
            return 0
        return max(0, int(time_budget_sec / rate))

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        if ops <= 0:
            return 0.0
        return ops * max(0.0, self._safe_rate(quantile))


class DefaultLinearEstimator(Estimator):
    """t ~ a*ops + b by least squares over a window, with fallbacks."""

    def __init__(self, window_size: int = 10, min_samples: int = 3):
        self.window_size = window_size
        self.min_samples = min_samples
        self.cold_start_ops = [1000, 2000, 3000]
        self._samples: Deque[Tuple[int, float]] = deque(maxlen=window_size)
        self._fit: Optional[FitResult] = None
        self.cold_cnt = 0

    def add_sample(self, ops: int, elapsed_sec: float):
        if ops <= 0 or elapsed_sec < 0:
            return
        self._samples.append((ops, elapsed_sec))
        self._fit = None

    def fit(self) -> Optional[FitResult]:
        n = len(self._samples)
        if n < self.min_samples:
            return None
        xs = [o for o, _ in self._samples]
        ys = [t for _, t in self._samples]
        mx = sum(xs) / n
        my = sum(ys) / n
        sxx = sum((x - mx) ** 2 for x in xs)
        if sxx == 0:
            raise ValueError("Degenerate samples.")
        sxy = sum((x - mx) * (y - my) for x, y in zip(xs, ys))
        a = sxy / sxx
        b = my - a * mx
        res = [y - (a * x + b) for x, y in zip(xs, ys)]
        self._fit = FitResult(a, b, _sample_std(res, sum(res) / n), n)
        return self._fit

    def fit_result(self) -> Optional[FitResult]:
        return self._fit if self._fit else self.fit()

    def _next_cold_start_ops(self) -> int:
        if self.cold_cnt < len(self.cold_start_ops):
            ops = self.cold_start_ops[self.cold_cnt]
            self.cold_cnt += 1
            return ops
        return self.cold_start_ops[-1]

    def _fallback_ops_from_recent_rates(self, time_budget_sec: float) -> int:
        # Ignore tiny runs (< 1% of the largest) and use the slowest rate seen.
        if time_budget_sec <= 0:
            return 0
        if not self._samples:
            return self._next_cold_start_ops()
        floor = max(o for o, _ in self._samples) * 0.01
        rates = [t / o for o, t in self._samples if o >= floor and o > 0 and t > 0]
        if not rates:
            return self._next_cold_start_ops()
        worst = max(rates)
        if worst <= 0:
            return self._next_cold_start_ops()
        return max(1, int(time_budget_sec / worst))

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        fr = self.fit_result()
        if fr is None:
            return self._next_cold_start_ops()
        if fr.slope_a <= 0:
            return self._fallback_ops_from_recent_rates(time_budget_sec)
        z = NormalDist().inv_cdf(confidence)
        usable = time_budget_sec - fr.intercept_b - z * fr.sigma
        if usable <= 0:
            return self._fallback_ops_from_recent_rates(time_budget_sec)
        ops = usable / fr.slope_a
        return int(ops) if ops > 0 else self._fallback_ops_from_recent_rates(time_budget_sec)

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        fr = self.fit_result()
        if fr is None:
            return float("inf")
        return fr.slope_a * ops + fr.intercept_b + NormalDist().inv_cdf(quantile) * fr.sigma


class PersistentEstimator(Estimator):
    """Wraps an estimator and keeps its samples in an SQLite file across runs.

    On construction the newest ``load_limit`` samples of ``kind`` are replayed
    into ``base`` (oldest first).
    """

    def __init__(self, base: Estimator, db_path: str, kind: str, load_limit: int = 100):
        self._base = base
        self._kind = kind
        os.makedirs(os.path.dirname(os.path.abspath(db_path)), exist_ok=True)
        self._conn = sqlite3.connect(db_path, check_same_thread=False)
        self._conn.execute(
            "CREATE TABLE IF NOT EXISTS samples (id INTEGER PRIMARY KEY AUTOINCREMENT, "
            "kind TEXT NOT NULL, ops INTEGER NOT NULL, elapsed REAL NOT NULL, ts REAL NOT NULL)"
        )
        self._conn.execute("CREATE INDEX IF NOT EXISTS idx_kind_ts ON samples(kind, ts)")
        self._conn.execute(
            "CREATE TABLE IF NOT EXISTS runs (id INTEGER PRIMARY KEY AUTOINCREMENT, "
            "kind TEXT NOT NULL, data_name TEXT NOT NULL, n_features INTEGER NOT NULL, "
            "n_inserted_instances INTEGER NOT NULL, ts REAL NOT NULL)"
        )
        self._conn.commit()
        self._load(load_limit)

    def _load(self, limit: int) -> None:
        rows = self._conn.execute(
            "SELECT ops, elapsed FROM samples WHERE kind=? ORDER BY ts DESC LIMIT ?",
            (self._kind, limit),
        ).fetchall()
        for ops, elapsed in reversed(rows):
            self._base.add_sample(int(ops), float(elapsed))

    def add_sample(self, ops: int, elapsed_sec: float) -> None:
        if ops <= 0 or elapsed_sec < 0:
            return
        self._base.add_sample(ops, elapsed_sec)
        self._conn.execute(
            "INSERT INTO samples(kind, ops, elapsed, ts) VALUES(?,?,?,?)",
            (self._kind, ops, elapsed_sec, _time.time()),
        )
        self._conn.commit()

    def estimate_ops(self, time_budget_sec: float, confidence: float = 0.95) -> int:
        return self._base.estimate_ops(time_budget_sec, confidence)

    def predict_time(self, ops: int, quantile: float = 0.95) -> float:
        return self._base.predict_time(ops, quantile)

    def log_run(self, data_name: str, n_features: int, n_inserted_instances: int) -> None:
        self._conn.execute(
            "INSERT INTO runs(kind, data_name, n_features, n_inserted_instances, ts) VALUES(?,?,?,?,?)",
            (self._kind, data_name, n_features, n_inserted_instances, _time.time()),
        )
        self._conn.commit()

    def close(self) -> None:
        try:
            self._conn.close()
        except Exception:
            pass
