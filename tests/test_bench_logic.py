"""Host-side logic of bench.py (no GPU): recall, clock summary, and the
roofline's choice of kernel, rates and traffic scaling."""
import types

import numpy as np

import bench


def _stats(**kw):
    base = dict(exact_ms=0.0, exact_flops=0.0, exact_launches=0, screen_ms=0.0, exact_rescored=0, exact_pairs=0,
                join_ms=0.0, join_rows=0, join_pairs=0, join_launches=0, cand_ms=0.0, cand_rows=0, cand_launches=0,
                sgd_ms=0.0, sgd_edges=0, sgd_negatives=0, sgd_launches=0)
    base.update(kw)
    return types.SimpleNamespace(**base)


def test_recall_counts_shared_ids():
    exact = np.array([[1, 2, 3], [4, 5, 6]])
    approx = np.array([[3, 2, 9], [6, 5, 4]])
    assert bench.recall(approx, exact) == (2 + 3) / 6


def test_roofline_picks_largest_time_and_scales_traffic():
    peaks = {"hbm_gbs": 1000.0, "bf16_tflops_sustained": 2000.0}
    t = bench.NCU_TRAFFIC["k_exact_dist"]
    st = _stats(exact_ms=10.0, exact_flops=2 * t["units"] * 4.0, exact_launches=4,
                sgd_ms=30.0, sgd_edges=1000, sgd_negatives=5000, sgd_launches=2)
    dom, agg = bench.roofline([st], d=784, peaks=peaks)
    assert dom == "k_sgd_persistent"
    # tensor kernel: FLOPs per launch over time per launch, against the sustained peak
    ex = agg["k_exact_dist"]
    assert ex["unit"] == "TFLOP/s" and ex["peak"] == 2000.0
    assert abs(ex["achieved"] - (2 * t["units"]) / (2.5e-3) / 1e12) < 1e-6 * ex["achieved"]
    # traffic scaled by FLOPs per launch (twice the captured launch here)
    assert abs(ex["traffic"] - 2 * t["bytes"]) < 1e-6 * t["bytes"]
    sgd = agg["k_sgd_persistent"]
    assert sgd["unit"] == "GB/s" and sgd["traffic"] == bench.NCU_TRAFFIC["k_sgd_persistent"]["bytes"]
    assert abs(sgd["achieved"] - (1000 * 28 + 6000 * 8) / 2 / 15e-3 / 1e9) < 1e-9


def test_roofline_without_launches_is_empty():
    dom, agg = bench.roofline([_stats()], d=16, peaks={})
    assert dom is None and agg == {}


def test_clock_summary_reports_throttle_reasons():
    c = bench.ClockSampler(0)
    c.samples = [["2070", "2070", "900", "Not Active", "Not Active", "Not Active", "Active"],
                 ["2055", "2070", "950", "Not Active", "Not Active", "Not Active", "Not Active"]]
    s = c.summary()
    assert s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"] and s["samples"] == 2


def test_embed_quality_matches_oracle_trustworthiness():
    # both spaces restricted to the subset: with every row in it, the score is
    # the plain trustworthiness the oracle computes
    import torch

    from oracle.knn import trustworthiness

    rng = np.random.default_rng(5)
    X = rng.normal(size=(300, 12)).astype(np.float32)
    E = (X[:, :2] + 0.3 * rng.normal(size=(300, 2))).astype(np.float32)
    t, kp = bench.embed_quality(torch.from_numpy(X), E, np.arange(300), k=10)
    assert abs(t - trustworthiness(X, E, 10)) < 1e-12
    assert 0.0 < kp <= 1.0
    # an embedding that keeps the input itself preserves every neighbour
    t2, kp2 = bench.embed_quality(torch.from_numpy(X[:, :2].copy()), X[:, :2].copy(), np.arange(300), k=10)
    assert t2 == 1.0 and kp2 == 1.0


def test_fp64_baseline_counts_rows():
    X = np.random.default_rng(1).normal(size=(3000, 16)).astype(np.float32)
    v, rows, dt = bench.fp64_bruteforce_baseline(X, k=5, target_s=0.0, block=512)
    assert rows == 512 and v > 0 and dt >= 0
