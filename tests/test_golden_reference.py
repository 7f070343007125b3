"""Pins against outputs of the reference itself (fixtures in tests/golden,
regenerated by tests/golden/make_golden.py from the reference tree)."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


def test_queue_rules_match_reference_queue_cuh(oracle_mod):
    # output of the reference's own cpp/src/queue.cuh on a fixed script
    assert oracle_mod.queue_script() == (GOLD / "queue_golden.txt").read_text()


@pytest.fixture(scope="module")
def gold():
    return json.loads((GOLD / "schedule_golden.json").read_text())


class _R:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def _drive(st, script):
    np.random.seed(1234)
    out = []
    for res in script:
        for tl in (0.5, 2.0, 10.0):
            out.append([int(v) for v in st.allocate(tl)])
        r = _R(**res)
        st.update(r)
        for name, flag in (("insertion", r.insertion_completed), ("update", r.update_completed),
                           ("embedding", r.embedding_completed)):
            if flag:
                st.on_operation_complete(name)
        out.append([float(x) for x in st.get_progress()])
    return out


def test_weighted_strategy_matches_reference(gold):
    from gpumap_gb300.schedule import WeightedStrategy

    assert _drive(WeightedStrategy(n_instances=70000, n_neighbors=15), gold["script"]) == gold["weighted"]


def test_weighted_linear_matches_reference(gold):
    from gpumap_gb300.schedule import DefaultLinearEstimator, WeightedStrategy

    st = WeightedStrategy(n_instances=70000, insertion_estimator=DefaultLinearEstimator(),
                          update_estimator=DefaultLinearEstimator(), embedding_estimator=DefaultLinearEstimator())
    assert _drive(st, gold["script"]) == gold["weighted_linear"]


def test_sequential_strategy_matches_reference(gold):
    from gpumap_gb300.schedule import SequentialPriorityStrategy

    assert _drive(SequentialPriorityStrategy(n_instances=70000), gold["script"]) == gold["sequential"]


@pytest.mark.parametrize("kind", ["mean_rate", "linear"])
def test_estimators_match_reference(gold, kind):
    from gpumap_gb300.schedule import DefaultLinearEstimator, MeanRateEstimator

    est = MeanRateEstimator() if kind == "mean_rate" else DefaultLinearEstimator()
    out = []
    for res in gold["script"]:
        est.add_sample(res["n_update_ops"], res["update_time"])
        row = []
        for budget in (0.0, 0.3, 1.0, 5.0):
            try:
                row.append(int(est.estimate_ops(budget, 0.95)))
            except ValueError:
                row.append(None)
        try:
            row.append(float(est.predict_time(1000, 0.9)))
        except ValueError:
            row.append(None)
        out.append(row)
    assert out == gold[kind]


def test_find_ab_params_matches_reference(gold):
    from gpumap_gb300.gpumap import find_ab_params

    for md, (a, b) in gold["ab_params"].items():
        ga, gb = find_ab_params(1.0, float(md))
        assert abs(ga - a) <= 1e-9 * max(1.0, abs(a)) and abs(gb - b) <= 1e-9 * max(1.0, abs(b))


def test_persistent_estimator_roundtrip(tmp_path):
    from gpumap_gb300.schedule import MeanRateEstimator, PersistentEstimator

    db = tmp_path / "est" / "h.sqlite"
    p = PersistentEstimator(MeanRateEstimator(), str(db), "update")
    for ops, t in ((1000, 0.5), (2000, 1.1), (1500, 0.7)):
        p.add_sample(ops, t)
    p.log_run("x", 8, 100)
    ref = p.estimate_ops(2.0)
    p.close()
    q = PersistentEstimator(MeanRateEstimator(), str(db), "update")
    assert q.estimate_ops(2.0) == ref
    q.close()


# ---- the reference's own CUDA fuzzy set and edge schedule ------------------
# Fixtures: tests/golden/ref_fuzzy_<case>.in (published k-NN tables from the
# oracle's progressive cycles) and .out (what the reference's own
# compute_fuzzy_graph, trim_graph, make_epochs_per_sample_kernel and
# compute_rounding_factor produced from them on a GB300, through
# oracle/refbuild/ref_fuzzy_driver.cu); tests/golden/make_ref_fuzzy.py makes both.
REF_FUZZY_CASES = ["euclid_k15", "euclid_k15_partial", "cosine_k10", "euclid_k30", "tiny_sentinels"]


def _sorted_by_edge(rows, cols, vals):
    order = np.lexsort((cols, rows))
    return rows[order], cols[order], vals[order]


@pytest.mark.parametrize("case", REF_FUZZY_CASES)
def test_fuzzy_schedule_matches_reference_build(oracle_mod, case):
    import sys

    sys.path.insert(0, str(GOLD))
    from make_ref_fuzzy import read_input, read_output

    c = read_input(GOLD / f"ref_fuzzy_{case}.in")
    r = read_output(GOLD / f"ref_fuzzy_{case}.out", c["n"])
    o = oracle_mod.fuzzy_schedule(c["pub_idx"], c["pub_dist"], c["k"], c["euclidean"], c["batch"],
                                  c["n_epochs"], c["alpha"])
    # integer work is bit-exact: the fuzzy-union COO and the trimmed schedule,
    # compared as sorted (row, col) lists (the reference appends by atomics)
    assert (o["nnz"], o["extras"], o["nnz2"]) == (r["nnz"], r["extras"], r["nnz2"])
    rr, rc, rv = _sorted_by_edge(r["coo_row"], r["coo_col"], r["coo_val"])
    orr, orc, ov = _sorted_by_edge(o["coo_row"], o["coo_col"], o["coo_val"])
    np.testing.assert_array_equal(orr, rr)
    np.testing.assert_array_equal(orc, rc)
    tr, tc, te = _sorted_by_edge(r["t_row"], r["t_col"], r["t_eps"])
    otr, otc, ote = _sorted_by_edge(o["t_row"], o["t_col"], o["t_eps"])
    np.testing.assert_array_equal(otr, tr)
    np.testing.assert_array_equal(otc, tc)
    assert o["rounding"] == r["rounding"] and o["max_w"] == r["max_w"]
    np.testing.assert_array_equal(o["rho"], r["rho"])
    # floating point: the reference bisects sigma on an FP32 sum of __expf
    # terms, the oracle on an FP64 sum of its own expf; the bisection may stop
    # one step apart (|psum - target| < 1e-5), which moves sigma by < 1e-5
    # relative and a weight exp(-(d - rho) / sigma) by up to a few e-5.
    srel = np.abs(o["sigma"] - r["sigma"]) / np.maximum(np.abs(r["sigma"]), 1e-30)
    assert srel.max() <= 1e-5, srel.max()
    for mine, ref in ((ov, rv), (ote, te)):
        rel = np.abs(mine - ref) / np.maximum(np.abs(ref), 1e-30)
        assert np.mean(rel <= 1e-5) >= 0.999, np.mean(rel <= 1e-5)
        assert rel.max() <= 3e-5, rel.max()
