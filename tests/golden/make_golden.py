"""Regenerates the committed golden fixtures from the reference itself.

Run where the reference tree is available (its root in GPUMAP_REFERENCE,
else the read-only mount this script was written against):

    python tests/golden/make_golden.py

* ``queue_golden.txt`` -- output of oracle/_ref/queue_golden, the reference's
  own cpp/src/queue.cuh compiled in place (oracle/build_oracle.py).
* ``schedule_golden.json`` -- allocations of the reference's Python
  WeightedStrategy / SequentialPriorityStrategy and estimates of its
  MeanRateEstimator / DefaultLinearEstimator on a scripted result sequence,
  plus ``find_ab_params`` for several min_dist values.  The reference package
  is imported from its source tree with ``cupy`` and the compiled ``_core``
  replaced by empty stand-in modules (neither is used by these functions).
"""
from __future__ import annotations

import json
import subprocess
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
import os

REF_PY = Path(os.environ.get("GPUMAP_REFERENCE", "/root/reference")) / "python"


def import_reference():
    sys.modules.setdefault("cupy", types.ModuleType("cupy"))
    core = types.ModuleType("gpumap._core")
    core.GPUMAPParams = object
    core.GPUMAP = object
    sys.modules["gpumap._core"] = core
    sys.path.insert(0, str(REF_PY))
    import gpumap.gpumap as g  # noqa: E402
    import gpumap.schedule as sch  # noqa: E402

    return g, sch


class FakeResult:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def result_script():
    """A fixed sequence of cycle results (times in seconds)."""
    rng = np.random.default_rng(7)
    out = []
    inserted = 0
    for c in range(30):
        ni = int(rng.integers(0, 3000)) if c < 20 else 0
        inserted += ni
        out.append(dict(
            n_insertion_ops=ni, n_update_ops=int(rng.integers(0, 9000)), n_embedding_ops=int(rng.integers(0, 6000)),
            insertion_time=float(rng.uniform(0.01, 2.0)), update_time=float(rng.uniform(0.0, 3.0)),
            embedding_time=float(rng.uniform(0.0, 1.5)), insertion_completed=c >= 20,
            update_completed=c >= 25, embedding_completed=c >= 28, n_inserted_instances=inserted,
            n_update_changed_edges=0, embedding_pending_edges=inserted,
            insertion_queue_size=0, update_queue_size=int(rng.integers(0, 500)),
            embedding_queue_size=inserted,
        ))
    return out


def drive_strategy(make, script):
    np.random.seed(1234)
    st = make()
    allocs = []
    for res in script:
        for tl in (0.5, 2.0, 10.0):
            allocs.append([int(v) for v in st.allocate(tl)])
        r = FakeResult(**res)
        st.update(r)
        if r.insertion_completed:
            st.on_operation_complete("insertion")
        if r.update_completed:
            st.on_operation_complete("update")
        if r.embedding_completed:
            st.on_operation_complete("embedding")
        allocs.append([float(x) for x in st.get_progress()])
    return allocs


def drive_estimator(make, script):
    est = make()
    out = []
    for res in script:
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
    return out


def main():
    exe = ROOT / "oracle" / "_ref" / "queue_golden"
    if not exe.exists():
        sys.path.insert(0, str(ROOT))
        from oracle.build_oracle import build_ref_queue

        build_ref_queue()
    (HERE / "queue_golden.txt").write_text(subprocess.run([str(exe)], capture_output=True, text=True,
                                                          check=True).stdout)

    g, sch = import_reference()
    script = result_script()
    gold = {
        "script": script,
        "weighted": drive_strategy(lambda: sch.WeightedStrategy(n_instances=70000, n_neighbors=15), script),
        "weighted_linear": drive_strategy(
            lambda: sch.WeightedStrategy(n_instances=70000, insertion_estimator=sch.DefaultLinearEstimator(),
                                         update_estimator=sch.DefaultLinearEstimator(),
                                         embedding_estimator=sch.DefaultLinearEstimator()), script),
        "sequential": drive_strategy(lambda: sch.SequentialPriorityStrategy(n_instances=70000), script),
        "mean_rate": drive_estimator(lambda: sch.MeanRateEstimator(), script),
        "linear": drive_estimator(lambda: sch.DefaultLinearEstimator(), script),
        "ab_params": {str(md): [float(v) for v in g.find_ab_params(1.0, md)] for md in (0.0, 0.05, 0.1, 0.25, 0.5, 1.0)},
    }
    (HERE / "schedule_golden.json").write_text(json.dumps(gold, indent=1))
    print("wrote", HERE / "queue_golden.txt", HERE / "schedule_golden.json")


if __name__ == "__main__":
    main()
