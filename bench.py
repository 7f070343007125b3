"""Benchmark: progressive insertion throughput (points inserted/s) at
recall@15 >= 0.95 on the 70,000 x 784 image-like workload, k=15, euclidean,
500 points per cycle.

One step = one complete progressive build: 140 cycles of
run_with_n_ops(500, U, E), then full update cycles run_with_n_ops(0, n, 0)
until recall@15 on 2,000 seeded query rows (against an exact FP64 brute
force computed before timing) reaches 0.95; the recall checks are inside the
timed region, as the metric counts every cycle until the target is met.

* ``value``  -- precision 1 (BF16 tensor-core distance tiles, FP32 re-score:
  the precision form of this workload) through the C ABI with the input
  already resident in HBM (gm_append_device), timed with CUDA events.
  ``value_no_overlap``, ``schedule_u2000`` (the plain schedule, U = 2000) and
  ``plain_fp32`` (the reference's NN-Descent restated, precision 0) are the
  same measurement for other settings.
* ``e2e``    -- the public Python API (gpumap_gb300.GPUMAP over pinned host
  chunks; every cycle copies its 500 rows host->device, each step ends by
  reading the k-NN table back to the host).
* ``run10``  -- GPUMAP.run(target_latency=10) with the default strategy
  until every row is in and recall@15 reaches the target.
* ``serving`` -- the served workload (serving_run): p50/p99 request latency
  and points/s with continuous batching against one cycle at a time.
* every line carries trustworthiness and k-NN preservation of its embedding
  on the same seeded 10,000-row subset.
* ``roofline`` -- the kernel with the largest summed time, its algorithmic
  bytes (or FLOPs) over its CUDA-event time (events recorded by the engine on
  its own stream), against MEASURED_PEAKS.json.
* ``cpu_baseline`` -- exact FP64 k-NN by brute force (numpy float64 GEMM on
  every host core) on seeded query rows of the same data, rows per second.
* ``--impl reference`` -- the reference's own CUDA build on the same GPU
  and workload, through its own Python API (see reference_arm).

Multi-GPU (torchrun): replicas only -- every rank builds its own copy of the
workload on its own GPU; no collective is on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_POINTS, N_FEATURES, K = 70_000, 784, 15
CHUNK = 500
UPD_OPS, EMB_OPS = 2000, 1000
MAX_FINAL_UPDATE_CYCLES = 40
RECALL_TARGET = 0.95
MAX_EPOCH = 200
RECALL_QUERIES = 2000
METRIC = "points inserted/s at recall@15>=0.95 (70k x 784, k=15, 500 points/cycle)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1])
    ap.add_argument("--overlap", type=int, default=1, choices=[0, 1],
                    help="run each cycle's embedding beside the next cycle's distance work")
    ap.add_argument("--update-ops", type=int, default=None,
                    help="U per cycle (default 0 for precision 1, 2000 for precision 0)")
    ap.add_argument("--embedding-ops", type=int, default=EMB_OPS)
    ap.add_argument("--max-final-updates", type=int, default=MAX_FINAL_UPDATE_CYCLES)
    ap.add_argument("--n-points", type=int, default=N_POINTS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-u2000", action="store_true")
    ap.add_argument("--no-run10", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--rows", type=int, default=None,
                    help="cosine-1m only: the same generator with ROWS rows (profiling); default 1,000,000")
    ap.add_argument("--workload", default="image-70k", choices=["image-70k", "cosine-1m", "serving", "batched-64"],
                    help="image-70k: the headline line; the others print their own line")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def exact_knn_gpu(X_dev, q_idx, k):
    """Exact neighbours of the query rows in float64 on the GPU (recall check)."""
    import torch

    Xd = X_dev.double()
    sq = (Xd * Xd).sum(1)
    out = []
    for s in range(0, len(q_idx), 256):
        qq = torch.as_tensor(q_idx[s : s + 256], device=Xd.device)
        d = sq[qq, None] + sq[None, :] - 2.0 * (Xd[qq] @ Xd.T)
        d[torch.arange(len(qq), device=d.device), qq] = float("inf")
        out.append(torch.topk(d, k, largest=False).indices.cpu().numpy())
    return np.concatenate(out)


def recall(approx, exact):
    """Mean |approx_row & exact_row| / k (rows hold distinct ids)."""
    approx = np.asarray(approx, dtype=np.int64)
    k = exact.shape[1]
    hits = (approx[:, :, None] == exact[:, None, :]).any(-1).sum()
    return float(hits) / (k * len(exact))


def flush_l2(buf):
    buf.zero_()


QUALITY_ROWS, QUALITY_SEED = 10_000, 7


def quality_subset(n: int) -> np.ndarray:
    """The seeded row subset on which every line's embedding is scored."""
    return np.sort(np.random.default_rng(QUALITY_SEED).choice(n, min(QUALITY_ROWS, n), replace=False))


def embed_quality(X_dev, emb, sub, k=K):
    """Trustworthiness (Venna and Kaski) and k-NN preservation of an embedding,
    both spaces restricted to the rows ``sub`` (FP64 on the GPU).

    trust = 1 - 2 / (m k (2m - 3k - 1)) * sum over rows i and embedding
    neighbours j of max(0, r(i, j) - k), r the rank of j among i's input-space
    neighbours (self 0); k-NN preservation = mean |NN_k(x_i) & NN_k(e_i)| / k.
    """
    import torch

    idx = torch.as_tensor(sub, device=X_dev.device)
    m = len(sub)

    def sqdist(A):
        sq = (A * A).sum(1)
        return sq[:, None] + sq[None, :] - 2.0 * (A @ A.T)

    dx = sqdist(X_dev[idx].double())
    dx.fill_diagonal_(-float("inf"))  # self ranks first
    order = torch.argsort(dx, dim=1)
    del dx
    rank = torch.empty_like(order)
    rank.scatter_(1, order, torch.arange(m, device=order.device).expand(m, m).contiguous())
    e = torch.as_tensor(np.ascontiguousarray(emb, dtype=np.float64), device=X_dev.device)[idx] \
        if isinstance(emb, np.ndarray) else emb[idx].double()
    de = sqdist(e)
    de.fill_diagonal_(float("inf"))
    nn_e = torch.topk(de, k, largest=False).indices
    del de
    pen = (rank.gather(1, nn_e) - k).clamp(min=0).sum().item()
    trust = 1.0 - 2.0 / (m * k * (2.0 * m - 3.0 * k - 1.0)) * pen
    nn_x = order[:, 1: k + 1]
    shared = (nn_x[:, :, None] == nn_e[:, None, :]).any(-1).sum().item()
    del order, rank
    return float(trust), float(shared) / (m * k)


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return platform.processor() or platform.machine()


def fp64_bruteforce_baseline(X, k=K, target_s=10.0, block=1024):
    """The CPU baseline: exact FP64 k-NN (numpy float64 GEMM, BLAS on every
    host core) of seeded query rows against all rows, for about target_s
    seconds; returns (rows per second, rows, seconds)."""
    Xd = np.ascontiguousarray(X, dtype=np.float64)
    sq = np.einsum("ij,ij->i", Xd, Xd)
    order = np.random.default_rng(99).permutation(len(Xd))
    done = 0
    t0 = time.perf_counter()
    while done < len(Xd) and (done == 0 or time.perf_counter() - t0 < target_s):
        q = order[done: done + block]
        d = sq[q, None] + sq[None, :] - 2.0 * (Xd[q] @ Xd.T)
        d[np.arange(len(q)), q] = np.inf
        np.argpartition(d, k, axis=1)[:, :k]
        done += len(q)
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def run_value_step(native, X_dev, n, d, upd, emb, max_final, stats_on, q_idx, exact, precision, overlap=0):
    import torch

    p = native.default_params(n_instances=n, n_features=d, n_neighbors=K, max_epoch=MAX_EPOCH,
                              device=torch.cuda.current_device(), precision=precision, overlap=overlap)
    p.a, p.b = 1.5769434602697652, 0.8950608778515733  # find_ab_params(1.0, 0.1)
    s = native.Session(p)
    s.set_stats(stats_on)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    base = X_dev.data_ptr()
    row_bytes = d * 4
    for c in range(0, n, CHUNK):
        m = min(CHUNK, n - c)
        s.append_device(base + c * row_bytes, m, d)
        s.run(m, upd, emb)
    v = s.view("indices")
    table = torch.as_tensor(_Cai(v.ptr, n, K + 1, 4, "<i4"), device="cuda")  # ids < 2^31
    q_dev = torch.as_tensor(q_idx, device="cuda")
    # the build ends once every row is in and recall@15 reaches the target;
    # full update cycles run (and count) only while it has not
    rounds = 0
    rec = recall(table[q_dev, :K].cpu().numpy(), exact)
    while rec < RECALL_TARGET and rounds < max_final:
        s.run(0, n, 0)
        rounds += 1
        rec = recall(table[q_dev, :K].cpu().numpy(), exact)
    s.view("embedding")  # waits for the last embedding (overlap mode)
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    st = s.stats()
    return s, ms, st, rec, rounds


class _Cai:
    def __init__(self, ptr, rows, cols, esz, typestr):
        self.__cuda_array_interface__ = {"version": 3, "shape": (rows, cols), "typestr": typestr,
                                         "strides": (cols * esz, esz), "data": (ptr, False)}


def run_e2e_step(X_host, n, d, upd, emb, max_final, q_idx, exact, precision, overlap=0):
    import torch

    import gpumap_gb300 as gm
    from gpumap_gb300.data_loader import ArrayDataLoader

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    params = gm.GPUMAPParams()
    params.n_instances, params.n_features, params.n_neighbors = n, d, K
    params.max_epoch = MAX_EPOCH
    params.precision = precision
    params.overlap = overlap
    model = gm.GPUMAP(ArrayDataLoader(X_host), params)
    for c in range(0, n, CHUNK):
        model.run_with_n_ops(min(CHUNK, n - c), upd, emb)
    rounds = 0
    idx = model.get_neighbor_indices().cpu().numpy()  # the step's result, device -> host
    rec = recall(idx[q_idx], exact)
    while rec < RECALL_TARGET and rounds < max_final:
        model.run_with_n_ops(0, n, 0)
        rounds += 1
        idx = model.get_neighbor_indices().cpu().numpy()
        rec = recall(idx[q_idx], exact)
    model.get_embedding()  # waits for the last embedding (overlap mode)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    model.close()
    return dt, rec, rounds


def run_target_latency(X_host, n, d, q_idx, exact, precision, overlap, target_s=10.0, max_cycles=60):
    """gpumap_gb300.GPUMAP.run(target_latency) cycles (the default weighted
    strategy splits each cycle's budget) until every row is in and recall@15
    reaches the target; returns (seconds, recall, cycles, allocations, model)."""
    import torch

    import gpumap_gb300 as gm
    from gpumap_gb300.data_loader import ArrayDataLoader

    params = gm.GPUMAPParams()
    params.n_instances, params.n_features, params.n_neighbors = n, d, K
    params.max_epoch = MAX_EPOCH
    params.precision = precision
    params.overlap = overlap
    np.random.seed(0)  # the strategy's warm-up jitter
    model = gm.GPUMAP(ArrayDataLoader(X_host), params)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    allocs, rec = [], 0.0
    for _ in range(max_cycles):
        r = model.run(target_s)
        allocs.append([int(r.n_insertion_ops), int(r.n_update_ops), int(r.n_embedding_ops)])
        if model.n_inserted_instances == n:
            rec = recall(model.get_neighbor_indices().cpu().numpy()[q_idx], exact)
            if rec >= RECALL_TARGET:
                break
    model.get_embedding()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, rec, len(allocs), allocs, model


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# ncu captures of the 30,000-point cut of this workload (k_exact_dist: the
# seed and store passes of cycle 31, 15,500 columns; k_sgd_persistent: the
# launch of cycle 40).  "per" names the unit the traffic scales with, so that
# a capture can be carried to this run's mean launch: the tile passes read
# their column operand once per block (bytes ~ FLOPs); the SGD launch's
# traffic is the first touch of its edge arrays (about the same per
# embedding call at any size, so it is used as measured).
NCU_TRAFFIC = {
    # one insertion block of 500 rows against 15,500 columns (dh 832): the
    # seed pass plus the store pass, DRAM read + write; scaled by FLOPs
    "k_exact_dist": {"bytes": (15401728 + 512) + (54068736 + 2715904), "per": "flop",
                     "units": 6 * 500 * 15500 * 832},
    # one embedding call (1,000 rows, ~26.7k edges, 200 epochs)
    "k_sgd_persistent": {"bytes": 870400 + 75008, "per": "launch", "units": 1},
}


def roofline(stats, d, peaks):
    """Per-kernel achieved rates; returns (dominant name, dict of all)."""
    hbm = peaks.get("hbm_gbs", 6800.0)
    tflops = peaks.get("bf16_tflops_sustained", 1700.0)
    agg = {}

    def add(name, ms, work, launches, bound):
        if ms <= 0 or launches <= 0:
            return
        rate = (work / launches) / ((ms / launches) / 1000.0)
        if bound == "tensor":
            ach, peak, unit = rate / 1e12, tflops, "TFLOP/s"
        else:
            ach, peak, unit = rate / 1e9, hbm, "GB/s"
        agg[name] = {"bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
                     "ms": ms, "launches": launches}

    st = {k: sum(getattr(s_, k) for s_ in stats) for k in (
        "exact_ms", "exact_flops", "exact_launches", "screen_ms", "exact_rescored", "exact_pairs",
        "join_ms", "join_rows", "join_pairs", "join_launches", "cand_ms", "cand_rows", "cand_launches",
        "sgd_ms", "sgd_edges", "sgd_negatives", "sgd_launches")}
    add("k_exact_dist", st["exact_ms"], st["exact_flops"], st["exact_launches"], "tensor")
    add("exact_screen", st["screen_ms"], st["exact_rescored"] * 2 * d * 4 + st["exact_pairs"] * 8,
        st["exact_launches"], "hbm")
    add("k_local_join", st["join_ms"], st["join_rows"] * d * 4 + st["join_pairs"] * 8, st["join_launches"], "hbm")
    add("k_candidate_dists", st["cand_ms"], st["cand_rows"] * d * 4, st["cand_launches"], "hbm")
    add("k_sgd_persistent", st["sgd_ms"], st["sgd_edges"] * 28 + (st["sgd_edges"] + st["sgd_negatives"]) * 8,
        st["sgd_launches"], "hbm")
    for name, t in NCU_TRAFFIC.items():
        if name not in agg:
            continue
        if t["per"] == "flop":
            per_launch = st["exact_flops"] / max(st["exact_launches"], 1)
            agg[name]["traffic"] = t["bytes"] * per_launch / t["units"]
        else:
            agg[name]["traffic"] = float(t["bytes"])
    dom = max(agg, key=lambda k: agg[k]["ms"]) if agg else None
    return dom, agg


SERVE_SESSIONS, SERVE_RATE, SERVE_SECONDS = 16, 40.0, 10.0
SERVE_SLOTS, SERVE_BUDGET = 4, 150 * 10**9


def serving_run(native, seconds=SERVE_SECONDS, rate=SERVE_RATE, capacity=True):
    """The served workload: 16 sessions (sizes log-uniform in [20k, 500k],
    dims uniform in [64, 784], seeded Gaussian mixtures), insertion requests
    of 500-5,000 rows arriving as a Poisson process at 40 per second, each
    running one cycle run_with_n_ops(rows, rows, rows) on its session, all
    state resident on the device under a 150 GB budget.  The same trace is
    replayed with SERVE_SLOTS slots (continuous batching: a request starts as
    soon as a slot and its session are free, cycles of different sessions
    overlap on the GPU) and with one slot (one session's cycle at a time, in
    arrival order); then all requests at once, for capacity.  Recall@15 of
    every session against FP64 brute force on 200 seeded rows each."""
    import torch

    from gpumap_gb300.datasets import mixture_stream, poisson_trace, session_specs
    from gpumap_gb300.serving import Server, TraceRequest, replay

    specs = session_specs(SERVE_SESSIONS, 20_000, 500_000, (64, 784), seed=0)
    events = poisson_trace(specs, rate, seconds, 500, 5000, seed=1)
    need = [0] * len(specs)
    for _, i, r in events:
        need[i] += r
    data = []
    for spec, m in zip(specs, need):
        rows = np.empty((m, spec["d"]), np.float32)
        got = 0
        for blk in mixture_stream(spec["n"], spec["d"], spec["centers"], spec["seed"]):
            take = min(len(blk), m - got)
            rows[got: got + take] = blk[:take]
            got += take
            if got >= m:
                break
        data.append(rows)
    cursor = [0] * len(specs)
    trace = []
    for t, i, r in events:
        trace.append(TraceRequest(t, i, data[i][cursor[i]: cursor[i] + r], r, r))
        cursor[i] += r

    def params(spec):
        p = native.default_params(n_instances=spec["n"], n_features=spec["d"], n_neighbors=K, max_epoch=MAX_EPOCH,
                                  precision=1, overlap=1)
        p.a, p.b = 1.5769434602697652, 0.8950608778515733
        return p

    def run(slots, timed):
        with Server(slots=slots, hbm_budget=SERVE_BUDGET) as srv:
            sids = [srv.open_session(params(sp)) for sp in specs]
            res = replay(srv, sids, trace, timed=timed)
            out = res.summary()
            out["bytes_in_use"] = int(srv.stats().bytes_in_use)
            recs = []
            for i, sp in enumerate(specs):
                m = need[i]
                if m < 2 * K:
                    continue
                x = torch.from_numpy(data[i]).cuda()
                q = np.random.default_rng(100 + i).choice(m, min(200, m), replace=False)
                ex = exact_knn_gpu(x, q, K)
                idx = srv.session(sids[i]).copy("pub_idx", np.uint32).reshape(-1, K + 1)[:m, :K]
                recs.append(recall(idx[q], ex))
            out["recall_at_15_min"] = min(recs) if recs else None
        torch.cuda.synchronize()
        return out

    line = {"workload": f"{len(specs)} sessions, sizes log-uniform [20k, 500k], dims [64, 784]; "
                        f"{len(trace)} requests of 500-5000 rows, Poisson {rate:g}/s for {seconds:g} s; "
                        "each request run_with_n_ops(rows, rows, rows), precision 1",
            "rows": int(sum(need)), "budget_bytes": SERVE_BUDGET}
    line["continuous"] = {"slots": SERVE_SLOTS, **run(SERVE_SLOTS, True)}
    line["one_at_a_time"] = {"slots": 1, **run(1, True)}
    if capacity:
        line["capacity_continuous"] = {"slots": SERVE_SLOTS, **run(SERVE_SLOTS, False)}
        line["capacity_one_at_a_time"] = {"slots": 1, **run(1, False)}
    return line


def cosine_1m_run(native, n=1_000_000, d=128, k=30, chunk=10_000, queries=10_000, fp32_rows=200_000):
    """The large cosine workload: 1,000,000 x 128 rows of a 100-component
    Zipf(1.1) mixture on the unit sphere (angular noise 0.15), metric cosine,
    k = 30, inserted 10,000 rows per cycle with run_with_n_ops(10000, 0,
    10000) (200 SGD epochs, 5 negative samples per edge).  Per-phase
    throughput from the engine's CUDA events and the cycles' phase times;
    recall@30 on 10,000 seeded queries against FP64 brute force over all
    rows.  Beside it, the FP32 path (precision 0, the reference's NN-Descent
    restated) on the first fp32_rows rows of the same data, with the same
    chunking and run_with_n_ops(10000, 10000, 10000)."""
    import torch

    from gpumap_gb300.datasets import cosine_zipf

    X, _ = cosine_zipf(n, d, seed=0)
    X_dev = torch.from_numpy(X).cuda()

    def exact_cos(Xd, q, kk):
        # X rows are unit length: 2 (1 - cos) orders as -x.y
        out = []
        for s0 in range(0, len(q), 512):
            qq = torch.as_tensor(q[s0: s0 + 512], device=Xd.device)
            sim = Xd[qq].double() @ Xd.double().T
            sim[torch.arange(len(qq), device=Xd.device), qq] = -float("inf")
            out.append(torch.topk(sim, kk).indices.cpu().numpy())
        return np.concatenate(out)

    def build(rows, precision, upd, emb_ops):
        m = len(rows)
        p = native.default_params(n_instances=m, n_features=d, n_neighbors=k, max_epoch=MAX_EPOCH,
                                  precision=precision, overlap=1, metric=1)
        p.a, p.b = 1.5769434602697652, 0.8950608778515733
        s = native.Session(p)
        s.set_stats(True)
        base = rows.data_ptr()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        phase = [0.0, 0.0, 0.0]
        for c in range(0, m, chunk):
            r = min(chunk, m - c)
            s.append_device(base + c * d * 4, r, d)
            res = s.run(r, upd, emb_ops)
            phase[0] += res.insertion_time
            phase[1] += res.update_time
            phase[2] += res.embedding_time
        s.view("embedding")
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        return s, wall, phase, s.stats()

    out = {"workload": f"cosine Zipf mixture {n}x{d}, k={k}, metric cosine, {chunk} rows per cycle, "
                       f"run_with_n_ops({chunk},0,{chunk}), {MAX_EPOCH} epochs, 5 negative samples"}
    s, wall, phase, st = build(X_dev, 1, 0, chunk)
    q = np.random.default_rng(5).choice(n, queries, replace=False)
    ex = exact_cos(X_dev, q, k)
    idx = s.copy("pub_idx", np.uint32).reshape(-1, k + 1)[:n, :k]
    out["precision1_bf16_split"] = {
        "points_per_s": n / wall, "seconds": wall, "recall_at_30": recall(idx[q], ex),
        "phase_s": phase, "tensor_tile_ms": st.exact_ms, "screen_ms": st.exact_ms and st.screen_ms,
        "tensor_tflops": st.exact_flops / (st.exact_ms / 1e3) / 1e12 if st.exact_ms else None,
        "sgd_ms": st.sgd_ms, "pairs_screened": int(st.exact_pairs), "pairs_rescored": int(st.exact_rescored),
        "overflow_blocks": int(st.exact_overflow_blocks), "kernel_launches": int(st.kernel_launches)}
    del s
    m = min(fp32_rows, n)
    s, wall, phase, st = build(X_dev[:m], 0, chunk, chunk)
    q2 = np.random.default_rng(6).choice(m, min(queries, m), replace=False)
    ex2 = exact_cos(X_dev[:m], q2, k)
    idx2 = s.copy("pub_idx", np.uint32).reshape(-1, k + 1)[:m, :k]
    s1 = out["precision1_bf16_split"]
    out["fp32_nndescent"] = {"rows": m, "points_per_s": m / wall, "seconds": wall,
                             "recall_at_30": recall(idx2[q2], ex2), "phase_s": phase,
                             "candidate_ms": st.cand_ms, "join_ms": st.join_ms, "sgd_ms": st.sgd_ms}
    del s
    return out


def batched_run(native, count=64, chunk=5000, slots=8):
    """The batched workload: 64 independent datasets (sizes log-uniform in
    [2,000, 200,000], dims from {32, 128, 784}, k from {10, 15, 30}, 5-20
    component Gaussian mixtures, data seed = dataset index), every one built
    completely: its rows in requests of 5,000 with run_with_n_ops(rows, 0,
    rows), precision 1.  All requests are queued at once on a server with
    ``slots`` slots (the datasets' cycles run concurrently, each session's in
    order) and, for comparison, on one slot (the 64 builds one after
    another).  Aggregate points/s = all rows / makespan; recall@k on 100
    seeded rows of every dataset against FP64 brute force."""
    import torch

    from gpumap_gb300.datasets import mixture_stream, session_specs
    from gpumap_gb300.serving import Server, TraceRequest, replay

    specs = session_specs(count, 2_000, 200_000, [32, 128, 784], seed=0)
    ks = np.random.default_rng(1).choice([10, 15, 30], size=count)
    data = [np.concatenate(list(mixture_stream(sp["n"], sp["d"], sp["centers"], sp["seed"]))) for sp in specs]
    # requests in round-robin over the datasets, each dataset's rows in order
    trace, cursors = [], [0] * count
    while True:
        added = False
        for i in range(count):
            c = cursors[i]
            if c < specs[i]["n"]:
                r = min(chunk, specs[i]["n"] - c)
                trace.append(TraceRequest(0.0, i, data[i][c: c + r], 0, r))
                cursors[i] += r
                added = True
        if not added:
            break

    def run(nslots):
        with Server(slots=nslots, hbm_budget=SERVE_BUDGET) as srv:
            sids = []
            for i, sp in enumerate(specs):
                p = native.default_params(n_instances=sp["n"], n_features=sp["d"], n_neighbors=int(ks[i]),
                                          max_epoch=MAX_EPOCH, precision=1, overlap=1)
                p.a, p.b = 1.5769434602697652, 0.8950608778515733
                sids.append(srv.open_session(p))
            res = replay(srv, sids, trace, timed=False)
            summ = res.summary()
            recs = []
            for i, sp in enumerate(specs):
                x = torch.from_numpy(data[i]).cuda()
                q = np.random.default_rng(200 + i).choice(sp["n"], 100, replace=False)
                ex = exact_knn_gpu(x, q, int(ks[i]))
                idx = srv.session(sids[i]).copy("pub_idx", np.uint32).reshape(-1, int(ks[i]) + 1)[:, : int(ks[i])]
                recs.append(recall(idx[q], ex))
        torch.cuda.synchronize()
        return {"slots": nslots, "points_per_s": summ["points_per_s"], "makespan_s": summ["span_s"],
                "requests": summ["requests"], "failed": summ["failed"], "recall_min": min(recs)}

    out = {"workload": f"{count} datasets, sizes log-uniform [2k, 200k], dims {{32,128,784}}, k {{10,15,30}}, "
                       f"requests of {chunk} rows run_with_n_ops(rows, 0, rows), precision 1",
           "rows": int(sum(sp["n"] for sp in specs))}
    out["batched"] = run(slots)
    out["sequential"] = run(1)
    return out


REF_WARMUP_ROWS = 5000
REF_PLATEAU = 0.002


def reference_arm(args, X, rank):
    """The reference's own CUDA build (oracle/refbuild), through its own
    Python API (gpumap.GPUMAP.run_with_n_ops over host arrays), on the same
    GB300 and workload.  The K timed steps together make one complete build:
    step i runs its share of the 500-row insertion cycles, the last step also
    the full update cycles that raise recall (run while recall@15 is below
    the target and a cycle still adds at least REF_PLATEAU).  Each warm-up
    step is a 5,000-row build of a separate model."""
    if rank != 0:
        return
    from oracle.refbuild import build_ref

    n, d = X.shape
    if not build_ref.reference_available():
        print(json.dumps({"impl": "reference", "unavailable": "the reference build is not installed "
                          "(oracle/refbuild/build_ref.py found no reference sources to compile)"}))
        return
    import torch

    torch.cuda.set_device(0)
    from oracle.refbuild import refrun

    X_dev = torch.from_numpy(X).cuda()
    q_idx = np.random.default_rng(123).choice(n, min(RECALL_QUERIES, n), replace=False)
    exact = exact_knn_gpu(X_dev, q_idx, K)
    upd, emb = UPD_OPS, args.embedding_ops
    for _ in range(args.warmup):
        m = refrun.make_model(X[:REF_WARMUP_ROWS], k=K, max_epoch=MAX_EPOCH)
        for c in range(0, REF_WARMUP_ROWS, CHUNK):
            m.run_with_n_ops(CHUNK, upd, emb)
        torch.cuda.synchronize()
        m.close()
        del m
    cycles = list(range(0, n, CHUNK))
    parts = [cycles[len(cycles) * i // args.steps: len(cycles) * (i + 1) // args.steps] for i in range(args.steps)]
    model = refrun.make_model(X, k=K, max_epoch=MAX_EPOCH)
    times, rounds, rec = [], 0, 0.0
    with ClockSampler(0) as clk:
        for i, part in enumerate(parts):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for c in part:
                model.run_with_n_ops(min(CHUNK, n - c), upd, emb)
            if i == len(parts) - 1:
                rec = recall(refrun.neighbor_indices(model)[q_idx], exact)
                while rec < RECALL_TARGET and rounds < args.max_final_updates:
                    model.run_with_n_ops(0, n, 0)
                    rounds += 1
                    prev, rec = rec, recall(refrun.neighbor_indices(model)[q_idx], exact)
                    if rec - prev < REF_PLATEAU:
                        break
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    total = sum(times)
    trust, knnp = embed_quality(X_dev, refrun.embedding(model), quality_subset(n))
    model.close()
    del model
    value = n / total
    config = {"workload": f"image-like mixture {n}x{d}, k={K}, euclidean, {CHUNK} points/cycle, "
                          f"run_with_n_ops({CHUNK},{upd},{emb}) per cycle, then run_with_n_ops(0,{n},0) while "
                          f"recall@15<{RECALL_TARGET} and a cycle adds >= {REF_PLATEAU}",
              "implementation": "the reference's own CUDA build (unmodified sources, nvcc sm_103a, RAFT/RMM "
                                "stand-in headers), driven through its Python GPUMAP over host arrays",
              "n_points": n, "n_features": d, "n_neighbors": K, "max_epoch": MAX_EPOCH,
              "update_ops": upd, "embedding_ops": emb,
              "steps_are": f"one complete build split into {args.steps} timed parts; "
                           f"warm-up steps are {REF_WARMUP_ROWS}-row builds",
              "parallelism": "single GPU"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded image-like mixture, 70k x 784)", "config": config,
            "recall_at_15": rec, "recall_valid": rec >= RECALL_TARGET, "final_update_cycles": rounds,
            "trustworthiness": trust, "knn_preservation": knnp,
            "quality_subset": f"{len(quality_subset(n))} seeded rows (seed {QUALITY_SEED})",
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": n * d * 4 // args.steps,
                    "d2h_bytes_per_step": 0, "note": "the reference's API takes host arrays: its timed "
                                                     "region includes every append's host-to-device copy"},
            "clocks": clk.summary()}
    # the reference's own latency-driven loop, run(target_latency=10), as far
    # as a bounded time allows
    try:
        m = refrun.make_model(X, k=K, max_epoch=MAX_EPOCH)
        np.random.seed(0)
        allocs, t0 = [], time.perf_counter()
        while time.perf_counter() - t0 < 120.0:
            r = m.run(10.0)
            allocs.append([int(r.n_insertion_ops), int(r.n_update_ops), int(r.n_embedding_ops)])
            if r.n_inserted_instances >= n:
                break
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        rows = int(r.n_inserted_instances)
        line["run10"] = {"value": rows / dt, "unit": "points/s", "rows_inserted": rows, "seconds": dt,
                         "cycles": len(allocs), "allocations": allocs,
                         "recall_at_15": recall(refrun.neighbor_indices(m)[q_idx], exact) if rows >= n else None}
        m.close()
    except Exception as e:  # a sub-line; the headline stands without it
        line["run10"] = {"error": str(e)[:200]}
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_info()
    # pure Python (the package's native library is not loaded by this import)
    from gpumap_gb300.datasets import image_like

    if args.workload != "image-70k" and args.impl != "reference":
        import torch

        from gpumap_gb300 import _native

        torch.cuda.set_device(0)
        _native.load()
        if args.workload == "cosine-1m":
            kw = {"n": args.rows, "fp32_rows": min(200_000, args.rows)} if args.rows else {}
            print(json.dumps({"workload_line": "cosine-1m", **cosine_1m_run(_native, **kw)}))
        elif args.workload == "batched-64":
            print(json.dumps({"workload_line": "batched-64", **batched_run(_native)}))
        else:
            print(json.dumps({"workload_line": "serving", "rate_40": serving_run(_native),
                              "rate_100": serving_run(_native, rate=100.0, capacity=False)}))
        return
    n, d = args.n_points, N_FEATURES
    X, _ = image_like(n, d, seed=0)
    if args.impl == "reference":
        reference_arm(args, X, rank)
        return

    upd = args.update_ops if args.update_ops is not None else (0 if args.precision == 1 else UPD_OPS)
    emb = args.embedding_ops
    config = {"workload": f"image-like mixture {n}x{d}, k={K}, euclidean, {CHUNK} points/cycle, "
                          f"run_with_n_ops({CHUNK},{upd},{emb}) per cycle, then "
                          f"run_with_n_ops(0,{n},0) until recall@15>={RECALL_TARGET}",
              "n_points": n, "n_features": d, "n_neighbors": K, "max_epoch": MAX_EPOCH,
              "precision": args.precision, "overlap": args.overlap, "update_ops": upd,
              "embedding_ops": emb,
              "schedule": f"headline: run_with_n_ops({CHUNK},{upd},{emb}); the plain schedule "
                          f"run_with_n_ops({CHUNK},{UPD_OPS},{emb}) is the schedule_u2000 line",
              "l2": "inputs (220 MB) larger than L2; 512 MB flush between steps",
              "parallelism": "replicas" if world > 1 else "single GPU"}

    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from gpumap_gb300 import _native

    native = _native
    native.load()
    X_dev = torch.from_numpy(X).cuda()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    q_idx = np.random.default_rng(123).choice(n, min(RECALL_QUERIES, n), replace=False)
    exact = exact_knn_gpu(X_dev, q_idx, K)
    sub = quality_subset(n)

    def step(precision, u, stats_on, overlap=args.overlap):
        return run_value_step(native, X_dev, n, d, u, emb, args.max_final_updates, stats_on, q_idx, exact,
                              precision, overlap)

    def quality(session):
        e = session.copy("embedding", np.float32).reshape(-1, 2)[:n]
        t, kp = embed_quality(X_dev, e, sub)
        return {"trustworthiness": t, "knn_preservation": kp}

    for _ in range(args.warmup):
        s, _, _, _, _ = step(args.precision, upd, False)
        del s
    barrier(world)
    times, recalls, rounds_l, launches, stats = [], [], [], 0, []
    last = None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            barrier(world)
            s, ms, st, rec, rounds = step(args.precision, upd, True)
            times.append(ms)
            rounds_l.append(rounds)
            launches += st.kernel_launches
            stats.append(st)
            recalls.append(rec)
            last = s
    total_ms = max_over_ranks(sum(times), world)
    ms_step = total_ms / args.steps
    value = world * n * args.steps / (total_ms / 1000.0)
    q_value = quality(last)
    del last

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    dom, kernels = roofline(stats, d, peaks)
    roof = dict(kernels[dom]) if dom else {}
    if dom:
        roof = {"kernel": dom, "bound": roof["bound"], "achieved": roof["achieved"], "peak": roof["peak"],
                "unit": roof["unit"], "frac": roof["frac"], "traffic": roof.get("traffic"),
                "peak_source": "measured (MEASURED_PEAKS.json, sustained bf16 / hbm copy)"}
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16+f32" if args.precision == 1 else "f32",
        "data": "synthetic (seeded image-like mixture, 70k x 784)", "config": config,
        "recall_at_15": min(recalls), "recall_valid": min(recalls) >= RECALL_TARGET,
        "final_update_cycles": rounds_l, "gpu_launches": int(launches), **q_value,
        "quality_subset": f"{len(sub)} seeded rows (seed {QUALITY_SEED}); both spaces restricted to them",
        "roofline": roof,
        "kernels": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                    for k, v in kernels.items()},
        "phase_s": [sum(s_.phase_s[i] for s_ in stats) / args.steps for i in range(3)],
    }
    if args.precision == 1:
        line["exact_pairs_per_step"] = sum(s_.exact_pairs for s_ in stats) / args.steps
        line["exact_rescored_per_step"] = sum(s_.exact_rescored for s_ in stats) / args.steps
    line["clocks"] = clk.summary()

    def subline(precision, u, overlap, **extra):
        s, _, _, _, _ = step(precision, u, False, overlap=overlap)
        del s
        flush_l2(flush)
        s, ms_s, _, rec_s, rounds_s = step(precision, u, False, overlap=overlap)
        out = {"value": n / (ms_s / 1000.0), "unit": "points/s", "recall_at_15": rec_s,
               "recall_valid": rec_s >= RECALL_TARGET, "final_update_cycles": rounds_s, **quality(s), **extra}
        del s
        return out

    if args.overlap:
        # the same build with the phases one after another (the reference's
        # order of work on the device)
        line["value_no_overlap"] = subline(args.precision, upd, 0)
    if args.precision == 1 and not args.no_u2000 and upd != UPD_OPS:
        # the same exact insertion under the plain schedule (U = 2000
        # NN-Descent update ops per cycle, which find nothing left to improve)
        line["schedule_u2000"] = subline(1, UPD_OPS, args.overlap,
                                         schedule=f"run_with_n_ops({CHUNK},{UPD_OPS},{emb})")
    if args.precision == 1 and not args.no_plain:
        line["plain_fp32"] = subline(0, UPD_OPS, args.overlap,
                                     schedule=f"run_with_n_ops({CHUNK},{UPD_OPS},{emb}) then up to "
                                              f"{args.max_final_updates} full update cycles",
                                     note="the reference's NN-Descent restated (precision 0)")
    X_pin = None
    if not args.no_e2e:
        X_pin = torch.from_numpy(X).pin_memory().numpy()
        run_e2e_step(X_pin, n, d, upd, emb, args.max_final_updates, q_idx, exact, args.precision, args.overlap)
        e2e_t, e2e_rec = [], []
        for _ in range(max(1, min(args.steps, 3))):
            flush_l2(flush)
            dt, rec, _ = run_e2e_step(X_pin, n, d, upd, emb, args.max_final_updates, q_idx, exact, args.precision,
                                      args.overlap)
            e2e_t.append(dt)
            e2e_rec.append(rec)
        tmax = max_over_ranks(sum(e2e_t), world)
        line["e2e"] = {"value": world * n * len(e2e_t) / tmax, "unit": "points/s",
                       "h2d_bytes_per_step": n * d * 4, "d2h_bytes_per_step": n * K * 4,
                       "recall_at_15": min(e2e_rec)}
        # the same from an ordinary (pageable) numpy array: rows staged
        # through the engine's pinned ingest ring
        flush_l2(flush)
        dt, rec, _ = run_e2e_step(X, n, d, upd, emb, args.max_final_updates, q_idx, exact, args.precision,
                                  args.overlap)
        line["e2e"]["pageable_host_rows"] = {"value": n / dt, "unit": "points/s", "recall_at_15": rec}
    if not args.no_run10:
        # the latency-driven loop: GPUMAP.run(target_latency=10) with the
        # default weighted strategy, from a cold start
        if X_pin is None:
            X_pin = torch.from_numpy(X).pin_memory().numpy()
        dt, rec, cyc, allocs, model = run_target_latency(X_pin, n, d, q_idx, exact, args.precision, args.overlap)
        t, kp = embed_quality(X_dev, model.get_embedding(), sub)
        model.close()
        line["run10"] = {"value": n / dt, "unit": "points/s", "seconds": dt, "recall_at_15": rec,
                         "recall_valid": rec >= RECALL_TARGET, "cycles": cyc, "allocations": allocs,
                         "trustworthiness": t, "knn_preservation": kp}
    if not args.no_serving and world == 1:
        line["serving"] = serving_run(native)
    if rank == 0 and not args.no_cpu_baseline:
        v, rows, dt = fp64_bruteforce_baseline(X, K)
        line["cpu_baseline"] = {"value": v, "unit": "rows/s (exact FP64 k-NN)", "cores": os.cpu_count(),
                                "cpu": cpu_model(), "kind": "fp64 brute force",
                                "sample": f"{rows} seeded query rows against all {n} rows in {dt:.1f} s "
                                          "(numpy float64 GEMM, BLAS threads on every host core)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
