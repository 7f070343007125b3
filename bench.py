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
* ``plain_fp32`` -- the reference's own algorithm (precision 0, FP32
  NN-Descent) on the same workload and clock, for comparison.
* ``e2e``    -- the public Python API (gpumap_gb300.GPUMAP over pinned host
  chunks; every cycle copies its 500 rows host->device, each step ends by
  reading the k-NN table back to the host).
* ``roofline`` -- the kernel with the largest summed time, its algorithmic
  bytes (or FLOPs) over its CUDA-event time (events recorded by the engine on
  its own stream), against MEASURED_PEAKS.json.
* ``cpu_baseline`` / ``--impl reference`` -- the CPU restatement of the
  reference path (oracle/) on a bounded sample of the same workload.

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


def cpu_baseline_sample(X, upd, emb, cycles=2):
    """Oracle (CPU restatement of the reference path) on the first cycles of
    the workload: points inserted per second, single thread."""
    from oracle.session import OracleSession

    n = cycles * CHUNK
    o = OracleSession(n, X.shape[1], k=K, max_epoch=MAX_EPOCH, a=1.5769434602697652, b=0.8950608778515733)
    t0 = time.perf_counter()
    for c in range(cycles):
        o.append(X[c * CHUNK : (c + 1) * CHUNK])
        o.run(CHUNK, min(upd, n), min(emb, n))
    dt = time.perf_counter() - t0
    return n / dt, dt, n


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# ncu captures of the 30,000-point cut of this workload (k_exact_dist: cycle
# 41, 20,500 columns, profiles/k_exact_dist_30k_x784.md; k_sgd_persistent:
# cycle 40, profiles/k_sgd_persistent_30k_x784.md).  "per" names the unit the
# traffic scales with, so that a capture can be carried to this run's mean
# launch: k_exact_dist reads its B operand once per launch (bytes ~ FLOPs);
# the SGD launch's traffic is the first touch of its edge arrays (about the
# same per embedding call at any size, so it is used as measured).
NCU_TRAFFIC = {
    "k_exact_dist": {"bytes": 69587968 + 5130496, "per": "flop", "units": 6 * 500 * 20500 * 832},
    "k_sgd_persistent": {"bytes": 864512 + 79104, "per": "launch", "units": 1},
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


def main():
    args = parse()
    rank, world, local = dist_info()
    from gpumap_gb300.datasets import image_like

    n, d = args.n_points, N_FEATURES
    X, _ = image_like(n, d, seed=0)
    upd = args.update_ops if args.update_ops is not None else (0 if args.precision == 1 else UPD_OPS)
    emb = args.embedding_ops
    config = {"workload": f"image-like mixture {n}x{d}, k={K}, euclidean, {CHUNK} points/cycle, "
                          f"run_with_n_ops({CHUNK},{upd},{emb}) per cycle, then "
                          f"run_with_n_ops(0,{n},0) until recall@15>={RECALL_TARGET}",
              "n_points": n, "n_features": d, "n_neighbors": K, "max_epoch": MAX_EPOCH,
              "precision": args.precision, "overlap": args.overlap, "update_ops": upd,
              "embedding_ops": emb,
              "l2": "inputs (220 MB) larger than L2; 512 MB flush between steps",
              "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        steps = []
        for i in range(args.warmup + args.steps):
            v, dt, npts = cpu_baseline_sample(X, UPD_OPS, emb, cycles=1)
            if i >= args.warmup:
                steps.append((v, dt))
        val = statistics.median([v for v, _ in steps])
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "points/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * statistics.median([t for _, t in steps]),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": val, "unit": "points/s", "cores": 1, "kind": "port",
                                 "sample": f"first {CHUNK} rows, one cycle run_with_n_ops({CHUNK},{UPD_OPS},{emb}) of "
                                           "the reference algorithm on one host thread; the reference's CUDA build "
                                           "is unavailable (needs RAFT/RMM and CUDA 12.6)"},
                "e2e": {"value": val, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

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

    def step(precision, u, stats_on, overlap=args.overlap):
        return run_value_step(native, X_dev, n, d, u, emb, args.max_final_updates, stats_on, q_idx, exact,
                              precision, overlap)

    for _ in range(args.warmup):
        s, _, _, _, _ = step(args.precision, upd, False)
        del s
    barrier(world)
    times, recalls, rounds_l, launches, stats = [], [], [], 0, []
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
            del s
    total_ms = max_over_ranks(sum(times), world)
    ms_step = total_ms / args.steps
    value = world * n * args.steps / (total_ms / 1000.0)

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
        "final_update_cycles": rounds_l, "gpu_launches": int(launches),
        "roofline": roof,
        "kernels": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                    for k, v in kernels.items()},
        "phase_s": [sum(s_.phase_s[i] for s_ in stats) / args.steps for i in range(3)],
    }
    if args.precision == 1:
        line["exact_pairs_per_step"] = sum(s_.exact_pairs for s_ in stats) / args.steps
        line["exact_rescored_per_step"] = sum(s_.exact_rescored for s_ in stats) / args.steps
    line["clocks"] = clk.summary()

    if args.overlap:
        # the same build with the phases one after another (the reference's
        # order of work on the device)
        s, _, _, _, _ = step(args.precision, upd, False, overlap=0)
        del s
        flush_l2(flush)
        s, ms_s, _, rec_s, _ = step(args.precision, upd, False, overlap=0)
        del s
        line["value_no_overlap"] = {"value": n / (ms_s / 1000.0), "unit": "points/s", "recall_at_15": rec_s}

    if args.precision == 1 and not args.no_u2000 and upd != UPD_OPS:
        # the same exact insertion under the plain path's schedule (U = 2000
        # NN-Descent update ops per cycle, which find nothing left to improve)
        s, _, _, _, _ = step(1, UPD_OPS, False)
        del s
        flush_l2(flush)
        s, ms1, _, rec1, rounds1 = step(1, UPD_OPS, False)
        del s
        line["schedule_u2000"] = {"value": n / (ms1 / 1000.0), "unit": "points/s", "recall_at_15": rec1,
                                  "schedule": f"run_with_n_ops({CHUNK},{UPD_OPS},{emb})",
                                  "final_update_cycles": rounds1}

    if args.precision == 1 and not args.no_plain:
        s, _, _, _, _ = step(0, UPD_OPS, False)
        del s
        flush_l2(flush)
        s, ms0, _, rec0, rounds0 = step(0, UPD_OPS, False)
        del s
        line["plain_fp32"] = {"value": n / (ms0 / 1000.0), "unit": "points/s", "recall_at_15": rec0,
                              "recall_valid": rec0 >= RECALL_TARGET, "final_update_cycles": rounds0,
                              "schedule": f"run_with_n_ops({CHUNK},{UPD_OPS},{emb}) then up to "
                                          f"{args.max_final_updates} full update cycles",
                              "note": "the reference's NN-Descent (precision 0); it plateaus below the recall "
                                      "target on this workload"}

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
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, npts = cpu_baseline_sample(X, UPD_OPS, emb, cycles=2)
        line["cpu_baseline"] = {"value": v, "unit": "points/s", "cores": 1, "kind": "port",
                                "sample": f"first {npts} rows in {npts // CHUNK} cycles of run_with_n_ops({CHUNK},"
                                          f"{UPD_OPS},{emb}) of the reference algorithm, {dt:.1f} s, one host thread"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
