"""Fixtures that pin the oracle's embed-time fuzzy set and edge schedule to the
reference's own CUDA functions.

Two steps, because the inputs come from the CPU oracle and the outputs from
the reference's build on a GPU:

    python tests/golden/make_ref_fuzzy.py inputs         # here: writes ref_fuzzy_<case>.in
    python tests/golden/make_ref_fuzzy.py run OUTDIR     # GPU machine: runs
        baseline/_ref/bin/ref_fuzzy_driver (oracle/refbuild/build_ref.py) on
        every input and writes ref_fuzzy_<case>.out into OUTDIR

The ``.out`` files are then committed beside the inputs.  Input and output
layouts are documented in oracle/refbuild/ref_fuzzy_driver.cu.  Each case is
a published k-NN table (k+1 columns, the last one the dirty flag) produced by
progressive oracle cycles on a seeded mixture, plus the embedding batch.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

# name: (n, d, k, metric, cycles, batch rule, n_epochs, seed)
CASES = {
    "euclid_k15": (600, 24, 15, 0, 3, "all", 200, 3),
    "euclid_k15_partial": (600, 24, 15, 0, 3, "stride3", 200, 4),
    "cosine_k10": (500, 16, 10, 1, 2, "stride2", 200, 5),
    "euclid_k30": (900, 20, 30, 0, 3, "first400", 500, 6),
    "tiny_sentinels": (12, 5, 15, 0, 1, "all", 200, 7),
}


def case_inputs(name):
    from gpumap_gb300.datasets import gaussian_mixture
    from oracle.session import OracleSession

    n, d, k, metric, cycles, rule, n_epochs, seed = CASES[name]
    X, _ = gaussian_mixture(n, d, seed=seed)
    o = OracleSession(n, d, k=k, metric=metric, max_epoch=20)
    per = -(-n // cycles)
    for c in range(cycles):
        chunk = X[c * per: (c + 1) * per]
        o.append(chunk)
        o.run(len(chunk), 2 * len(chunk), len(chunk))
    pidx = o.copy("pub_idx", np.uint32).reshape(-1, k + 1)[:n]
    pdist = o.copy("pub_dist", np.float32).reshape(-1, k + 1)[:n]
    ids = np.arange(n, dtype=np.int32)
    batch = {"all": ids, "stride3": ids[::3], "stride2": ids[1::2], "first400": ids[:400]}[rule]
    return dict(n=n, k=k, euclidean=int(metric == 0), n_epochs=n_epochs, alpha=1.0,
                pub_idx=np.ascontiguousarray(pidx), pub_dist=np.ascontiguousarray(pdist),
                batch=np.ascontiguousarray(batch, dtype=np.int32))


def write_input(path: Path, c) -> None:
    with open(path, "wb") as f:
        np.array([c["n"], c["k"], c["euclidean"], len(c["batch"]), c["n_epochs"]], np.int32).tofile(f)
        np.array([c["alpha"]], np.float32).tofile(f)
        c["pub_idx"].astype(np.uint32).tofile(f)
        c["pub_dist"].astype(np.float32).tofile(f)
        c["batch"].astype(np.int32).tofile(f)


def read_input(path: Path):
    raw = path.read_bytes()
    n, k, eucl, nb, n_epochs = np.frombuffer(raw, np.int32, 5)
    alpha = float(np.frombuffer(raw, np.float32, 1, 20)[0])
    off = 24
    w = int(k) + 1
    pidx = np.frombuffer(raw, np.uint32, n * w, off).reshape(n, w)
    off += 4 * n * w
    pdist = np.frombuffer(raw, np.float32, n * w, off).reshape(n, w)
    off += 4 * n * w
    batch = np.frombuffer(raw, np.int32, nb, off)
    return dict(n=int(n), k=int(k), euclidean=int(eucl), n_epochs=int(n_epochs), alpha=alpha,
                pub_idx=pidx, pub_dist=pdist, batch=batch)


def read_output(path: Path, n: int):
    raw = path.read_bytes()
    nnz, extras, nnz2 = (int(v) for v in np.frombuffer(raw, np.int32, 3))
    max_w, rounding = (float(v) for v in np.frombuffer(raw, np.float32, 2, 12))
    off = 20
    out = dict(nnz=nnz, extras=extras, nnz2=nnz2, max_w=max_w, rounding=rounding)

    def take(key, dt, cnt):
        nonlocal off
        out[key] = np.frombuffer(raw, dt, cnt, off)
        off += 4 * cnt

    take("sigma", np.float32, n)
    take("rho", np.float32, n)
    take("coo_row", np.int32, nnz)
    take("coo_col", np.int32, nnz)
    take("coo_val", np.float32, nnz)
    take("t_row", np.int32, nnz2)
    take("t_col", np.int32, nnz2)
    take("t_eps", np.float32, nnz2)
    return out


def main():
    mode = sys.argv[1]
    if mode == "inputs":
        for name in CASES:
            write_input(HERE / f"ref_fuzzy_{name}.in", case_inputs(name))
            print("wrote", name)
    elif mode == "run":
        sys.path.insert(0, str(ROOT / "oracle" / "refbuild"))
        import build_ref

        drv = build_ref.fuzzy_driver_path()
        outdir = Path(sys.argv[2])
        outdir.mkdir(parents=True, exist_ok=True)
        for name in CASES:
            subprocess.run([str(drv), str(HERE / f"ref_fuzzy_{name}.in"), str(outdir / f"ref_fuzzy_{name}.out")],
                           check=True)
    else:
        raise SystemExit(f"unknown mode {mode}")


if __name__ == "__main__":
    main()
