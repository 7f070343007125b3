"""Builds the CPU oracle (test infrastructure only).

* ``oracle/_build/libgm_oracle.so`` from ``oracle/gm_oracle.cpp`` (g++,
  -ffp-contract=off so no multiply-add is fused behind the code's back; on
  x86_64 -mfma lets fmaf() compile to one instruction, same result).
* ``oracle/_ref/queue_golden`` -- when the reference tree is present, the
  reference's own cpp/src/queue.cuh (plain C++, no RAFT/RMM) compiled in place
  with the driver ``oracle/ref_queue_driver.cpp``; used to regenerate the
  committed queue fixtures.  The reference's CUDA path is built separately by
  oracle/refbuild/build_ref.py.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# the reference tree: GPUMAP_REFERENCE, else the read-only mount this recipe was written against
REFERENCE = Path(os.environ.get("GPUMAP_REFERENCE", "/root/reference"))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(map(str, cmd)), flush=True)
    res = subprocess.run(list(map(str, cmd)), capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{res.stdout}\n{res.stderr}")


def lib_path() -> Path:
    return BUILD / "libgm_oracle.so"


def build_oracle(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "gm_oracle.cpp"
    out = lib_path()
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    _run([os.environ.get("CXX", "g++"), *flags, src, "-o", out], verbose)
    return out


def build_ref_queue(verbose: bool = False) -> Path | None:
    queue_h = REFERENCE / "cpp" / "src" / "queue.cuh"
    if not queue_h.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "queue_golden"
    drv = HERE / "ref_queue_driver.cpp"
    _run([os.environ.get("CXX", "g++"), "-O1", "-std=c++17", "-x", "c++", f"-I{queue_h.parent}",
          drv, "-o", out], verbose)
    return out


def build(verbose: bool = False) -> None:
    build_oracle(verbose)
    try:
        build_ref_queue(verbose)
    except RuntimeError as e:  # the reference is optional; report and continue
        print(f"reference queue build skipped: {e}", file=sys.stderr)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(lib_path())
