"""Builds the native parts of gpumap_gb300 in-tree.

* ``gpumap_gb300/_lib/libgpumap_gb300.so`` -- CUDA kernels, engine and C ABI,
  compiled by nvcc for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
* ``gpumap_gb300/_core*.so`` -- pybind11 module over the C ABI; pybind11 comes
  from the headers bundled with PyTorch (no separate pybind11 install needed).

Translation units compile in parallel; unchanged objects are reused.
"""
from __future__ import annotations

import importlib.util
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
ROOT = PKG.parent
OBJDIR = ROOT / "_build" / "obj"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC"]
LIB_NAME = "libgpumap_gb300.so"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def lib_path() -> Path:
    return LIBDIR / LIB_NAME


def core_path() -> Path:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return PKG / f"_core{suffix}"


def _torch_include() -> Path:
    spec = importlib.util.find_spec("torch")
    if spec is None or spec.origin is None:
        raise RuntimeError("PyTorch headers (for pybind11) not found")
    inc = Path(spec.origin).parent / "include"
    if not (inc / "pybind11" / "pybind11.h").exists():
        raise RuntimeError(f"pybind11 headers not found under {inc}")
    return inc


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    OBJDIR.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    srcs = sorted(CSRC.glob("*.cu")) + [p for p in sorted(CSRC.glob("*.cpp")) if p.name != "gm_core_pybind.cpp"]
    jobs_to_run = []
    objs = []
    for src in srcs:
        obj = OBJDIR / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src, *hdrs]):
            continue
        cmd = [nvcc, *ARCH, *NVCC_FLAGS]
        if src.suffix == ".cpp":
            cmd += ["-x", "cu"]
        cmd += ["-c", str(src), "-o", str(obj)]
        jobs_to_run.append(cmd)
    with ThreadPoolExecutor(max_workers=jobs or min(8, max(1, os.cpu_count() or 1))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs_to_run))
    lib = lib_path()
    if jobs_to_run or not _newer(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs)], verbose)
    return lib


def build_core(verbose: bool = False) -> Path:
    src = CSRC / "gm_core_pybind.cpp"
    out = core_path()
    lib = lib_path()
    if _newer(out, [src, lib, *_headers()]):
        return out
    py_inc = sysconfig.get_paths()["include"]
    cxx = os.environ.get("CXX", "g++")
    cmd = [
        cxx, "-O2", "-shared", "-fPIC", "-std=c++17", "-fvisibility=hidden",
        f"-I{_torch_include()}", f"-I{py_inc}", str(src),
        f"-L{LIBDIR}", "-lgpumap_gb300", "-Wl,-rpath,$ORIGIN/_lib", "-o", str(out),
    ]
    _run(cmd, verbose)
    return out


def build(verbose: bool = False) -> None:
    build_library(verbose)
    build_core(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(lib_path())
    print(core_path())
