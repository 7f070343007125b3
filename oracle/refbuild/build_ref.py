"""Builds the reference's own CUDA path (jjmmwon/gpumap, unmodified) for
sm_103a, as the like-for-like baseline and as a parity pin.

The reference's build needs RAPIDS (RAFT/RMM 26.02), conda and CMake; none
of them is used here.  Instead:

* ``install()`` copies the reference's ``cpp/`` tree and its Python package
  ``python/gpumap`` into ``baseline/_ref/src`` (git-ignored; it travels with
  the repository to the GPU machine, where the reference tree is absent).
  The source tree is taken from the ``GPUMAP_REFERENCE`` environment
  variable, or the ``src`` argument, else from the read-only mount this
  recipe was written against.
* ``build()`` compiles ``cpp/bindings/binding.cu`` and ``cpp/src/impl.cu``
  exactly as shipped with nvcc (``-gencode arch=compute_103a,code=sm_103a``)
  against the stand-in headers in ``oracle/refbuild/shim`` (RAFT/RMM names
  only) and the pybind11 headers bundled with PyTorch, into the extension
  ``baseline/_ref/gpumap/_core``, next to an unmodified copy of the
  reference's Python package.  That is the layout ``pip install --target
  baseline/_ref`` would have produced.  One object is added to the module:
  ``zeroed_new.cpp``, a zero-filling operator new with hidden visibility,
  which makes an uninitialised read in the reference's Bloom filter
  deterministic (the file says why).  It also compiles two test drivers
  into ``baseline/_ref/bin``: ``ref_fuzzy_driver`` (the reference's own
  fuzzy-set and edge-scheduling functions on a k-NN table read from a file,
  oracle/refbuild/ref_fuzzy_driver.cu) and ``ref_embed_driver`` (its whole
  embedding step, SGD included, on a table and an initial embedding,
  oracle/refbuild/ref_embed_driver.cu).

``reference_available()`` says whether the built module is present.
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
SHIM = HERE / "shim"
REF_OUT = ROOT / "baseline" / "_ref"
SRC_COPY = REF_OUT / "src"
PKG_OUT = REF_OUT / "gpumap"
OBJ = REF_OUT / "_obj"
BIN = REF_OUT / "bin"
DEFAULT_SRC = "/root/reference"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "-DLIBCUDACXX_ENABLE_EXPERIMENTAL_MEMORY_RESOURCE", "--expt-relaxed-constexpr", "--extended-lambda",
         "-diag-suppress", "177,550,20012,20014"]


def _source(src: str | None) -> Path | None:
    cand = src or os.environ.get("GPUMAP_REFERENCE") or DEFAULT_SRC
    p = Path(cand)
    return p if (p / "cpp" / "src" / "impl.cuh").exists() else None


def install(src: str | None = None) -> bool:
    """Copies the reference sources into baseline/_ref/src (no edits)."""
    ref = _source(src)
    if ref is None:
        return SRC_COPY.exists()
    SRC_COPY.mkdir(parents=True, exist_ok=True)
    for part in ("cpp", "python/gpumap"):
        dst = SRC_COPY / part
        if dst.exists():
            shutil.rmtree(dst)
        shutil.copytree(ref / part, dst, ignore=shutil.ignore_patterns("__pycache__"))
    _writable(SRC_COPY)
    return True


def _writable(root: Path) -> None:
    # the mount is read-only; the copy must stay replaceable
    for p in [root, *root.rglob("*")]:
        p.chmod(p.stat().st_mode | 0o200)


def core_path() -> Path:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return PKG_OUT / f"_core{suffix}"


def fuzzy_driver_path() -> Path:
    return BIN / "ref_fuzzy_driver"


def embed_driver_path() -> Path:
    return BIN / "ref_embed_driver"


def reference_available() -> bool:
    return core_path().exists()


def _torch_include() -> Path:
    spec = importlib.util.find_spec("torch")
    if spec is None or spec.origin is None:
        raise RuntimeError("PyTorch (for its bundled pybind11 headers) not found")
    return Path(spec.origin).parent / "include"


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build(verbose: bool = False) -> Path | None:
    """Compiles the reference module; returns its path, or None when the
    reference sources are not installed."""
    cpp = SRC_COPY / "cpp"
    if not (cpp / "src" / "impl.cu").exists():
        return None
    out = core_path()
    deps = sorted(cpp.rglob("*.cu*")) + sorted(SHIM.rglob("*.h*")) + [HERE / "ref_fuzzy_driver.cu",
                                                                      HERE / "ref_embed_driver.cu",
                                                                      HERE / "zeroed_new.cpp",
                                                                      HERE / "zeroed_new.map"]
    OBJ.mkdir(parents=True, exist_ok=True)
    PKG_OUT.mkdir(parents=True, exist_ok=True)
    # the reference's Python package, unmodified
    for f in (SRC_COPY / "python" / "gpumap").rglob("*"):
        if f.is_file():
            dst = PKG_OUT / f.relative_to(SRC_COPY / "python" / "gpumap")
            dst.parent.mkdir(parents=True, exist_ok=True)
            if not dst.exists() or dst.stat().st_mtime < f.stat().st_mtime:
                if dst.exists():
                    dst.unlink()
                shutil.copy2(f, dst)
                dst.chmod(dst.stat().st_mode | 0o200)
    if _newer(out, deps) and _newer(fuzzy_driver_path(), deps) and _newer(embed_driver_path(), deps):
        return out
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    if not os.path.exists(nvcc):
        nvcc = "nvcc"
    inc = [f"-I{SHIM}", f"-I{cpp / 'include'}", f"-I{cpp / 'src'}", f"-I{cpp / 'bindings'}",
           f"-I{_torch_include()}", f"-I{sysconfig.get_paths()['include']}"]
    units = [cpp / "bindings" / "binding.cu", cpp / "src" / "impl.cu"]
    cmds = [[nvcc, *ARCH, *FLAGS, *inc, "-c", str(u), "-o", str(OBJ / (u.stem + ".o"))] for u in units]
    # zero-filled allocations inside the module (see zeroed_new.cpp: the
    # reference's Bloom filter reads members before they are initialised)
    cmds.append([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-c",
                 str(HERE / "zeroed_new.cpp"), "-o", str(OBJ / "zeroed_new.o")])
    BIN.mkdir(parents=True, exist_ok=True)
    for drv, path in (("ref_fuzzy_driver.cu", fuzzy_driver_path()), ("ref_embed_driver.cu", embed_driver_path())):
        cmds.append([nvcc, *ARCH, *FLAGS, f"-I{SHIM}", f"-I{cpp / 'include'}", f"-I{cpp / 'src'}",
                     str(HERE / drv), "-o", str(path)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr[-6000:]}")

    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(run, cmds))
    run([nvcc, *ARCH, "-shared", "-o", str(out), *[str(OBJ / (u.stem + ".o")) for u in units],
         str(OBJ / "zeroed_new.o"), "-Xlinker", f"--version-script={HERE / 'zeroed_new.map'}"])
    return out


if __name__ == "__main__":
    install(sys.argv[1] if len(sys.argv) > 1 else None)
    print(build(verbose=True))
