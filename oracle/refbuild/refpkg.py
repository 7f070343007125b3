"""Imports the reference's own Python package (``gpumap``, installed with its
compiled ``_core`` under ``baseline/_ref`` by ``oracle/refbuild/build_ref.py``).

Test and benchmark infrastructure only.  Two of the reference's imports are
absent on the GPU machine and stand-ins are registered for them before the
import, touching none of the reference's code:

* ``cupy`` -- the reference wraps its ``__cuda_array_interface__`` views with
  ``cupy.asarray`` (python/gpumap/gpumap.py:148-162); the stand-in wraps them
  with ``torch.as_tensor`` on the current CUDA device, which reads the same
  interface and supports the same slicing.
* ``sklearn.datasets.fetch_openml`` -- imported at module level by the
  reference's data loader (python/gpumap/data_loader.py:4) and used only by
  its download-based loaders, which are not used here.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

REF_DIR = Path(__file__).resolve().parent.parent.parent / "baseline" / "_ref"


def _cupy_standin() -> types.ModuleType:
    m = types.ModuleType("cupy")

    class _View:
        # torch rejects the read-only flag the reference sets on its views;
        # the stand-in only reads through them
        def __init__(self, cai):
            d = dict(cai)
            d["data"] = (d["data"][0], False)
            self.__cuda_array_interface__ = d

    def asarray(obj):
        import torch

        return torch.as_tensor(_View(obj.__cuda_array_interface__), device="cuda")

    m.asarray = asarray
    m.ndarray = object
    return m


def _sklearn_standin() -> tuple[types.ModuleType, types.ModuleType]:
    sk = types.ModuleType("sklearn")
    ds = types.ModuleType("sklearn.datasets")

    def fetch_openml(*a, **k):
        raise RuntimeError("dataset download is not available (no network)")

    ds.fetch_openml = fetch_openml
    sk.datasets = ds
    return sk, ds


def load():
    """Returns the reference's ``gpumap`` package, or raises ImportError."""
    if "gpumap" in sys.modules:
        return sys.modules["gpumap"]
    if not (REF_DIR / "gpumap").is_dir():
        raise ImportError(f"reference not installed under {REF_DIR}")
    try:
        import cupy  # noqa: F401
    except ImportError:
        sys.modules["cupy"] = _cupy_standin()
    try:
        import sklearn.datasets  # noqa: F401
    except ImportError:
        sk, ds = _sklearn_standin()
        sys.modules.setdefault("sklearn", sk)
        sys.modules["sklearn.datasets"] = ds
    if str(REF_DIR) not in sys.path:
        sys.path.insert(0, str(REF_DIR))
    import gpumap

    if not Path(gpumap.__file__).resolve().is_relative_to(REF_DIR.resolve()):
        raise ImportError(f"imported gpumap from {gpumap.__file__}, not the reference install")
    return gpumap
