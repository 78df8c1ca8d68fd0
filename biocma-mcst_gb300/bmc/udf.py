"""Runtime-loaded cell models ("udf_model"): build, load, describe.

A model library is one CUDA source file that defines a model struct and
expands ``BMC_DEFINE_UDF`` (``csrc/bmc_udf.cuh``).  :func:`build_udf`
compiles it with the library's own flags into ``lib/udf/<name>.so``;
:func:`load_udf` registers it with libbmc (``bmc_udf_load``) and returns the
model id to use in a scenario; :func:`udf_model` wraps both into a
:class:`~bmc.scenarios.ModelSpec`.

Reference: the reference builds a UDF as a shared library (apps/udf_model/
meson.build) and binds it with UnsafeUDF::Loader::init_lib
(apps/libs/models/ext/udf_includes.cpp L58-L78).
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

from . import _lib
from . import build as _build

UDF_DIR = os.path.join(_build.LIBDIR, "udf")
EXAMPLES = os.path.join(_build.PKG, "udf")
HEADERS = ("bmc_udf.cuh", "bmc_kernel_templates.cuh", "bmc_kernels.cuh", "bmc_device.cuh",
           "bmc_launch.h")


def example(name: str) -> str:
    """Path of a model source shipped in the package's ``udf/`` folder."""
    return os.path.join(EXAMPLES, name)


def _stale(src: str, out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = [src, os.path.join(os.path.dirname(_build.PKG), "include", "bmc.h")]
    deps += [os.path.join(_build.CSRC, h) for h in HEADERS]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_udf(src: str, out: str | None = None, force: bool = False) -> str:
    """Compile a model source into a model library (sm_103a, separately
    rounded multiply/add on device and host, hidden visibility)."""
    name = os.path.splitext(os.path.basename(src))[0]
    out = out or os.path.join(UDF_DIR, f"lib{name}.so")
    if not force and not _stale(src, out):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp"
    cmd = [_build.nvcc(), *_build.ARCH, *_build.FLAGS, "-Xcompiler", "-fvisibility=hidden",
           "--cudart", "shared", "-shared", "-I", _build.CSRC, src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"model library build failed for {src}:\n{r.stderr}")
    os.replace(tmp, out)
    return out


def load_udf(path: str | None) -> int:
    """Register a model library with libbmc; returns its model id.  With
    path None, libbmc reads the path from BIOMC_LIB_UDF."""
    mid = ct.c_int32()
    _lib.call("bmc_udf_load", None if path is None else path.encode(), ct.byref(mid))
    return mid.value


def udf_info(model_id: int) -> dict:
    info = _lib.UdfInfo()
    _lib.call("bmc_udf_get_info", model_id, ct.byref(info))
    return {
        "n_var": info.n_var, "n_ctb": info.n_ctb, "separable": bool(info.separable),
        "f32": bool(info.has_f32), "f64": bool(info.has_f64),
        "names": [info.names[k].decode() for k in range(info.n_names)],
        "species": [info.species[k].decode() for k in range(info.n_species)],
    }


def host_model(model_id: int, f64: bool) -> _lib.UdfHostModel:
    m = _lib.UdfHostModel()
    _lib.call("bmc_udf_get_host_model", model_id, 1 if f64 else 0, ct.byref(m))
    return m


def udf_model(src: str, f64: bool, params=None, value_bound=None, name: str | None = None):
    """Build and load a model library; returns the ModelSpec of a scenario
    that uses it.  value_bound: bound on |basis| (separable models) or on
    |contribution j| of one particle (general models)."""
    from .scenarios import ModelSpec

    path = build_udf(src)
    mid = load_udf(path)
    info = udf_info(mid)
    p = np.zeros(16)
    if params is not None:
        p[: len(params)] = params
    vb = np.asarray(value_bound if value_bound is not None else [1.0], dtype=np.float64)
    names = tuple(info["names"])
    return ModelSpec(name or os.path.splitext(os.path.basename(src))[0], mid, info["n_var"],
                     info["n_ctb"], f64, p, vb, separable=info["separable"], udf_path=path,
                     export_names=names, export_index=tuple(range(len(names))),
                     species=tuple(info["species"]))
