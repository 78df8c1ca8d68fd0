"""Runtime-loaded cell models (the reference's "udf_model").

CPU part: a model library builds with nvcc, loads into libbmc without a
GPU, reports its metadata, exports nothing but its entry points, and its
host functions driven by the oracle reproduce the oracle's own compiled-in
Monod model bit for bit.  GPU part: the library's kernels give results
bit-identical to the built-in model and to the oracle driving the same
library's host functions.
"""
import ctypes as ct
import os
import re
import subprocess

import numpy as np
import pytest

from bmc import scenarios, udf
from conftest import ROOT

MINIMAL_PARAMS = [2e-8, 2e-6, 1e-3, 0.6e-6, 0.5]  # ldot_max, l_max, k, diameter, yield


def monod_udf_spec(f64: bool):
    base = scenarios.monod(f64=f64)
    return udf.udf_model(udf.example("monod_udf.cu"), f64, params=base.params[:6],
                         value_bound=base.value_bound)


def minimal_udf_spec():
    lin = np.float32(1000) * np.float32(np.pi) * np.float32(0.6e-6) ** 2 / np.float32(4)
    phi_max = float(np.float32(2e-8) * lin / np.float32(0.5))
    return udf.udf_model(udf.example("minimal_udf.cu"), False, params=MINIMAL_PARAMS,
                         value_bound=[2.0 * phi_max])


def test_library_builds_and_loads_without_gpu():
    spec = monod_udf_spec(True)
    assert spec.model_id >= 64
    info = udf.udf_info(spec.model_id)
    assert info == {"n_var": 2, "n_ctb": 1, "separable": True, "f32": True, "f64": True,
                    "names": ["mass", "age"], "species": ["glucose"]}
    # the same path maps to the same id
    assert udf.load_udf(spec.udf_path) == spec.model_id
    mini = minimal_udf_spec()
    assert mini.model_id != spec.model_id
    assert udf.udf_info(mini.model_id)["separable"] is False
    assert udf.udf_info(mini.model_id)["f64"] is False


def test_library_exports_only_its_entry_points():
    path = udf.build_udf(udf.example("minimal_udf.cu"))
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" [TDBR] (\w+)", out))
    assert exported == {"bmc_udf_abi", "bmc_udf_kernel_set", "set_nvar_udf", "set_nc_udf",
                        "separable_udf", "names_udf", "species_udf", "host_model_udf"}


def test_load_errors_and_env_path(monkeypatch):
    from bmc import _lib

    with pytest.raises(_lib.BmcError):
        udf.load_udf("/nonexistent/libnothing.so")
    # a shared library that is not a model library
    with pytest.raises(_lib.BmcError, match="not a model library"):
        udf.load_udf(_lib.lib_path())
    monkeypatch.delenv("BIOMC_LIB_UDF", raising=False)
    with pytest.raises(_lib.BmcError, match="BIOMC_LIB_UDF"):
        udf.load_udf(None)
    path = udf.build_udf(udf.example("monod_udf.cu"))
    monkeypatch.setenv("BIOMC_LIB_UDF", path)
    assert udf.load_udf(None) == udf.load_udf(path)
    with pytest.raises(_lib.BmcError, match="precision"):
        udf.host_model(udf.load_udf(udf.build_udf(udf.example("minimal_udf.cu"))), True)


def test_struct_layouts_match_header(tmp_path):
    from bmc import _lib

    src = tmp_path / "sz.c"
    src.write_text('#include "bmc.h"\n#include <stdio.h>\nint main(void){printf("%zu %zu\\n",'
                   'sizeof(bmc_udf_info), sizeof(bmc_udf_host_model));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert sizes == [ct.sizeof(_lib.UdfInfo), ct.sizeof(_lib.UdfHostModel)]


@pytest.mark.parametrize("f64", [True, False])
def test_oracle_with_library_host_functions_matches_builtin(oracle_mod, f64):
    """The library's host functions, driven by the oracle, reproduce the
    oracle's compiled-in Monod model bit for bit (divisions included)."""
    fast = scenarios.monod(f64=f64, mu_max=0.05)
    spec = monod_udf_spec(f64)
    spec.params[:] = fast.params
    sc_b = scenarios.small_ring(3000, f64=f64, model=fast, feeds=True)
    sc_b.alloc_factor = 3.0
    sc_u = scenarios.small_ring(3000, f64=f64, model=spec, feeds=True)
    sc_u.alloc_factor = 3.0
    cap = (sc_b.capacity + 1023) // 1024 * 1024
    ob = oracle_mod.Oracle(sc_b, phys_capacity=cap)
    ou = oracle_mod.Oracle(sc_u, phys_capacity=cap)
    assert ob.init_particles() == ou.init_particles()
    births = 0
    for _ in range(150):
        sb, su = ob.step(), ou.step()
        births += sb["births"]
        assert sb == su
    assert births > 0
    pb, pu = ob.particles(), ou.particles()
    for k in pb:
        assert np.array_equal(pb[k], pu[k]), k
    assert np.array_equal(ob.C, ou.C)


@pytest.mark.gpu
@pytest.mark.parametrize("f64", [True, False])
def test_gpu_library_matches_builtin_model(f64):
    from bmc.sim import GpuScenario
    from test_gpu_parity import same_bits

    fast = scenarios.monod(f64=f64, mu_max=0.05)
    spec = monod_udf_spec(f64)
    spec.params[:] = fast.params
    sc_b = scenarios.small_ring(20000, f64=f64, model=fast, feeds=True)
    sc_u = scenarios.small_ring(20000, f64=f64, model=spec, feeds=True)
    sc_b.alloc_factor = sc_u.alloc_factor = 3.0
    gb, gu = GpuScenario(sc_b), GpuScenario(sc_u)
    assert gb.weight == gu.weight
    for k in range(4):
        sb, su = gb.run(40), gu.run(40)
        assert sb == su, k
    assert sb["error"] == 0
    pb, pu = gb.particles(), gu.particles()
    for k in ("pos", "status", "id"):
        assert np.array_equal(pb[k], pu[k]), k
    for k in ("state", "age_h", "age_d"):
        assert same_bits(pb[k], pu[k]), k
    lb, lu = gb.liquid(), gu.liquid()
    for k in ("C", "M", "src"):
        assert same_bits(lb[k], lu[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [None, (288, 4, 0)])
def test_gpu_library_model_matches_oracle(oracle_mod, shape):
    """A model that is not built into libbmc (the general contribution
    path): GPU kernels from the library against the oracle driving the
    library's host functions, step by step."""
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

    sc = scenarios.small_ring(16000, f64=False, model=minimal_udf_spec(), feeds=True)
    sc.alloc_factor = 2.0
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    births = 0
    for k in range(40):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        births += gs["births"]
    assert births > 0
    assert_same_particles(g, o, "end")


STOCHASTIC_PARAMS = [2e-8, 2e-6, 1e-3, 0.6e-6, 0.5, 0.01]  # ..., p_div


def stochastic_udf_spec(f64: bool):
    lin = np.float32(1000) * np.float32(np.pi) * np.float32(0.6e-6) ** 2 / np.float32(4)
    phi_max = float(np.float32(2e-8) * lin / np.float32(0.5))
    return udf.udf_model(udf.example("stochastic_udf.cu"), f64, params=STOCHASTIC_PARAMS,
                         value_bound=[4.0 * phi_max])


def test_context_model_host_functions(oracle_mod):
    """A model that draws in update and reads its compartment's
    concentrations: the library exports update_ctx (no update), and the
    oracle drives it with the draws of purpose 3 and the concentrations."""
    spec = stochastic_udf_spec(False)
    hm = udf.host_model(spec.model_id, False)
    assert hm.update_ctx and hm.update_ctx != hm.update
    assert not udf.host_model(monod_udf_spec(False).model_id, False).update_ctx
    sc = scenarios.small_ring(4000, f64=False, model=spec, feeds=True)
    sc.alloc_factor = 2.0
    o1, o2 = oracle_mod.Oracle(sc), oracle_mod.Oracle(sc)
    o1.init_particles()
    o2.init_particles()
    births = 0
    for _ in range(20):
        s1, s2 = o1.step(), o2.step()
        assert s1 == s2
        births += s1["births"]
    assert births > 0  # chance divisions (p_div = 0.01 per step)
    # the draws matter: another seed gives other lengths
    o3 = oracle_mod.Oracle(scenarios.small_ring(4000, f64=False, model=spec, feeds=True, seed=9))
    o3.init_particles()
    o3.step()
    assert not np.array_equal(o3.particles()["state"], o1.particles()["state"][:, : o3.n_used])


@pytest.mark.gpu
@pytest.mark.parametrize("f64", [False, True])
@pytest.mark.parametrize("shape", [None, (256, 2, 0)])
def test_gpu_context_model_matches_oracle(oracle_mod, f64, shape):
    """update_ctx with draws and raw concentrations: GPU kernels from the
    library against the oracle driving the library's host functions."""
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

    sc = scenarios.small_ring(12000, f64=f64, model=stochastic_udf_spec(f64), feeds=True)
    sc.alloc_factor = 2.0
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    births = 0
    for k in range(25):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        births += gs["births"]
    assert births > 0
    assert_same_particles(g, o, "end")
