"""The C-ABI from C++: the BmcBackend binding a maintainer adds to the
reference's simulation core, compiled as a program against include/bmc.h and linked to libbmc.so
(tests/cpp/backend_demo.cpp).  On the CPU it must compile and link; on the
GPU it runs a scenario through bmc_step_read every iteration and its
counters, fields and final particles must equal the Python binding's run of
the same scenario bit for bit; its pipelined loop (bmc_step_enqueue /
bmc_step_collect) must write the same bytes."""
import os
import struct
import subprocess

import numpy as np
import pytest

from bmc import scenarios
from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "backend_demo.cpp")


def build_demo(tmp_path) -> str:
    from bmc import _lib

    lib = _lib.lib_path()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "backend_demo")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", libdir, "-lbmc", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def test_binding_compiles_and_links(tmp_path):
    exe = build_demo(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def write_input(path, sc, n_steps):
    from bmc.sim import scenario_desc, transition_coo

    net = sc.net
    d = scenario_desc(sc)
    rows, cols, vals = transition_coo(net)
    with open(path, "wb") as f:
        f.write(bytes(d))
        f.write(struct.pack("<IIIQdddIIQ", net.n_c, net.K, sc.n_species, sc.n_particles, sc.x0, sc.dt,
                            sc.alloc_factor, n_steps, len(sc.feeds), len(vals)))
        for a, t in ((net.volume, np.float64), (net.neighbors, np.uint64), (net.out_flow, np.float64),
                     (net.cdf, np.float64), (rows, np.uint64), (cols, np.uint64), (vals, np.float64),
                     (sc.c0, np.float64)):
            f.write(np.ascontiguousarray(a, dtype=t).tobytes())
        from bmc import _lib

        for fd in sc.feeds:
            x = _lib.Feed()
            x.inlet, x.outlet, x.flow = fd.inlet, fd.outlet, fd.flow
            for sp in range(len(fd.conc)):
                x.conc[sp] = float(fd.conc[sp])
            f.write(bytes(x))


@pytest.mark.gpu
def test_cpp_binding_equals_python_binding(tmp_path):
    from bmc.sim import GpuScenario

    sc = scenarios.workload(2, n_particles=200_000)
    n_steps = 12
    exe = build_demo(tmp_path)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, sc, n_steps)
    subprocess.run([exe, inp, outp], check=True)
    raw = open(outp, "rb").read()
    off = 0
    (w,) = struct.unpack_from("<d", raw, off)
    off += 8
    g = GpuScenario(sc)
    assert w == g.weight
    ne = sc.net.n_c * sc.n_species
    conc = np.zeros((sc.net.n_c, sc.n_species))
    for k in range(n_steps):
        row = np.frombuffer(raw, np.uint64, 6, off)
        off += 48
        c_cpp = np.frombuffer(raw, np.float64, ne, off)
        off += ne * 8
        st = g.step_read(conc)
        assert list(row) == [st["n_used"], st["births"], st["exits"], st["moves"], st["overflow"], st["error"]], k
        assert np.array_equal(c_cpp.view(np.uint64), conc.ravel().view(np.uint64)), k
    (n,) = struct.unpack_from("<Q", raw, off)
    off += 8
    p = g.particles()
    assert n == len(p["pos"])
    nv = sc.model.n_var
    st_cpp = np.frombuffer(raw, np.float64, nv * n, off).reshape(nv, n)
    off += nv * n * 8
    assert np.array_equal(st_cpp.view(np.uint64), p["state"].view(np.uint64))
    assert np.array_equal(np.frombuffer(raw, np.uint32, n, off), p["pos"])
    off += 4 * n
    assert np.array_equal(np.frombuffer(raw, np.uint8, n, off), p["status"])
    off += n
    assert np.array_equal(np.frombuffer(raw, np.uint32, n, off), p["id"])
    off += 4 * n
    ev = np.frombuffer(raw, np.uint64, 6, off)
    off += 48
    assert list(ev) == list(g.events().values())
    assert np.array_equal(np.frombuffer(raw, np.float64, n, off).view(np.uint64), g.mass().view(np.uint64))
    g.close()


@pytest.mark.gpu
def test_cpp_pipelined_loop_equals_step_read_loop(tmp_path):
    """The same program with bmc_step_enqueue / bmc_step_collect (two steps
    in flight, feeds set before every enqueue) writes the same bytes as with
    bmc_step_read every iteration."""
    sc = scenarios.workload(2, n_particles=200_000)
    exe = build_demo(tmp_path)
    inp = str(tmp_path / "in.bin")
    write_input(inp, sc, 12)
    a, b = str(tmp_path / "a.bin"), str(tmp_path / "b.bin")
    subprocess.run([exe, inp, a], check=True)
    subprocess.run([exe, inp, b, "pipelined"], check=True)
    assert open(a, "rb").read() == open(b, "rb").read()
