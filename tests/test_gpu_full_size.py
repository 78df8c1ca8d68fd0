"""GPU path against the CPU restatement at the benchmark's full sizes.

The CPU restatement steps 1e7 particles in a few tens of milliseconds on the
host's cores, so the benchmark workloads are compared bit for bit at the
sizes they are measured at, not only at reduced particle counts:

* the 8^3 toroidal-vortex lattice, FP64 Monod + overflow, 1e7 particles
  (the default benchmark): 200 steps, the first 10 one at a time with the
  counters and the liquid compared after each, then two captured graph runs
  of 95 steps; the whole particle container after step 10 and at the end;
* the 16^3 lattice in FP32, 5e7 particles: 30 steps, counters and liquid
  after each, the container after step 10 and at the end;
* the batched form's 256 uneven scenarios (1.9e8 particles in total,
  FP32 Monod) advanced together by one batched launch sequence per step
  for 4 steps, every scenario then compared with the restatement run alone.

State, ages and concentrations are compared bitwise, counts exactly.
"""
import os

import numpy as np
import pytest

from bmc import scenarios

from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair, same_bits

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def test_lattice512_overflow_fp64_full_size(oracle_mod):
    sc = scenarios.workload(2)
    assert sc.n_particles == 10_000_000 and sc.net.n_c == 512 and sc.model.f64
    g, o = make_pair(oracle_mod, sc)
    g.set_shape(544, 2, 0)
    births = exits = 0
    for k in range(10):
        gs, os_ = g.step(), o.step(THREADS)
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        exits += gs["exits"]
    assert_same_particles(g, o, "step 10")
    done = 10
    for n in (95, 95):
        gs = g.run(n)
        o.run(n, THREADS)
        done += n
        os_ = o.stats()
        assert gs["step"] == done and gs["error"] == 0
        assert gs["n_used"] == o.n_used, f"run to {done}"
        assert gs["inactive"] == os_["inactive"], f"run to {done}"
        assert_same_liquid(g, o, f"run to {done}")
    assert_same_particles(g, o, f"step {done}")
    assert exits > 0  # particles leave through the outlet at compartment 511
    g.close()


def test_lattice4096_overflow_fp32_full_size(oracle_mod):
    sc = scenarios.workload(3)
    assert sc.n_particles == 50_000_000 and sc.net.n_c == 4096 and not sc.model.f64
    g, o = make_pair(oracle_mod, sc)
    g.set_shape(544, 2, 0)
    moves = 0
    for k in range(30):
        gs, os_ = g.step(), o.step(THREADS)
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        moves += gs["moves"]
        if k == 9:
            assert_same_particles(g, o, "step 10")
    assert moves > 0
    assert_same_particles(g, o, "step 30")
    g.close()


def test_batched_form_full_size(oracle_mod):
    from bmc.sim import GpuBatch, GpuScenario

    scens = [scenarios.batch_scenario(k, seed=1234) for k in range(256)]
    total = sum(s.n_particles for s in scens)
    assert 1.5e8 < total < 2.5e8
    members = [GpuScenario(s) for s in scens]
    b = GpuBatch(members)
    b.set_shape(544, 2, 0)
    steps = 4
    b.run(steps, 0.1)
    b.synchronize()
    b.close()
    for k, (sc, g) in enumerate(zip(scens, members)):
        where = f"scenario {k} ({sc.net.n_c} compartments, {sc.n_particles} particles)"
        o = oracle_mod.Oracle(sc, phys_capacity=g.cap)
        o.init_particles()
        o.set_weight(g.weight)
        o.run(steps, THREADS)
        gs, os_ = g.stats(), o.stats()
        assert gs["step"] == steps and gs["error"] == 0, where
        for key in ("n_used", "inactive"):
            assert gs[key] == os_[key], f"{where}: {key}"
        assert_same_particles(g, o, where)
        lq = g.liquid()
        for key, ref in (("C", o.C), ("M", o.M), ("src", o.src)):
            assert same_bits(lq[key], ref), f"{where}: {key}"
        g.close()
        del o
