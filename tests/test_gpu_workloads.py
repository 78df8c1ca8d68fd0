"""GPU path against the CPU restatement on the benchmark's own networks.

Each benchmark workload is stepped with its own generator, seed, model,
precision, feeds and time step, and compared bit for bit with the oracle:

* the 10-compartment ring with two random links per compartment (seed 42),
  1e5 particles, FP64 Monod, dt 0.1 s, closed reactor, all 1000 steps:
  step by step for the first 200 (statistics and liquid every step), then
  in captured graph runs of 200 steps;
* the 8^3 toroidal-vortex lattice (512 compartments, four species, FP64
  Monod + overflow, glucose inlet at 0, outlet at 511, dt 0.05 s) at 1e6
  particles for 10 steps, in the launch shape the benchmark uses;
* the 16^3 lattice (4096 compartments) in FP32 at 2e6 particles for 5 steps.

Every floating value is compared bitwise (state, ages, concentrations,
masses, sources); integers exactly.  Particle counts are reduced from the
benchmark's (1e7, 5e7) so the single oracle finishes in seconds; the
networks, models and parameters are the benchmark's.
"""
import os

import numpy as np
import pytest

from bmc import scenarios

from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def test_ring10_monod_fp64_as_configured(oracle_mod):
    sc = scenarios.workload(1)
    assert sc.n_particles == 100_000 and sc.n_steps == 1000 and sc.net.n_c == 10 and sc.seed == 42
    assert not sc.feeds and sc.model.f64
    g, o = make_pair(oracle_mod, sc)
    for k in range(200):
        gs, os_ = g.step(), o.step(THREADS)
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        if k % 50 == 49:
            assert_same_particles(g, o, f"step {k}")
    done = 200
    while done < sc.n_steps:
        gs = g.run(200)
        o.run(200, THREADS)
        done += 200
        assert gs["step"] == done and gs["error"] == 0
        assert gs["n_used"] == o.n_used
        assert_same_liquid(g, o, f"run to {done}")
        assert_same_particles(g, o, f"run to {done}")


def test_lattice512_overflow_fp64_own_network(oracle_mod):
    sc = scenarios.workload(2, n_particles=1_000_000)
    assert sc.net.n_c == 512 and sc.model.f64 and sc.feeds[0].outlet == 511
    g, o = make_pair(oracle_mod, sc)
    moves = 0
    for k in range(10):
        gs, os_ = g.step(), o.step(THREADS)
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        moves += gs["moves"]
    assert moves > 0
    assert_same_particles(g, o, "end")


def test_lattice4096_overflow_fp32_own_network(oracle_mod):
    sc = scenarios.workload(3, n_particles=2_000_000)
    assert sc.net.n_c == 4096 and not sc.model.f64
    g, o = make_pair(oracle_mod, sc)
    for k in range(5):
        gs, os_ = g.step(), o.step(THREADS)
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
    assert_same_particles(g, o, "end")
