"""Two-phase flow: gas phase, gas-liquid transfer, clearNegs.

The CPU restatement follows SimulationUnit::ode_step with a gas phase
(apps/libs/simulation/src/simulation.model.cpp L132-L150): transfer from the
old concentrations, gas step with -mtr, liquid step with +mtr, then
clearNegs.  CPU tests check its mass bookkeeping; the GPU tests compare the
device step with it bit for bit.
"""
import numpy as np
import pytest

from bmc import networks, scenarios


def two_phase(n_particles=8000, f64=True, feeds=True):
    sc = scenarios.workload(2, n_particles=n_particles, f64=f64)
    net = networks.lattice_vortex(3, side=0.2, peak_velocity=0.5, noise=0.1, seed=3, max_courant=0.4, dt=0.1)
    sc.net = net
    sc.c0 = sc.c0[: net.n_c]
    sc.dt = 0.1
    sc.feeds[0].outlet = net.n_c - 1
    sc.feeds[0].flow = 1e-4
    sc = scenarios.with_gas(sc, kla=0.05, henry=0.03)
    if not feeds:
        sc.feeds = []
        sc.gas.feeds = []
    return sc


def test_transfer_moves_mass_between_phases_only(oracle_mod):
    """Closed reactor, no particles: liquid + gas mass of every species is
    conserved up to rounding while O2 dissolves."""
    sc = two_phase(n_particles=1024, feeds=False)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    o.s.n_used = 0  # no cell: only transport and transfer
    total0 = o.M.sum(axis=0) + o.Mg.sum(axis=0)
    c_o2 = o.C[:, 1].mean()
    for _ in range(50):
        o.step()
    total1 = o.M.sum(axis=0) + o.Mg.sum(axis=0)
    assert np.allclose(total0, total1, rtol=1e-12, atol=1e-15)
    assert o.C[:, 1].mean() > c_o2  # liquid O2 rises towards H * Cg
    assert np.all(o.mtr[:, [0, 2, 3]] == 0.0)  # only the transferred species moves


def test_transfer_formula(oracle_mod):
    sc = two_phase(n_particles=1024, feeds=False)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    o.s.n_used = 0
    C0, Cg0 = o.C.copy(), o.Cg.copy()
    o.step()
    expect = (sc.gas.kla * (Cg0 * sc.gas.henry[None, :] - C0)) * sc.net.volume[:, None]
    assert np.array_equal(o.mtr, expect)


@pytest.mark.gpu
@pytest.mark.parametrize("f64", [True, False])
def test_gpu_two_phase_matches_oracle(oracle_mod, f64):
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair, same_bits

    sc = two_phase(n_particles=20000, f64=f64)
    g, o = make_pair(oracle_mod, sc)
    for k in range(12):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        gg = g.gas()
        for key, ref in (("Cg", o.Cg), ("Mg", o.Mg), ("mtr", o.mtr)):
            assert same_bits(gg[key], ref), f"step {k}: {key}"
    assert_same_particles(g, o, "end")
    # graph-replayed steps agree too
    g.run(10)
    o.run(10)
    assert_same_liquid(g, o, "run")
    assert same_bits(g.gas()["Cg"], o.Cg)
