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


def test_turbulence_kla_as_the_reference_correlation():
    """FlowmapTurbulence (impl_mtr.cpp L100-L145), evaluated independently:
    water at 20 C (1.0023e-6 m^2/s after the reference's rounding), oxygen
    diffusivity 1e-9 m^2/s, bubbles of 5 mm."""
    from bmc import cma

    rng = np.random.default_rng(4)
    eps = rng.uniform(0.0, 2.0, 50)
    vl = rng.uniform(0.5e-3, 2e-3, 50)
    vg = vl * rng.uniform(0.0, 0.3, 50)
    got = cma.turbulence_kla(eps, vl, vg)
    nu = 1.0023e-6
    alpha = vg / (vl + vg)
    want = 0.3 * (eps * nu) ** 0.25 * (nu / 1e-9) ** -0.5 * (6.0 * alpha / (5e-3 * (1 - alpha)))
    assert np.allclose(got, want, rtol=1e-14, atol=0.0)
    assert got[vg == 0.0].size == 0 or np.all(got[vg == 0.0] == 0.0)
    # no gas, no interface; no turbulence, no transfer
    assert cma.turbulence_kla(np.ones(1), np.ones(1), np.zeros(1))[0] == 0.0
    assert cma.turbulence_kla(np.zeros(1), np.ones(1), np.ones(1))[0] == 0.0


@pytest.mark.parametrize("bad", [dict(vl=0.0), dict(vg=-1.0), dict(eps=-1.0), dict(db=0.0)])
def test_turbulence_kla_refuses_bad_inputs(bad):
    from bmc import _lib, cma

    args = dict(eps=1.0, vl=1e-3, vg=1e-4, db=5e-3)
    args.update(bad)
    with pytest.raises(_lib.BmcError):
        cma.turbulence_kla(np.array([args["eps"]]), np.array([args["vl"]]), np.array([args["vg"]]), args["db"])


@pytest.mark.gpu
def test_gpu_two_phase_with_turbulence_kla_matches_oracle(oracle_mod):
    """The O2 transfer of a two-phase lattice with kla from a turbulence
    field (FlowmapTurbulence): device and restatement step for step."""
    from bmc import cma
    from test_gpu_parity import assert_same_liquid, assert_same_stats, make_pair, same_bits

    sc = two_phase(n_particles=20000)
    eps = np.random.default_rng(8).lognormal(-1.0, 0.7, sc.net.n_c)
    kla = cma.turbulence_kla(eps, sc.net.volume, sc.gas.net.volume)
    sc.gas.kla[:, 1] = kla
    sc.gas.henry[:] = 0.0
    sc.gas.henry[1] = 3.181e-2
    g, o = make_pair(oracle_mod, sc)
    for k in range(8):
        assert_same_stats(g.step(), o.step(), f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        gg = g.gas()
        for key, ref in (("Cg", o.Cg), ("mtr", o.mtr)):
            assert same_bits(gg[key], ref), f"step {k}: {key}"
    assert np.any(g.gas()["mtr"][:, 1] != 0.0)
