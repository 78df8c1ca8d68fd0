"""Flow-map cycle: several flow-map states of one mesh replayed in turn.

The reference's transitioner (rcmtool, not in the source tree) advances the
flow map every n_per_flowmap steps and the main loop swaps volumes,
neighbours, out-flows, probabilities and the liquid transition
(apps/core/src/host_specific.cpp L255-L266).  The CPU restatement switches
its domain arrays at the same steps; the GPU switches on the device inside
the captured step.  Parity unpinned against the reference at this boundary
(no transitioner source); GPU against the restatement bit for bit.
"""
import dataclasses

import numpy as np
import pytest

from bmc import networks, scenarios


def maps(n_maps=3, n=4, seed=7):
    out = []
    rng = np.random.default_rng(seed)
    for k in range(n_maps):
        net = networks.lattice_vortex(n, side=0.2, peak_velocity=0.5, noise=0.1, seed=seed + k,
                                      max_courant=0.4, dt=0.1)
        net.volume = net.volume * rng.uniform(0.8, 1.2, size=net.n_c)
        out.append(net)
    assert len({m.K for m in out}) == 1
    return out


def flowmap_scenario(n_particles=20000, t_per=0.35, n_maps=3, f64=True):
    fm = maps(n_maps)
    sc = scenarios.workload(2, n_particles=n_particles, f64=f64)
    sc.net = fm[0]
    sc.c0 = sc.c0[: fm[0].n_c]
    sc.feeds[0].outlet = fm[0].n_c - 1
    sc.feeds[0].flow = 2e-4
    sc.dt = 0.1
    sc.flowmaps = fm
    sc.t_per_flowmap = t_per
    return sc


def test_steps_per_flowmap_formula():
    sc = flowmap_scenario()
    assert sc.n_per_flowmap == int(0.35 / 0.1) + 1 == 4
    assert dataclasses.replace(sc, t_per_flowmap=0.0).n_per_flowmap == 1
    assert dataclasses.replace(sc, flowmaps=sc.flowmaps[:1]).n_per_flowmap == 1


def test_identical_maps_equal_fixed_domain(oracle_mod):
    """A cycle of copies of one map is the fixed-domain run, bit for bit."""
    sc = flowmap_scenario(n_particles=5000)
    same = dataclasses.replace(sc, flowmaps=[sc.net, sc.net, sc.net])
    fixed = dataclasses.replace(sc, flowmaps=[])
    a, b = oracle_mod.Oracle(same), oracle_mod.Oracle(fixed)
    assert a.init_particles() == b.init_particles()
    for _ in range(13):
        assert a.step() == b.step()
    pa, pb = a.particles(), b.particles()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(a.C, b.C)


def test_map_cycle_changes_the_run(oracle_mod):
    sc = flowmap_scenario(n_particles=5000)
    a = oracle_mod.Oracle(sc)
    b = oracle_mod.Oracle(dataclasses.replace(sc, flowmaps=[]))
    a.init_particles()
    b.init_particles()
    for _ in range(9):
        a.step()
        b.step()
    assert a._map_cur == (9 - 1) // 4 % 3
    assert not np.array_equal(a.particles()["pos"], b.particles()["pos"])


@pytest.mark.gpu
def test_gpu_flowmap_cycle_matches_oracle(oracle_mod):
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

    sc = flowmap_scenario()
    g, o = make_pair(oracle_mod, sc)
    for k in range(14):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
    assert_same_particles(g, o, "end")


@pytest.mark.gpu
def test_gpu_flowmap_graph_run_and_batch_equal_steps(oracle_mod):
    from bmc.sim import GpuBatch, GpuScenario
    from test_gpu_parity import assert_same_liquid, assert_same_particles

    sc = flowmap_scenario()
    g = GpuScenario(sc)
    g.run(14)  # one captured graph per step, replayed
    o = oracle_mod.Oracle(sc, phys_capacity=g.cap)
    o.init_particles()
    o.set_weight(g.weight)
    o.run(14)
    assert_same_particles(g, o, "graph run")
    assert_same_liquid(g, o, "graph run")
    # in a batch with a fixed-domain scenario of the same model
    other = dataclasses.replace(sc, flowmaps=[], seed=99, n_particles=3000)
    m1, m2 = GpuScenario(sc), GpuScenario(other)
    b = GpuBatch([m1, m2])
    b.run(14, sc.dt)
    b.synchronize()
    assert_same_particles(m1, o, "batched")
    assert_same_liquid(m1, o, "batched")
    b.close()


@pytest.mark.gpu
def test_gpu_domain_calls_refused_while_cycling():
    from bmc import _lib
    from bmc.sim import GpuScenario

    sc = flowmap_scenario(n_particles=2000)
    g = GpuScenario(sc)
    net = sc.net
    vol = np.ascontiguousarray(net.volume, dtype=np.float64)
    nbr = np.ascontiguousarray(net.neighbors, dtype=np.uint64)
    outf = np.ascontiguousarray(net.out_flow, dtype=np.float64)
    cdf = np.ascontiguousarray(net.cdf, dtype=np.float64)
    with pytest.raises(_lib.BmcError, match="flow-map"):
        _lib.call("bmc_domain_update", g.handle, net.n_c, net.K, vol.ctypes.data, nbr.ctypes.data,
                  outf.ctypes.data, cdf.ctypes.data)
    _lib.call("bmc_flowmap_clear", g.handle)
    _lib.call("bmc_domain_update", g.handle, net.n_c, net.K, vol.ctypes.data, nbr.ctypes.data,
              outf.ctypes.data, cdf.ctypes.data)


def gas_flowmap_scenario(n_particles=20000, seed=3):
    """The flow-map scenario with a gas phase whose state changes with the
    maps: per map, a gas ring on 10 % of that map's liquid volumes (varied)
    and the turbulence kla of a dissipation field of its own."""
    from bmc import cma
    from bmc.networks import Network

    sc = scenarios.with_gas(flowmap_scenario(n_particles=n_particles), kla=0.05, henry=3.181e-2)
    rng = np.random.default_rng(seed)
    gmaps, klas = [], []
    for net in sc.flowmaps:
        vol = net.volume * 0.1 * rng.uniform(0.8, 1.2, size=net.n_c)
        src = np.arange(net.n_c)
        q = 0.2 * float(np.min(vol)) / sc.dt
        gmaps.append(Network(net.n_c, vol, src, (src + 1) % net.n_c, q * rng.uniform(0.8, 1.2, size=net.n_c)).finalize())
        kla = np.zeros((net.n_c, sc.n_species))
        kla[:, 1] = cma.turbulence_kla(rng.lognormal(-1.0, 0.5, net.n_c), net.volume, vol)
        klas.append(kla)
    sc.gas.flowmaps = gmaps
    sc.gas.kla_maps = klas
    return sc


def test_identical_gas_states_equal_a_fixed_gas_domain(oracle_mod):
    """Maps whose gas states all equal the gas phase's domain run as the fixed
    gas domain, bit for bit."""
    sc = gas_flowmap_scenario(n_particles=5000)
    same = dataclasses.replace(sc, gas=dataclasses.replace(sc.gas, flowmaps=[sc.gas.net] * 3, kla_maps=[]))
    fixed = dataclasses.replace(sc, gas=dataclasses.replace(sc.gas, flowmaps=[], kla_maps=[]))
    a, b = oracle_mod.Oracle(same), oracle_mod.Oracle(fixed)
    a.init_particles()
    b.init_particles()
    for _ in range(13):
        assert a.step() == b.step()
    assert np.array_equal(a.Cg, b.Cg) and np.array_equal(a.C, b.C)


def test_gas_states_switch_with_the_maps(oracle_mod):
    """A switch replaces the gas volumes and keeps the gas masses; the run
    then departs from the fixed gas domain."""
    sc = gas_flowmap_scenario(n_particles=5000)
    a = oracle_mod.Oracle(sc)
    b = oracle_mod.Oracle(dataclasses.replace(sc, gas=dataclasses.replace(sc.gas, flowmaps=[], kla_maps=[])))
    a.init_particles()
    b.init_particles()
    for _ in range(9):
        a.step()
        b.step()
    assert a._map_cur == (9 - 1) // 4 % 3
    assert not np.array_equal(a.Cg, b.Cg)
    # the masses the switch keeps: Cg follows them through the new volumes
    # at the next step, never jumps at the switch itself
    assert np.all(np.isfinite(a.Cg)) and np.all(a.Mg >= 0)


@pytest.mark.gpu
def test_gpu_gas_flowmaps_match_oracle(oracle_mod):
    """Two-phase run whose gas domain and kla switch with the flow maps:
    device and restatement step for step, and in captured graph runs."""
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair, same_bits

    sc = gas_flowmap_scenario()
    g, o = make_pair(oracle_mod, sc)
    for k in range(14):
        assert_same_stats(g.step(), o.step(), f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        gg = g.gas()
        for key, ref in (("Cg", o.Cg), ("Mg", o.Mg), ("mtr", o.mtr)):
            assert same_bits(gg[key], ref), f"step {k}: {key}"
    assert_same_particles(g, o, "steps")
    g.run(10)
    o.run(10)
    assert_same_liquid(g, o, "graph run")
    assert same_bits(g.gas()["Cg"], o.Cg)
