"""Time-varying feeds (the reference's FeedDescriptor Linear and Exponential
variants, apps/libs/simulation/src/feed_descriptor.cpp L12-L36, applied by
SimulationUnit::update_feed, simulation.model.cpp L73-L111).

The flows are evaluated on the device at the scenario's relative time every
main-loop step: the inlet sources, the outlet sink and the outlet's leaving
flow with its exit threshold.  GPU results are compared bit for bit with the
CPU restatement step by step, through captured graph runs and in a batch.
"""
import dataclasses

import numpy as np
import pytest

from bmc import scenarios

from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair


def scheduled(n=8000, kind=scenarios.FEED_LINEAR, seed=3):
    """Ring of 10 with a linear feed through inlet 0 / outlet 9 whose flow
    grows ninefold over 40 steps, and an inlet-only exponential feed."""
    sc = scenarios.small_ring(n, feeds=True, seed=seed)
    fd = sc.feeds[0]
    fd.kind, fd.f0, fd.rate = kind, 1e-5, 2e-5
    if kind == scenarios.FEED_EXPONENTIAL:
        fd.f0, fd.rate = -0.99999, 1e-4  # f0 + exp(1e-4 t): 1e-5 at t = 0, then growing
    conc = np.zeros(sc.n_species)
    conc[0] = 1e-4
    sc.feeds.append(scenarios.Feed(3, -1, 0.0, conc, kind=scenarios.FEED_EXPONENTIAL, f0=0.0, rate=-2.0))
    return sc


def test_oracle_linear_feed_grows_the_outflow(oracle_mod):
    sc = scheduled()
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    exits = 0
    for k in range(40):
        st = o.step(2)
        exits += st["exits"]
        assert o.s.feed_flow[0] == pytest.approx(1e-5 + 2e-5 * (0.1 * k), rel=1e-12)
    assert exits > 0
    assert o.s.t_rel == pytest.approx(4.0, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [scenarios.FEED_LINEAR, scenarios.FEED_EXPONENTIAL])
def test_scheduled_feeds_step_by_step(oracle_mod, kind):
    sc = scheduled(kind=kind)
    g, o = make_pair(oracle_mod, sc)
    exits = 0
    for k in range(40):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        exits += gs["exits"]
    assert exits > 0
    assert_same_particles(g, o, "end")
    assert g.feed_time() == o.s.t_rel


@pytest.mark.gpu
def test_scheduled_feeds_in_graph_runs_and_cycles(oracle_mod):
    """bmc_run replays a captured step graph: the flows still follow the
    relative time; a cycle alone (bmc_cycle) leaves the time where it is."""
    sc = scheduled()
    g, o = make_pair(oracle_mod, sc)
    g.run(25)
    o.run(25)
    assert_same_liquid(g, o, "run 25")
    assert_same_particles(g, o, "run 25")
    t = g.feed_time()
    assert t == o.s.t_rel
    g.cycle()
    assert g.feed_time() == t
    g.close()


@pytest.mark.gpu
def test_scheduled_feeds_in_a_batch(oracle_mod):
    from bmc.sim import GpuBatch, GpuScenario

    scs = [scheduled(6000, seed=s) for s in (3, 4, 5)]
    scs[1] = dataclasses.replace(scs[1], feeds=[dataclasses.replace(f) for f in scs[1].feeds])
    scs[1].feeds[0].rate = 5e-5
    gs = [GpuScenario(s) for s in scs]
    os_ = []
    for g, s in zip(gs, scs):
        o = oracle_mod.Oracle(s, phys_capacity=g.cap)
        o.init_particles()
        o.set_weight(g.weight)
        os_.append(o)
    b = GpuBatch(gs)
    b.run(20, 0.1)
    b.synchronize()
    for g, o in zip(gs, os_):
        o.run(20)
        assert_same_liquid(g, o, "batch")
        assert_same_particles(g, o, "batch")
    b.close()


@pytest.mark.gpu
def test_schedules_follow_the_feeds():
    """One schedule per feed, in the feeds' order; bad kinds are refused."""
    from bmc import _lib
    from bmc.sim import GpuScenario

    g = GpuScenario(scheduled())
    one = (_lib.FeedSchedule * 1)()
    with pytest.raises(_lib.BmcError):
        _lib.call("bmc_set_feed_schedules", g.handle, 1, one)
    two = (_lib.FeedSchedule * 2)()
    two[0].kind = 7
    with pytest.raises(_lib.BmcError):
        _lib.call("bmc_set_feed_schedules", g.handle, 2, two)
    g.close()
