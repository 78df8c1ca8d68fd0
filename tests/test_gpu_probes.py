"""Time-event probes and event tallies on the GPU against the CPU
restatement.

Division times are stored in slot order within a step on both sides, so
they are compared value for value; leaving times are stored in the order
the device's threads reach the exit (as the reference's atomic counter
orders them), so they are compared as sorted lists while the buffer has
room, and as a sub-multiset of the restatement's once it is full.  Event
counts are always equal."""
import numpy as np
import pytest

from bmc import scenarios

from test_gpu_parity import assert_same_particles, assert_same_stats, make_pair

pytestmark = pytest.mark.gpu

LEAVING, DIVISION = 0, 1


def _scenario():
    # every particle asks to divide, the container fills (refused requests),
    # a strong outlet: exits and compactions every few steps
    sc = scenarios.zero_d(3000, model=scenarios.monod(f64=True, m_div=1.0), outlet=True)
    sc.feeds[0].flow = 1e-3
    return sc


def _same_probes(g, o, where, full=False):
    gd, nd = g.probe_read(DIVISION)
    od, n2 = o.probe_read(DIVISION)
    assert nd == n2, f"{where}: division count"
    assert np.array_equal(gd.view(np.uint64), od.view(np.uint64)), f"{where}: division times"
    gl, nl = g.probe_read(LEAVING)
    ol, n3 = o.probe_read(LEAVING)
    assert nl == n3, f"{where}: leaving count"
    if not full:
        assert np.array_equal(np.sort(gl).view(np.uint64), np.sort(ol).view(np.uint64)), f"{where}: leaving times"
    return nd, nl


def test_probes_match_the_restatement(oracle_mod):
    g, o = make_pair(oracle_mod, _scenario(), capacity=4096)
    g.probe_enable(1 << 18)
    o.probe_enable(1 << 18)
    for k in range(8):
        assert_same_stats(g.step(), o.step(), f"step {k}")
        _same_probes(g, o, f"step {k}")
    # in captured graph runs too
    g.run(12)
    o.run(12)
    nd, nl = _same_probes(g, o, "graph run")
    assert nd > 1000 and nl > 100
    assert_same_particles(g, o, "end")


def test_full_buffers_count_on_and_clear(oracle_mod):
    cap = 64
    g, o = make_pair(oracle_mod, _scenario(), capacity=4096)
    g.probe_enable(cap)
    o.probe_enable(cap)
    big = oracle_mod.Oracle(_scenario(), phys_capacity=g.cap)  # every leaving time
    big.init_particles()
    big.set_weight(g.weight)
    big.probe_enable(1 << 18)
    for k in range(6):
        g.step()
        o.step()
        big.step()
    nd, nl = _same_probes(g, o, "full", full=True)
    assert nd > cap and nl > cap
    gl, _ = g.probe_read(LEAVING)
    assert len(gl) == cap
    everything = list(np.sort(big.probe_read(LEAVING)[0]))
    for v in gl:  # each kept leaving time is one of the step's events
        everything.remove(v)
    g.probe_clear(DIVISION)
    g.probe_clear(LEAVING)
    o.probe_clear(DIVISION)
    o.probe_clear(LEAVING)
    assert g.probe_read(DIVISION)[1] == 0 and g.probe_read(LEAVING)[1] == 0
    for k in range(2):
        g.step()
        o.step()
    _same_probes(g, o, "after clear", full=True)


def test_probes_in_a_batch_equal_alone():
    from bmc.sim import GpuBatch, GpuScenario

    scens = [_scenario(), scenarios.small_ring(20000, model=scenarios.monod(f64=True, m_div=1.05), feeds=True)]
    members = [GpuScenario(s, capacity=32768) for s in scens]
    alone = [GpuScenario(s, capacity=32768) for s in scens]
    for g in members + alone:
        g.probe_enable(1 << 16)
    b = GpuBatch(members)
    b.run(6, 0.1)
    b.synchronize()
    for g in alone:
        g.run(6, 0.1)
    for k, (gb, ga) in enumerate(zip(members, alone)):
        db, nb = gb.probe_read(DIVISION)
        da, na = ga.probe_read(DIVISION)
        assert nb == na and np.array_equal(db, da), f"member {k}: division times"
        lb, mb = gb.probe_read(LEAVING)
        la, ma = ga.probe_read(LEAVING)
        assert mb == ma and np.array_equal(np.sort(lb), np.sort(la)), f"member {k}: leaving times"
    assert members[0].probe_read(DIVISION)[1] > 0 and members[1].probe_read(LEAVING)[1] > 0
    b.close()


def test_probes_are_off_by_default():
    from bmc.sim import GpuScenario

    g = GpuScenario(_scenario(), capacity=4096)
    g.run(4)
    for p in (LEAVING, DIVISION):
        values, n = g.probe_read(p)
        assert n == 0 and len(values) == 0


def _oracle_events(o, steps):
    ev = dict.fromkeys(("NewParticle", "Exit", "Move", "Death", "Overflow", "ChangeWeight"), 0)
    for _ in range(steps):
        st = o.step()
        ev["NewParticle"] += int(o.s.requested_divisions)
        ev["Exit"] += st["exits"]
        ev["Move"] += st["moves"]
        ev["Overflow"] += st["overflow"]
    return ev


def test_event_tallies_accumulate_over_graph_runs(oracle_mod):
    """MC::EventContainer: counts summed over every step since the last
    clear, in captured graph runs too; a division request is a NewParticle
    event whether or not it found room."""
    sc = scenarios.small_ring(8000, model=scenarios.monod(f64=True, m_div=1.0), feeds=True)
    g, o = make_pair(oracle_mod, sc, capacity=9216)  # room for a quarter of the first requests
    g.run(7)
    want = _oracle_events(o, 7)
    got = g.events(clear=True)
    assert got == want
    assert want["Overflow"] > 0 and want["Move"] > 0 and want["Exit"] > 0
    assert g.events() == dict.fromkeys(want, 0)
    g.step()
    g.run(4)
    assert g.events() == _oracle_events(o, 5)


def test_event_tallies_in_a_batch_equal_alone():
    from bmc.sim import GpuBatch, GpuScenario

    scens = [_scenario(), scenarios.small_ring(20000, model=scenarios.monod(f64=True, m_div=1.05), feeds=True)]
    members = [GpuScenario(s, capacity=32768) for s in scens]
    alone = [GpuScenario(s, capacity=32768) for s in scens]
    b = GpuBatch(members)
    b.run(5, 0.1)
    b.synchronize()
    for g in alone:
        g.run(5, 0.1)
    for gb, ga in zip(members, alone):
        assert gb.events() == ga.events()
        assert gb.events()["NewParticle"] > 0
    b.close()
