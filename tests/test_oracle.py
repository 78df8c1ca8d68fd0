"""Invariants of the CPU restatement (test infrastructure checks itself)."""
import numpy as np
import pytest

from bmc import scenarios


def test_particle_conservation_and_ids(oracle_mod):
    sc = scenarios.small_ring(3000, feeds=True, n_steps=30)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    total_exits = 0
    for _ in range(30):
        st = o.step()
        total_exits += st["exits"]
    p = o.particles()
    live = int((p["status"] == 0).sum())
    assert live == 3000 - total_exits + (o.s.next_id - 3000)
    assert len(np.unique(p["id"])) == o.n_used


def test_compaction_gap_filling_keeps_multiset(oracle_mod):
    sc = scenarios.small_ring(2048, n_steps=1)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    rng = np.random.default_rng(0)
    dead = rng.choice(2048, size=300, replace=False)
    before = o.particles()
    o.status[dead] = 2
    keep_ids = set(before["id"][np.setdiff1d(np.arange(2048), dead)].tolist())
    import ctypes as ct

    oracle_mod.lib().orc_remove_inactive(ct.byref(o.s), 300)
    after = o.particles()
    assert o.n_used == 2048 - 300
    assert set(after["id"].tolist()) == keep_ids
    assert (after["status"] == 0).all()
    # gap filling moves only the tail: untouched head slots keep their ids
    head = np.setdiff1d(np.arange(2048 - 300), dead)
    assert np.array_equal(after["id"][head], before["id"][head])


def test_threads_do_not_change_results(oracle_mod):
    sc = scenarios.workload(2, n_particles=20000, n_steps=5)
    a = oracle_mod.Oracle(sc)
    a.init_particles()
    b = oracle_mod.Oracle(sc)
    b.init_particles()
    for _ in range(5):
        a.step(1)
        b.step(4)
    pa, pb = a.particles(), b.particles()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(a.C, b.C)
    assert np.array_equal(a.src, b.src)


def test_births_and_overflow(oracle_mod):
    m = scenarios.monod(f64=True, m_div=0.5)  # everyone above the division mass
    sc = scenarios.small_ring(1000, model=m)
    o = oracle_mod.Oracle(sc, phys_capacity=1500)
    o.init_particles()
    st = o.step()
    assert st["births"] == 500 and st["overflow"] == 500
    assert o.n_used == 1500
    p = o.particles()
    assert (p["id"][1000:] == np.arange(1000, 1500)).all()
    assert (p["state"][0, :500] < 0.56).all()  # divided mothers halved
    assert (p["state"][0, 500:1000] > 0.89).all()  # refused divisions leave mothers whole


def test_liquid_uniform_field_is_steady(oracle_mod):
    sc = scenarios.small_ring(2000, n_steps=1)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    o.s.weight = 0.0  # no contributions
    c0 = o.C.copy()
    for _ in range(5):
        o.step()
    assert np.allclose(o.C, c0, rtol=1e-12, atol=0)


def test_tag3d_quirk_drops_contributions(oracle_mod):
    sc = scenarios.small_ring(4096, feeds=True)
    a = oracle_mod.Oracle(sc)
    a.init_particles()
    b = oracle_mod.Oracle(sc, quirk_tag3d=True)
    b.init_particles()
    a.status[5] = 2
    b.status[5] = 2
    a.s.inactive = b.s.inactive = 1
    a.cycle()
    b.cycle()
    # slots 6..31 of the first chunk are skipped by the quirk
    assert (np.abs(b.src[:, 0]).sum()) < (np.abs(a.src[:, 0]).sum())


def test_reserve_keeps_the_particles(oracle_mod):
    sc = scenarios.small_ring(3000, feeds=True)
    o = oracle_mod.Oracle(sc, phys_capacity=4096)
    o.init_particles()
    o.run(3)
    before = o.particles()
    o.reserve(10240)
    assert o.cap == 10240
    after = o.particles()
    for k in before:
        assert np.array_equal(np.asarray(before[k]), np.asarray(after[k])), k
    o.run(3)  # still steps
