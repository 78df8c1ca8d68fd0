"""Batched form: many uneven scenarios advanced by one set of launches per
step give, for each scenario, exactly the result it gives alone (and the CPU
restatement's): draws are keyed by particle, sums are exact."""
import numpy as np
import pytest

from bmc import scenarios

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    ui = {8: np.uint64, 4: np.uint32}[a.dtype.itemsize]
    return a.shape == b.shape and bool(np.all((a.view(ui) == b.view(ui)) | (np.isnan(a) & np.isnan(b))))


def assert_same(g1, g2, where):
    p1, p2 = g1.particles(), g2.particles()
    for k in ("pos", "status", "id"):
        assert np.array_equal(p1[k], p2[k]), f"{where}: {k}"
    for k in ("age_h", "age_d", "state"):
        assert same_bits(p1[k], p2[k]), f"{where}: {k}"
    l1, l2 = g1.liquid(), g2.liquid()
    for k in ("C", "M", "src"):
        assert same_bits(l1[k], l2[k]), f"{where}: {k}"


def _mix(n=7, scale=0.02):
    return [scenarios.batch_scenario(k, seed=77, particle_scale=scale) for k in range(n)]


@pytest.mark.parametrize("shape", [(256, 2, 0), (1024, 1, 0), (288, 4, 0), (544, 2, 0)])
def test_batch_equals_alone(shape):
    from bmc.sim import GpuBatch, GpuScenario

    scens = _mix()
    batch_members = [GpuScenario(s) for s in scens]
    alone = [GpuScenario(s) for s in scens]
    b = GpuBatch(batch_members)
    b.set_shape(*shape)
    steps = 9
    b.run(steps, 0.1)
    b.synchronize()
    for g in alone:
        g.run(steps)
    for k, (gb, ga) in enumerate(zip(batch_members, alone)):
        st = gb.stats()
        assert st["step"] == steps and st["error"] == 0
        assert_same(gb, ga, f"scenario {k} ({scens[k].net.n_c} compartments, {scens[k].n_particles} particles)")
    b.close()


def test_batch_member_matches_oracle(oracle_mod):
    from bmc.sim import GpuBatch, GpuScenario

    scens = _mix(5, 0.01)
    members = [GpuScenario(s) for s in scens]
    b = GpuBatch(members)
    b.run(6, 0.1)
    b.synchronize()
    k = int(np.argmax([s.net.n_c for s in scens]))
    o = oracle_mod.Oracle(scens[k], phys_capacity=members[k].cap)
    o.init_particles()
    o.set_weight(members[k].weight)
    o.run(6)
    pg, po = members[k].particles(), o.particles()
    for key in ("pos", "status", "id"):
        assert np.array_equal(pg[key], po[key]), key
    assert same_bits(pg["state"], po["state"])
    assert same_bits(members[k].liquid()["C"], o.C)
    b.close()


def test_batch_then_alone_continues_consistently():
    """A scenario can leave a batch and continue alone (serving retires and
    re-forms batches between chunks)."""
    from bmc.sim import GpuBatch, GpuScenario

    scens = _mix(4, 0.01)
    mixed = [GpuScenario(s) for s in scens]
    ref = GpuScenario(scens[2])
    b = GpuBatch(mixed)
    b.run(4, 0.1)
    b.synchronize()
    b.close()
    b2 = GpuBatch([mixed[0], mixed[2]])
    b2.run(3, 0.1)
    b2.synchronize()
    mixed[2].run(2)
    ref.run(9)
    assert_same(mixed[2], ref, "regrouped")
    b2.close()


def test_slot_batch_fill_empty_refill_equals_alone():
    """Scenarios entering and leaving slots between runs advance exactly as
    they would alone, and empty slots do nothing."""
    from bmc.sim import GpuBatch, GpuScenario

    scens = _mix(6, 0.02)
    members = [GpuScenario(s) for s in scens]
    alone = [GpuScenario(s) for s in scens]
    b = GpuBatch.slots(8, scens[0].model)
    for k in range(4):
        b.set_slot(2 * k, members[k])  # slots 0, 2, 4, 6; 1, 3, 5, 7 empty
    b.run(5, 0.1)
    b.synchronize()
    b.set_slot(2, None)  # members[1] leaves after 5 steps
    b.set_slot(3, members[4])  # members[4] joins
    b.run(4, 0.1)
    b.synchronize()
    b.set_slot(7, members[5])
    b.run(3, 0.1)
    b.synchronize()
    steps = [12, 5, 12, 12, 7, 3]
    for g, n in zip(alone, steps):
        g.run(n)
    for k, (gm, ga) in enumerate(zip(members, alone)):
        assert gm.stats()["step"] == steps[k]
        assert_same(gm, ga, f"scenario {k}")
    for slot in (0, 3, 4, 6, 7):
        b.set_slot(slot, None)
    b.close()


@pytest.mark.parametrize("n_small,n_large", [(17, 25), (300, 700)])
def test_slot_batch_recaptures_when_a_larger_domain_joins(n_small, n_large):
    """A scenario with more compartments joining after the step graph was
    captured needs more liquid-step blocks (and, past 256 compartments, more
    plan slices) even when its shared accumulator rounds to the same size:
    the batch re-captures, and both scenarios advance as they would alone."""
    from bmc.sim import GpuBatch, GpuScenario

    def ring(n_c, seed):  # 4 species: 8 compartments per liquid-step block
        return scenarios.small_ring(3000, n_c=n_c, feeds=True, seed=seed, model=scenarios.overflow(f64=True))

    small, large = ring(n_small, 3), ring(n_large, 4)
    gs, gl = GpuScenario(small), GpuScenario(large)
    a_s, a_l = GpuScenario(small), GpuScenario(large)
    b = GpuBatch.slots(4, small.model)
    b.set_slot(0, gs)
    b.run(3, small.dt)
    b.synchronize()
    b.set_slot(1, gl)
    b.run(4, small.dt)
    b.synchronize()
    a_s.run(7)
    a_l.run(4)
    assert_same(gs, a_s, "small")
    assert_same(gl, a_l, "large")
    b.set_slot(0, None)
    b.set_slot(1, None)
    b.close()
