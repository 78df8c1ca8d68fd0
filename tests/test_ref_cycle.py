"""The oracle's cycle composition against the reference's own compiled cycle.

tests/golden/ref_cycle.json records what the reference's particle cycle —
its cycle functors and particle container, compiled from its headers
unmodified (oracle/refbuild/ref_cycle.cpp) — produced, step by step, when run
from the oracle's initial container with the oracle's concentrations and
per-slot draws (tests/golden/make_ref_cycle_golden.py).  Here the oracle runs
the same scenarios and must reproduce, every step of 40:

* the digest of the normalized container (counts, statuses, state bits,
  compartments of Idle particles, both ages), so the update, division into
  the buffer, move, exit, compaction (gap filling) and merge are composed
  as the reference composes them;
* the births, exits and moves its events counted;
* per contribution and compartment, the exact sum of the operands the
  reference's scatter received, within the float rounding of the weight the
  reference multiplies by (2^-22 of the operands' magnitude sum);
* with the chunk early return of the reference's Tag3D scatter emulated,
  the reference's float scatter itself to float accumulation rounding, until
  the first compaction.

The GPU path equals the oracle bit for bit (tests/test_gpu_*.py), so these
records tie it to the reference's composition as well.  Where the
reference's compiled cycle is present (the build container), a live run
checks fresh scenarios too.
"""
import importlib.util
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_cycle.json")


def _gen():
    spec = importlib.util.spec_from_file_location("make_ref_cycle_golden",
                                                  os.path.join(HERE, "golden", "make_ref_cycle_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def gen(oracle_mod):
    return _gen()


def test_golden_made_without_assert_failures(golden):
    assert golden["assert_failures"] == 0
    assert golden["steps"] == 40
    tot = {k: sum(c["totals"][k] for c in golden["cases"].values()) for k in ("births", "exits", "moves",
                                                                               "compactions")}
    # the records exercise every part of the composition
    assert tot["births"] > 1000 and tot["exits"] > 1000 and tot["moves"] > 10000 and tot["compactions"] > 40


CASES = ["fixed_ring", "acetate_ring", "acetate_ring_scheduled_outlet", "fixed_ring_compact_every_step",
         "acetate_0d", "acetate_lattice",
         "fixed_ring_chunk_quirk", "acetate_ring_chunk_quirk"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_the_reference_cycle(oracle_mod, golden, gen, name):
    import ref_cycle

    build, kw = {n: (b, k) for n, b, k in gen.cases()}[name]
    rec = golden["cases"][name]
    assert rec["quirk"] == bool(kw.get("quirk_tag3d"))
    sc = build()
    o = oracle_mod.Oracle(sc, phys_capacity=8 * sc.n_particles, **kw)
    o.init_particles()
    model = sc.model.model_id
    n_ctb = sc.model.n_ctb
    compacted = False
    for k, st in enumerate(rec["steps"]):
        inactive_before = int(o.s.inactive)
        o.step()
        s = o.stats()
        where = f"{name} step {k}"
        assert o.n_used == st["n"], where
        assert (s["births"], s["exits"]) == (st["births"], st["exits"]), where
        if inactive_before == 0:
            assert s["moves"] == st["moves"], where
        assert ref_cycle.digest(o.particles(), s["births"], model) == st["digest"], where
        src = np.asarray(o.src).reshape(sc.net.n_c, -1)[:, :n_ctb].T.ravel()
        exact = np.array(st["exact"], np.uint64).view(np.float64)
        absum = np.array(st["absum"], np.uint32).view(np.float32).astype(np.float64)
        scatter = np.array(st["scatter"], np.uint32).view(np.float32).astype(np.float64)
        if rec["quirk"]:
            if not compacted:
                assert np.all(np.abs(src - scatter) <= golden["scatter_tol"] * absum + 1e-300), where
        else:
            assert np.all(np.abs(src - exact) <= 2.0 ** -22 * absum + 1e-300), where
        compacted = compacted or bool(st["compacted"])


def test_the_reference_scatter_drops_contributions_behind_departed_particles(golden):
    """What the reference's Tag3D scatter loses, from the records: with
    departed particles waiting for compaction, its float sums fall short of
    the exact sum of their own operands by up to a fifth of the operands'
    magnitude (the GPU and the oracle sum every Idle particle)."""
    worst = 0.0
    for name in ("fixed_ring", "acetate_ring"):
        for st in golden["cases"][name]["steps"]:
            exact = np.array(st["exact"], np.uint64).view(np.float64)
            absum = np.array(st["absum"], np.uint32).view(np.float32).astype(np.float64)
            scatter = np.array(st["scatter"], np.uint32).view(np.float32).astype(np.float64)
            ok = absum > 0
            worst = max(worst, float(np.max(np.abs(scatter[ok] - exact[ok]) / absum[ok])))
    assert 0.05 < worst < 0.5


def test_live_reference_cycle_when_built(oracle_mod):
    """Fresh scenarios (other seeds, a lattice with longer rows, exits
    compacted every step) through the reference's compiled cycle beside
    the oracle: every comparison is zero."""
    import ref_cycle

    if not ref_cycle.available():
        pytest.skip("reference cycle not built here")
    from bmc import networks, scenarios

    keys = ("count", "status", "state", "pos", "age_h", "age_d", "births", "exits", "overflow", "moves", "contrib")
    for seed, model in ((21, scenarios.simple_acetate()), (22, scenarios.fixed_length())):
        sc = scenarios.small_ring(2500, model=model, feeds=True, seed=seed)
        net = networks.lattice_vortex(3, side=0.1, peak_velocity=0.05, noise=0.3, seed=seed, max_courant=0.5,
                                      dt=sc.dt)
        sc.net = net
        sc.c0 = np.tile(sc.c0[:1], (net.n_c, 1))
        sc.feeds[0].outlet = net.n_c - 1
        sc.feeds[0].flow = 1e-4
        sc.dead_ratio_threshold = 0.0
        o = oracle_mod.Oracle(sc, phys_capacity=8 * sc.n_particles)
        o.init_particles()
        R = ref_cycle.RefCycle(o, particles_per_team=128)
        for k in range(15):
            r = R.step()
            bad = {a: r[a] for a in keys if r.get(a)}
            assert not bad and r["digest_ref"] == r["digest_oracle"], (seed, k, bad)
        assert R.misses() == 0
        R.close()
