"""Free-running statistical agreement (32 seeds, 99 % family-wise bands).

The reference's Kokkos path draws from a XorShift1024 pool; the GPU path
from Philox4x32-10, so free-running runs agree as distributions.  Two
comparisons:

* against the reference's own particle cycle: tests/golden/ref_stats.json
  holds the summaries of 32 free-running runs of the reference's compiled
  cycle functors and particle container on the SimpleAcetate 10-ring,
  drawing from their own xorshift1024* stream, coupled to the oracle's
  liquid step (tests/golden/make_ref_stats_golden.py); the GPU's and the
  oracle's summaries (Philox) must fall within the bands of
  `stat_bands.band_test`, and a planted change (outlet flow doubled) must
  fall outside;
* the Monod 10-ring of the benchmark's model, GPU (Philox) against the
  oracle on an independent xorshift stream, and the band test's own checks.
"""
import dataclasses
import os

import numpy as np
import pytest

from bmc import scenarios
from stat_bands import N_SEEDS, band_test, seeded, summary

XORSHIFT = 1
THREADS = max(1, min(16, os.cpu_count() or 1))


def free_scenario(n_particles: int, n_steps: int):
    """10-compartment ring with a glucose feed and an outlet, Monod growth
    fast enough (0.05/s) that divisions and exits both happen."""
    sc = scenarios.small_ring(n_particles=n_particles, n_c=10, seed=1, f64=True,
                              model=scenarios.monod(f64=True, mu_max=0.05), n_steps=n_steps,
                              dt=0.1, feeds=True)
    sc.alloc_factor = 4.0
    return sc


# the reference's recorded runs used seeds REFERENCE_SEED0 + k; the GPU and
# the oracle use other seeds, so the samples are independent
REFERENCE_SEED0 = 900
GOLDEN_STATS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_stats.json")


def reference_scenario():
    """SimpleAcetate (a model of the reference) on the 10-ring with a glucose
    feed and an outlet: 4000 particles, 200 steps of 0.1 s; divisions,
    moves and exits all happen."""
    sc = scenarios.small_ring(4000, model=scenarios.simple_acetate(), feeds=True, n_steps=200)
    sc.alloc_factor = 4.0
    return sc


def reference_stats() -> np.ndarray:
    import json

    with open(GOLDEN_STATS) as f:
        g = json.load(f)
    assert g["assert_failures"] == 0 and len(g["summaries"]) == N_SEEDS
    return np.array(g["summaries"])


def oracle_summary(oracle_mod, scen, draw_mode: int) -> np.ndarray:
    o = oracle_mod.Oracle(scen, phys_capacity=(scen.capacity + 1023) // 1024 * 1024,
                          draw_mode=draw_mode)
    o.init_particles()
    o.run(scen.n_steps, n_threads=THREADS)
    st = o.stats()
    assert st["error"] == 0 and st["overflow"] == 0
    return summary(o.particles(), o.C, scen.net.n_c, scen.n_particles, st["next_id"])


def test_oracle_matches_the_reference_cycle_free_running(oracle_mod):
    ref = reference_stats()
    a = np.stack([oracle_summary(oracle_mod, seeded(reference_scenario(), 100 + k), 0) for k in range(N_SEEDS)])
    assert a[:, 21].mean() > 0 and ref[:, 21].mean() > 0  # births on both sides
    ok, ratio, worst = band_test(a, ref)
    assert ok, f"statistic {worst} outside its band (ratio {ratio:.2f})"


def test_reference_comparison_sees_a_planted_change(oracle_mod):
    """The same comparison with the outlet flow doubled on the oracle's side
    must fail."""
    ref = reference_stats()
    base = reference_scenario()
    planted = dataclasses.replace(base, feeds=[dataclasses.replace(base.feeds[0], flow=2.0 * base.feeds[0].flow)])
    a = np.stack([oracle_summary(oracle_mod, seeded(planted, 100 + k), 0) for k in range(N_SEEDS)])
    assert not band_test(a, ref)[0]


def test_reference_records_replay_when_built(oracle_mod):
    """Where the reference's compiled cycle is present, a recorded run
    replays to the same summary (the records are deterministic)."""
    import importlib.util

    import ref_cycle

    if not ref_cycle.available():
        pytest.skip("reference cycle not built here")
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_ref_stats_golden",
                                                  os.path.join(here, "golden", "make_ref_stats_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    assert np.array_equal(np.array(m.run(REFERENCE_SEED0 + 3)), reference_stats()[3])


@pytest.mark.gpu
def test_gpu_free_running_matches_the_reference_cycle(oracle_mod):
    from bmc.sim import GpuScenario

    ref = reference_stats()
    gs = []
    for k in range(N_SEEDS):
        sc = seeded(reference_scenario(), 100 + k)
        g = GpuScenario(sc)
        g.run(sc.n_steps)
        st = g.stats()
        assert st["error"] == 0 and st["overflow"] == 0
        gs.append(summary(g.particles(), g.liquid()["C"], sc.net.n_c, sc.n_particles, st["next_id"]))
        g.close()
    a = np.stack(gs)
    ok, ratio, worst = band_test(a, ref)
    assert ok, f"statistic {worst} outside its band (ratio {ratio:.2f})"


def test_band_test_accepts_and_rejects():
    rng = np.random.default_rng(0)
    a = rng.normal(1.0, 0.1, size=(N_SEEDS, 5))
    b = rng.normal(1.0, 0.1, size=(N_SEEDS, 5))
    assert band_test(a, b)[0]
    b[:, 3] += 0.5
    ok, _, worst = band_test(a, b)
    assert not ok and worst == 3


def test_oracle_draw_sources_agree(oracle_mod):
    base = free_scenario(4000, 200)
    a = np.stack([oracle_summary(oracle_mod, seeded(base, 100 + k), 0) for k in range(N_SEEDS)])
    b = np.stack([oracle_summary(oracle_mod, seeded(base, 900 + k), XORSHIFT)
                  for k in range(N_SEEDS)])
    assert a[:, 21].mean() > 0  # births happened
    ok, ratio, worst = band_test(a, b)
    assert ok, f"statistic {worst} outside its band (ratio {ratio:.2f})"


def test_band_test_detects_a_planted_model_change(oracle_mod):
    """The same comparison with the outlet flow doubled on one side must
    fail: the bands are tight enough to see a real difference."""
    base = free_scenario(4000, 200)
    planted = dataclasses.replace(base, feeds=[dataclasses.replace(base.feeds[0],
                                                                   flow=2.0 * base.feeds[0].flow)])
    a = np.stack([oracle_summary(oracle_mod, seeded(base, 100 + k), 0) for k in range(N_SEEDS)])
    b = np.stack([oracle_summary(oracle_mod, seeded(planted, 900 + k), XORSHIFT)
                  for k in range(N_SEEDS)])
    assert not band_test(a, b)[0]


@pytest.mark.gpu
def test_gpu_free_running_matches_independent_stream(oracle_mod):
    from bmc.sim import GpuScenario

    base = free_scenario(20000, 300)
    gs, os_ = [], []
    for k in range(N_SEEDS):
        sc = seeded(base, 100 + k)
        g = GpuScenario(sc)
        g.run(sc.n_steps)
        st = g.stats()
        assert st["error"] == 0 and st["overflow"] == 0
        gs.append(summary(g.particles(), g.liquid()["C"], sc.net.n_c, sc.n_particles,
                          st["next_id"]))
        g.close()
        os_.append(oracle_summary(oracle_mod, seeded(base, 900 + k), XORSHIFT))
    a, b = np.stack(gs), np.stack(os_)
    assert a[:, 21].mean() > 0 and a[:, 20].mean() > 0
    ok, ratio, worst = band_test(a, b)
    assert ok, f"statistic {worst} outside its band (ratio {ratio:.2f})"
