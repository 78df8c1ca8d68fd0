"""GPU path (libbmc through its C-ABI) against the CPU restatement.

Integer outcomes (compartments, statuses, ids, counts) and every floating
value (state, ages, concentrations, masses, sources) are compared bit for
bit: the draws are the same Philox stream on both sides, contribution sums
are exact integer sums, and both sides round each operation the same way.
"""
import numpy as np
import pytest

from bmc import scenarios

pytestmark = pytest.mark.gpu


def make_pair(oracle_mod, scen, capacity=None):
    from bmc.sim import GpuScenario

    g = GpuScenario(scen, capacity=capacity)
    o = oracle_mod.Oracle(scen, phys_capacity=g.cap)
    w = o.init_particles()
    # the initial mass and volume totals are summed in different orders
    # (tree reduction on the device); the oracle then takes the device weight
    assert abs(w - g.weight) <= 1e-12 * g.weight
    o.set_weight(g.weight)
    return g, o


def same_bits(a, b) -> bool:
    """Bitwise equality, except that any NaN equals any NaN (payloads differ
    between the CPU and the GPU)."""
    if a.shape != b.shape:
        return False
    ui = {8: np.uint64, 4: np.uint32}[a.dtype.itemsize]
    eq = a.view(ui) == b.view(ui)
    return bool(np.all(eq | (np.isnan(a) & np.isnan(b))))


def assert_same_particles(g, o, where=""):
    pg, po = g.particles(), o.particles()
    assert len(pg["pos"]) == len(po["pos"]), where
    for k in ("pos", "status", "id"):
        assert np.array_equal(pg[k], po[k]), f"{where}: {k}"
    for k in ("age_h", "age_d", "state"):
        assert same_bits(pg[k], po[k]), f"{where}: {k}"


def assert_same_liquid(g, o, where=""):
    lq = g.liquid()
    for k, ref in (("C", o.C), ("M", o.M), ("src", o.src)):
        assert same_bits(lq[k], ref), f"{where}: {k}"


def assert_same_stats(gs, os_, where=""):
    for k in ("n_used", "births", "exits", "moves", "overflow"):
        assert gs[k] == os_[k], f"{where}: {k} gpu={gs[k]} cpu={os_[k]}"
    assert gs["error"] == 0, where


def test_draws_match_oracle(oracle_mod):
    from bmc.sim import debug_draws

    ids = np.arange(0, 5000, 7, dtype=np.uint32)
    for step, purpose in ((0, 0), (123, 1), (0xFFFFFFFF, 2)):
        got = debug_draws(0x1234ABCD5678, ids, step, purpose)
        ref = np.stack([oracle_mod.draws(0x1234ABCD5678, int(i), step, purpose) for i in ids])
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_init_identical(oracle_mod):
    g, o = make_pair(oracle_mod, scenarios.small_ring(5000))
    assert_same_particles(g, o, "init")


@pytest.mark.parametrize("f64", [True, False])
def test_ring_monod_steps(oracle_mod, f64):
    sc = scenarios.small_ring(6000, f64=f64, feeds=True)
    g, o = make_pair(oracle_mod, sc)
    for k in range(12):
        gs = g.step()
        os_ = o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
    assert_same_particles(g, o, "end")


@pytest.mark.parametrize("shape", [None, (256, 2, 0), (544, 2, 0)])
@pytest.mark.parametrize("n_c", [1, 3])
def test_tiny_domains_warp_aggregated_scatter(oracle_mod, n_c, shape):
    """Domains of at most 4 compartments sum the contributions of a warp per
    compartment before the shared-memory atomic: sums stay exact."""
    if n_c == 1:
        sc = scenarios.zero_d(20000, model=scenarios.monod(f64=False), outlet=True)
    else:
        sc = scenarios.small_ring(20000, n_c=n_c, f64=False, feeds=True)
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    for k in range(8):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
    assert_same_particles(g, o, "end")


def test_cycle_only_uses_given_concentrations(oracle_mod):
    sc = scenarios.small_ring(3000, feeds=False)
    g, o = make_pair(oracle_mod, sc)
    gs = g.cycle()
    o.cycle()
    o.post_cycle()
    o.s.step += 1
    assert gs["moves"] == o.s.moves
    assert_same_particles(g, o, "cycle")
    assert np.array_equal(g.liquid()["src"].view(np.uint64), o.src.view(np.uint64))


# default launch shape, and the shape that stages tiles through the copy engine
SHAPES = [None, (288, 4, 0), (256, 2, 0)]


def test_cycle_external_host_and_device_pointers(oracle_mod):
    """bmc_cycle_external: the caller's concentrations in, the cycle's
    contributions out, bit for bit as the restatement's cycle."""
    sc = scenarios.small_ring(6000, feeds=True)
    g, o = make_pair(oracle_mod, sc)
    rng = np.random.default_rng(11)
    torch = pytest.importorskip("torch")
    for k in range(4):
        conc = rng.uniform(0.5, 8.0, size=(sc.net.n_c, sc.n_species))
        if k % 2 == 0:
            src, st = g.cycle_external(conc)
        else:
            dc = torch.tensor(conc, dtype=torch.float64, device="cuda")
            out = torch.zeros_like(dc)
            _, st = g.cycle_external(dc, out)
            src = out.cpu().numpy()
        o.C[:] = conc
        o.cycle()
        o.post_cycle()
        o.s.step += 1
        assert same_bits(src, o.src), f"cycle {k}"
        assert st["moves"] == o.s.moves and st["exits"] == o.s.exits, f"cycle {k}"
    assert_same_particles(g, o, "end")


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("f64", [True, False])
def test_lattice_overflow_model(oracle_mod, f64, shape):
    sc = scenarios.workload(2, n_particles=40000, n_steps=6, f64=f64)
    sc.net = __import__("bmc.networks", fromlist=["x"]).lattice_vortex(4, seed=7)
    sc.c0 = sc.c0[: sc.net.n_c]
    sc.feeds[0].outlet = sc.net.n_c - 1
    sc.feeds[0].flow = 2e-4
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    for k in range(6):
        gs = g.step()
        os_ = o.step(4)
        assert_same_stats(gs, os_, f"step {k}")
    assert_same_liquid(g, o, "end")
    assert_same_particles(g, o, "end")


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("general", [False, True])
def test_fixed_length_reference_model(oracle_mod, general, shape):
    sc = scenarios.small_ring(16000, model=scenarios.fixed_length(general=general), feeds=True)
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    births = 0
    for k in range(60):
        gs = g.step()
        os_ = o.step()
        assert_same_stats(gs, os_, f"step {k}")
        births += gs["births"]
    assert births > 0
    assert np.isfinite(g.particles()["state"]).all()
    assert_same_particles(g, o, "end")
    assert_same_liquid(g, o, "end")


@pytest.mark.parametrize("shape", SHAPES)
def test_divisions_overflow_and_compaction(oracle_mod, shape):
    # division mass inside the initial range: many births, refusals once full
    m = scenarios.monod(f64=True, m_div=1.0)
    sc = scenarios.zero_d(3000, model=m, outlet=True)
    sc.feeds[0].flow = 1e-3  # strong outlet: exits trigger compaction
    g, o = make_pair(oracle_mod, sc, capacity=4096)
    if shape:
        g.set_shape(*shape)
    saw = {"births": 0, "overflow": 0, "compacted": 0}
    for k in range(25):
        gs = g.step()
        os_ = o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert gs["compacted"] == os_["compacted"], f"step {k}"
        saw["births"] += gs["births"]
        saw["overflow"] += gs["overflow"]
        saw["compacted"] += gs["compacted"]
        assert_same_particles(g, o, f"step {k}")
    assert saw["births"] > 0 and saw["compacted"] > 0
    assert_same_liquid(g, o, "end")


def test_graph_run_equals_steps(oracle_mod):
    sc = scenarios.small_ring(5000, feeds=True)
    g, o = make_pair(oracle_mod, sc)
    gs = g.run(15)
    o.run(15)
    assert gs["n_used"] == o.n_used and gs["step"] == 15
    assert_same_particles(g, o, "run")
    assert_same_liquid(g, o, "run")


def test_repartition_and_force_remove(oracle_mod):
    sc = scenarios.small_ring(4096, feeds=True)
    sc.feeds[0].flow = 2e-3
    g, o = make_pair(oracle_mod, sc)
    for _ in range(5):
        g.step()
        o.step()
    assert np.array_equal(g.repartition(), o.repartition())
    g.force_remove_dead()
    import ctypes as ct

    oracle_mod.lib().orc_remove_inactive(ct.byref(o.s), o.s.inactive)
    assert_same_particles(g, o, "force_remove_dead")


@pytest.mark.parametrize("shape", [(256, 1, 0), (256, 2, 0), (256, 4, 1), (512, 2, 0), (1024, 1, 0),
                                   (288, 4, 0), (288, 4, 1), (544, 2, 0)])
def test_launch_shapes_bit_identical(oracle_mod, shape):
    """Results do not depend on the launch shape: sums are exact."""
    sc = scenarios.workload(2, n_particles=30000, f64=True)
    sc.net = __import__("bmc.networks", fromlist=["x"]).lattice_vortex(4, seed=9)
    sc.c0 = sc.c0[: sc.net.n_c]
    sc.feeds[0].outlet = sc.net.n_c - 1
    sc.feeds[0].flow = 3e-4
    g, o = make_pair(oracle_mod, sc)
    g.set_shape(*shape)
    g.run(7)
    o.run(7, 2)
    assert_same_particles(g, o, f"shape {shape}")
    assert_same_liquid(g, o, f"shape {shape}")
