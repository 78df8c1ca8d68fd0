"""Edge cases of the GPU path against the CPU restatement: an empty
container, a container that empties, ragged particle counts around tile and
warp boundaries, rows longer than any benchmark's, exhausted particle ids,
and malformed inputs that the library must refuse (the scenario stays
usable afterwards)."""
import ctypes as ct

import numpy as np
import pytest

from bmc import networks, scenarios

pytestmark = pytest.mark.gpu


def _parity(g, o, steps, where):
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats

    for k in range(steps):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"{where} step {k}")
        assert_same_liquid(g, o, f"{where} step {k}")
    assert_same_particles(g, o, where)


def test_empty_container(oracle_mod):
    from bmc.sim import GpuScenario

    sc = scenarios.small_ring(0, feeds=True)
    g = GpuScenario(sc, capacity=1024, init=False)
    empty = dict(state=np.zeros((2, 0)), pos=np.zeros(0, np.uint32), status=np.zeros(0, np.uint8),
                 age_h=np.zeros(0, np.float32), age_d=np.zeros(0, np.float32), id=np.zeros(0, np.uint32))
    g.set_particles(empty, 0)
    g.set_weight(1.0)
    o = oracle_mod.Oracle(sc, phys_capacity=g.cap)
    o.set_weight(1.0)
    _parity(g, o, 6, "empty")
    assert g.stats()["n_used"] == 0


def test_container_that_empties(oracle_mod):
    """A 0-D reactor with an outlet faster than growth: every particle
    leaves, the container compacts to nothing and keeps stepping."""
    from test_gpu_parity import make_pair

    sc = scenarios.zero_d(3000, outlet=True)
    sc.feeds[0].flow = 1e-2  # dt F / V = 1: 63 % of the particles leave per step
    g, o = make_pair(oracle_mod, sc)
    _parity(g, o, 30, "emptying")
    st = g.stats()
    assert st["n_used"] - st["inactive"] == 0


@pytest.mark.parametrize("shape", [None, (256, 2, 0)])
@pytest.mark.parametrize("n", [1, 31, 1023, 1025, 2047])
def test_ragged_particle_counts(oracle_mod, n, shape):
    from test_gpu_parity import make_pair

    sc = scenarios.small_ring(n, n_c=16, feeds=True)
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    _parity(g, o, 4, f"n={n}")


def complete_graph(n_c=13, seed=5):
    rng = np.random.default_rng(seed)
    src, dst = [], []
    for i in range(n_c):
        for j in range(n_c):
            if i != j:
                src.append(i)
                dst.append(j)
    src, dst = np.array(src), np.array(dst)
    flow = rng.uniform(0.5e-5, 2e-5, size=len(src))
    vol = rng.uniform(0.5e-3, 2e-3, size=n_c)
    return networks.Network(n_c, vol, src, dst, flow).finalize()


@pytest.mark.parametrize("shape", [None, (256, 2, 0)])
@pytest.mark.parametrize("n_c", [9, 10, 13])
def test_long_neighbour_rows(oracle_mod, shape, n_c):
    """Every compartment connected to all others: rows of 8 entries (the
    longest the threshold count covers), 9 and 12 (the bisection)."""
    from test_gpu_parity import make_pair

    net = complete_graph(n_c)
    assert net.K == n_c - 1
    sc = scenarios.small_ring(8000, feeds=True)
    sc.net = net
    sc.c0 = np.full((net.n_c, 1), 5.0)
    sc.feeds[0].outlet = net.n_c - 1
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    _parity(g, o, 6, f"K={net.K}")


def test_automatic_shape_with_one_staging_block_per_sm(oracle_mod):
    """10,648 compartments: the shared accumulator and the stage buffers of
    two blocks do not fit on an SM, so the automatic shape runs one
    tile-staging block per SM; results stay those of the CPU restatement."""
    from test_gpu_parity import make_pair

    net = networks.lattice_vortex(22, side=1.0, peak_velocity=0.5, noise=0.1, seed=7, max_courant=0.4, dt=0.05)
    sc = scenarios.workload(2, n_particles=60000, f64=True)
    sc.net = net
    sc.c0 = np.tile(sc.c0[:1], (net.n_c, 1))
    sc.feeds[0].outlet = net.n_c - 1
    g, o = make_pair(oracle_mod, sc)
    _parity(g, o, 3, "n_c=10648")


def _on_lattice(sc, n):
    """The scenario moved onto an n^3 vortex lattice (outlet in the last
    compartment, the first compartment's concentrations everywhere)."""
    net = networks.lattice_vortex(n, side=1.0, peak_velocity=0.5, noise=0.1, seed=7, max_courant=0.4, dt=sc.dt)
    sc.net = net
    sc.c0 = np.tile(sc.c0[:1], (net.n_c, 1))
    for f in sc.feeds:
        f.outlet = net.n_c - 1
    return sc


def test_domain_beyond_any_shared_accumulator(oracle_mod):
    """32,768 compartments: a shared accumulator (256 KiB) fits no block, so
    the contributions go straight to the scenario's global accumulator;
    results stay those of the CPU restatement."""
    from test_gpu_parity import make_pair

    sc = _on_lattice(scenarios.workload(2, n_particles=200000, f64=True), 32)
    assert sc.net.n_c == 32768
    g, o = make_pair(oracle_mod, sc)
    _parity(g, o, 3, "n_c=32768")


def test_general_model_beyond_the_shared_accumulator(oracle_mod):
    """The per-particle contribution path (FixedLength through its general
    form) on 32,768 compartments, summed in the global accumulator."""
    from test_gpu_parity import make_pair

    sc = _on_lattice(scenarios.small_ring(100000, model=scenarios.fixed_length(general=True), feeds=True,
                                          dt=0.05), 32)
    g, o = make_pair(oracle_mod, sc)
    _parity(g, o, 3, "general n_c=32768")


def test_batch_with_a_domain_beyond_the_shared_accumulator():
    """A batch holding one 32,768-compartment domain sums every member's
    contributions in the global accumulators; each member still equals its
    run alone (where the small ones use the shared accumulator)."""
    from bmc.sim import GpuBatch, GpuScenario
    from test_gpu_batch import assert_same

    scens = [_on_lattice(scenarios.workload(2, n_particles=100000, f64=True), 32)]
    scens += [scenarios.small_ring(20000, model=scenarios.overflow(f64=True), feeds=True, seed=s, dt=0.05)
              for s in (3, 4)]
    members = [GpuScenario(s) for s in scens]
    alone = [GpuScenario(s) for s in scens]
    b = GpuBatch(members)
    b.run(3, 0.05)
    b.synchronize()
    for g in alone:
        g.run(3)
    for k, (gb, ga) in enumerate(zip(members, alone)):
        assert gb.stats()["step"] == 3 and gb.stats()["error"] == 0
        assert_same(gb, ga, f"member {k} ({scens[k].net.n_c} compartments)")
    b.close()


def test_register_streaming_shape_refuses_a_domain_beyond_shared_memory():
    """The register-streaming kernels keep a shared accumulator: asked for on
    a domain whose accumulator fits no block, the step is refused."""
    from bmc import _lib
    from bmc.sim import GpuScenario

    sc = _on_lattice(scenarios.workload(2, n_particles=20000, f64=True), 32)
    g = GpuScenario(sc)
    g.set_shape(256, 2, 0)
    with pytest.raises(_lib.BmcError) as e:
        g.step()
    assert e.value.code == -6  # BMC_E_UNSUPPORTED
    assert g.stats()["step"] == 0


def test_particle_id_space_exhaustion():
    """Births that would pass 2^32 ids set the error word (never a fault)."""
    from bmc import _lib
    from bmc.sim import GpuScenario

    m = scenarios.monod(f64=True, m_div=1.0)  # every particle asks to divide
    sc = scenarios.zero_d(2000, model=m, outlet=False)
    g = GpuScenario(sc, capacity=8192)
    parts = g.particles()
    g.set_particles(parts, (1 << 32) - 10)
    with pytest.raises(_lib.BmcError) as e:
        g.step()
    assert e.value.code == -5  # BMC_E_DEVICE
    st = _lib.StepStats()
    assert _lib.load().bmc_read_stats(g.handle, ct.byref(st)) == -5
    assert st.error & 4


def test_malformed_inputs_are_refused():
    from bmc import _lib
    from bmc.sim import GpuScenario

    sc = scenarios.small_ring(2000, feeds=True)
    g = GpuScenario(sc)
    net = sc.net
    L = _lib.load()

    def domain(vol, nbr, outf, cdf):
        return L.bmc_domain_update(g.handle, net.n_c, net.K, vol.ctypes.data, nbr.ctypes.data,
                                   outf.ctypes.data, cdf.ctypes.data)

    vol = np.ascontiguousarray(net.volume, dtype=np.float64)
    nbr = np.ascontiguousarray(net.neighbors, dtype=np.uint64)
    outf = np.ascontiguousarray(net.out_flow, dtype=np.float64)
    cdf = np.ascontiguousarray(net.cdf, dtype=np.float64)
    bad = cdf.copy()
    bad[0, 0] = np.nan
    assert domain(vol, nbr, outf, bad) == -1 and b"NaN" in L.bmc_last_error()
    bad = cdf.copy()
    bad[0, :] = bad[0, ::-1] * 0.5  # decreasing row
    if net.K > 1 and bad[0, 0] > bad[0, 1]:
        assert domain(vol, nbr, outf, bad) == -1 and b"non-decreasing" in L.bmc_last_error()
    badn = nbr.copy()
    badn[1, 0] = net.n_c
    assert domain(vol, badn, outf, cdf) == -1 and b"out of range" in L.bmc_last_error()
    badv = vol.copy()
    badv[2] = 0.0
    assert domain(badv, nbr, outf, cdf) == -1 and b"volumes" in L.bmc_last_error()
    # feeds outside the domain
    f = (_lib.Feed * 1)()
    f[0].inlet = net.n_c
    f[0].outlet = -1
    f[0].flow = 1e-5
    assert L.bmc_set_feeds(g.handle, 1, f) == -1
    # more particles than the container holds
    n = g.cap + 1
    z = np.zeros(n)
    assert L.bmc_set_particles(g.handle, n, np.zeros((2, n)).ctypes.data, np.zeros(n, np.uint32).ctypes.data,
                               np.zeros(n, np.uint8).ctypes.data, np.zeros(n, np.float32).ctypes.data,
                               np.zeros(n, np.float32).ctypes.data, np.zeros(n, np.uint32).ctypes.data,
                               ct.c_uint64(n)) == -4
    del z
    # the scenario still steps after the refusals
    st = g.step()
    assert st["error"] == 0 and st["n_used"] > 0


def test_step_read_equals_step_then_read_liquid():
    """bmc_step_read returns the counters and concentrations bmc_step +
    bmc_read_liquid return, including after the step limit is reached."""
    from bmc.sim import GpuScenario

    sc = scenarios.small_ring(5000, feeds=True)
    g1, g2 = GpuScenario(sc), GpuScenario(sc)
    g1.set_step_limit(6)
    g2.set_step_limit(6)
    conc = np.zeros((sc.net.n_c, sc.n_species))
    for k in range(8):
        s1 = g1.step()
        c1 = g1.liquid()["C"]
        s2 = g2.step_read(conc)
        assert s1 == s2, k
        assert np.array_equal(c1.view(np.uint64), conc.view(np.uint64)), k
    # with the counters current on the host, one concentration buffer (not
    # both) travels back per step, beside the control block
    from bmc.sim import transfer_bytes

    g2.set_step_limit(0)
    g2.step_read(conc)
    d0 = transfer_bytes()[1]
    g2.stats()
    ctl_bytes = transfer_bytes()[1] - d0
    d0 = transfer_bytes()[1]
    g2.step_read(conc)
    assert transfer_bytes()[1] - d0 == ctl_bytes + sc.net.n_c * sc.n_species * 8
    g1.set_step_limit(0)
    g1.step()
    g1.step()
    assert np.array_equal(g1.liquid()["C"].view(np.uint64), conc.view(np.uint64))
    with pytest.raises(ValueError):
        g2.step_read(np.zeros(3))


def test_pipelined_steps_equal_step_read():
    """bmc_step_enqueue / bmc_step_collect with two steps in flight give
    the counters and concentrations bmc_step_read gives, bit for bit,
    through the step limit; other stepping calls wait for the collects."""
    from bmc import _lib
    from bmc.sim import GpuScenario

    sc = scenarios.small_ring(5000, feeds=True)
    g1, g2 = GpuScenario(sc), GpuScenario(sc)
    g1.set_step_limit(9)
    g2.set_step_limit(9)
    shape = (sc.net.n_c, sc.n_species)
    ref = []
    for _ in range(12):
        c = np.zeros(shape)
        ref.append((g1.step_read(c), c))
    slots = [(_lib.StepStats(), np.zeros(shape)) for _ in range(2)]
    got = []
    g2.step_enqueue(*slots[0])
    for k in range(1, 13):
        if k < 12:
            g2.step_enqueue(*slots[k % 2])
        g2.step_collect()
        st, c = slots[(k - 1) % 2]
        got.append((st.as_dict(), c.copy()))
    for k, ((s1, c1), (s2, c2)) in enumerate(zip(ref, got)):
        assert s1 == s2, k
        assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64)), k
    # a third step in flight, a collect with nothing enqueued and a plain
    # step between enqueue and collect are refused
    g2.set_step_limit(0)
    g2.step_enqueue(*slots[0])
    g2.step_enqueue(*slots[1])
    with pytest.raises(_lib.BmcError):
        g2.step_enqueue(_lib.StepStats(), np.zeros(shape))
    with pytest.raises(_lib.BmcError):
        g2.step()
    g2.step_collect()
    g2.step_collect()
    with pytest.raises(_lib.BmcError):
        g2.step_collect()
    g1.set_step_limit(0)
    g1.step()
    c1 = np.zeros(shape)
    g1.step_read(c1)
    assert np.array_equal(c1.view(np.uint64), slots[1][1].view(np.uint64))
    assert g2.step() == g1.step()


def test_pipelined_steps_with_other_calls_between():
    """A step's transfer goes out with the next call on the scenario: calls
    between an enqueue and its collect (counter and field reads, feeds, a
    liquid read, the weight through a descriptor upload) see and leave the
    results bmc_step_read gives."""
    from bmc import _lib
    from bmc.sim import GpuScenario

    sc = scenarios.small_ring(5000, feeds=True)
    g1, g2 = GpuScenario(sc), GpuScenario(sc)
    shape = (sc.net.n_c, sc.n_species)
    feeds = (_lib.Feed * len(sc.feeds))()
    for k, fd in enumerate(sc.feeds):
        feeds[k].inlet, feeds[k].outlet, feeds[k].flow = fd.inlet, fd.outlet, fd.flow
        for sp in range(len(fd.conc)):
            feeds[k].conc[sp] = float(fd.conc[sp])
    for k in range(6):
        c1 = np.zeros(shape)
        s1 = g1.step_read(c1)
        st, c2 = _lib.StepStats(), np.zeros(shape)
        g2.step_enqueue(st, c2)
        if k % 3 == 0:
            g2.stats()
        elif k % 3 == 1:
            g2.liquid()
        else:
            _lib.call("bmc_set_feeds", g2.handle, len(sc.feeds), feeds)
            g2.set_weight(g2.weight)
        g2.step_collect()
        assert st.as_dict() == s1, k
        assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64)), k
    assert np.array_equal(g1.liquid()["C"].view(np.uint64), g2.liquid()["C"].view(np.uint64))


def test_bounded_wait_gives_up_with_the_timeout_bit():
    """The bounded mbarrier wait of the cycle kernels, on a barrier nothing
    completes, returns after its limit with BMC_ERR_TIMEOUT; the context
    stays usable (a wait that is satisfied returns at once)."""
    from bmc import _lib

    L = _lib.load()
    err, ns = ct.c_uint32(), ct.c_uint64()
    assert L.bmc_debug_wait(ct.c_uint64(50_000_000), 0, ct.byref(err), ct.byref(ns)) == 0
    assert err.value == 16  # BMC_ERR_TIMEOUT
    assert 50_000_000 <= ns.value < 1_000_000_000
    assert L.bmc_debug_wait(ct.c_uint64(50_000_000), 1, ct.byref(err), ct.byref(ns)) == 0
    assert err.value == 0 and ns.value < 50_000_000
    # a scenario still steps afterwards
    from bmc.sim import GpuScenario

    g = GpuScenario(scenarios.small_ring(2000, feeds=True))
    assert g.step()["error"] == 0


@pytest.mark.parametrize("n_c", [4, 5, 256, 257])
def test_scatter_forms_at_their_boundaries(oracle_mod, n_c):
    """Domains of 4 compartments (warp-aggregated scatter), 5 and 256
    (accumulator copies) and 257 (one accumulator): the same sums."""
    from test_gpu_parity import make_pair

    sc = scenarios.small_ring(6000, n_c=n_c, feeds=True, model=scenarios.overflow(f64=True))
    g, o = make_pair(oracle_mod, sc)
    _parity(g, o, 4, f"n_c={n_c}")


def test_reserve_grows_the_container_between_steps(oracle_mod):
    """A container too small for the births overflows; grown with
    bmc_reserve between steps (the reference's _resize on growth) it keeps
    its particles in place and stays equal to the CPU restatement grown the
    same way; the births then fit."""
    from test_gpu_parity import make_pair

    m = scenarios.monod(f64=True, m_div=1.0)  # every particle asks to divide
    sc = scenarios.zero_d(3000, model=m, outlet=False)
    g, o = make_pair(oracle_mod, sc, capacity=4096)
    assert g.cap == 4096 and o.cap == 4096
    gs, os_ = g.step(), o.step()
    assert gs["overflow"] == os_["overflow"] > 0  # 3000 requests, 1096 free slots
    before = g.particles()
    g.reserve(3 * 4096)
    o.reserve(3 * 4096)
    after = g.particles()
    for k in ("pos", "status", "id"):
        assert np.array_equal(before[k], after[k]), k
    assert np.array_equal(before["state"].view(np.uint64), after["state"].view(np.uint64))
    _parity(g, o, 3, "after reserve")
    assert g.stats()["n_used"] > 4096
