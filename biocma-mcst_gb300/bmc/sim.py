"""Host-side mirror of the reference's simulation-core objects for this path.

``GpuScenario`` plays the role of SimulationUnit + ParticlesContainer +
ReactorDomain + ScalarSimulation (apps/libs/simulation/public/simulation/
simulation.hpp; apps/libs/mc/public/mc/particles_container.hpp): it creates
a libbmc scenario from a :class:`bmc.scenarios.Scenario`, uploads the
domain, transition, concentrations and feeds, initialises the particles
and exposes cycleProcess / one main-loop step / n steps.  Every call goes
through the C-ABI; nothing here computes the cycle.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from ._lib import Feed, ScenarioDesc, StepStats, call

# the reference's MC::EventType order (events.hpp L17-L26)
EVENTS = ("NewParticle", "Exit", "Move", "Death", "Overflow", "ChangeWeight")


def _p(a: np.ndarray):
    return ct.c_void_p(a.ctypes.data)


def scenario_desc(scen, capacity: int | None = None) -> ScenarioDesc:
    m = scen.model
    d = ScenarioDesc()
    d.model.model = m.model_id
    d.model.f64 = 1 if m.f64 else 0
    d.model.n_var = m.n_var
    d.model.n_ctb = m.n_ctb
    for k in range(16):
        d.model.params[k] = float(m.params[k])
    d.n_species = scen.n_species
    d.capacity = capacity or scen.capacity
    d.seed = scen.seed
    d.dead_ratio_threshold = scen.dead_ratio_threshold
    d.min_removal = scen.min_removal
    for j in range(len(m.value_bound)):
        d.value_bound[j] = float(m.value_bound[j])
    return d


def transition_coo(net):
    """COO of the transition matrix: off-diagonal F(i->j), diagonal -Q_out."""
    rows = np.concatenate([net.src, np.arange(net.n_c)]).astype(np.uint64)
    cols = np.concatenate([net.dst, np.arange(net.n_c)]).astype(np.uint64)
    vals = np.concatenate([net.flow, -net.out_flow]).astype(np.float64)
    return rows, cols, vals


class GpuScenario:
    def __init__(self, scen, capacity: int | None = None, init: bool = True,
                 n_particles: int | None = None):
        self.scen = scen
        self.lib = _lib.load()
        self.handle = ct.c_void_p()
        desc = scenario_desc(scen, capacity)
        call("bmc_scenario_create", ct.byref(desc), ct.byref(self.handle))
        self.cap = (int(desc.capacity) + 1023) // 1024 * 1024  # slots, rounded to whole tiles
        net = scen.net
        vol = np.ascontiguousarray(net.volume, dtype=np.float64)
        nbr = np.ascontiguousarray(net.neighbors, dtype=np.uint64)
        outf = np.ascontiguousarray(net.out_flow, dtype=np.float64)
        cdf = np.ascontiguousarray(net.cdf, dtype=np.float64)
        call("bmc_domain_update", self.handle, net.n_c, net.K, _p(vol), _p(nbr), _p(outf), _p(cdf))
        r, c, v = transition_coo(net)
        call("bmc_set_transition_coo", self.handle, net.n_c, len(v), _p(r), _p(c), _p(v))
        c0 = np.ascontiguousarray(scen.c0, dtype=np.float64)
        call("bmc_set_concentrations", self.handle, _p(c0))
        if scen.feeds:
            arr = (Feed * len(scen.feeds))()
            for k, fd in enumerate(scen.feeds):
                arr[k].inlet = fd.inlet
                arr[k].outlet = fd.outlet
                arr[k].flow = fd.flow
                for sp in range(len(fd.conc)):
                    arr[k].conc[sp] = float(fd.conc[sp])
            call("bmc_set_feeds", self.handle, len(scen.feeds), arr)
            if any(fd.kind != 0 for fd in scen.feeds):
                self.set_feed_schedules(scen.feeds)
        if scen.gas is not None:
            self.set_gas(scen.gas)
        for fm in scen.flowmaps:
            self.add_flowmap(fm)
        if scen.gas is not None:
            for k, gnet in enumerate(scen.gas.flowmaps):
                self.add_flowmap_gas(k, gnet, scen.gas.kla_maps[k] if scen.gas.kla_maps else None)
        if scen.flowmaps:
            call("bmc_flowmap_period", self.handle, scen.t_per_flowmap)
        self.weight = None
        if init:
            self.init_particles(n_particles)

    def close(self):
        if self.handle:
            _lib.load().bmc_scenario_destroy(self.handle)
            self.handle = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ---------------------------------------------------------------
    def init_particles(self, n: int | None = None) -> float:
        n = self.scen.n_particles if n is None else n
        w = ct.c_double()
        call("bmc_init_particles", self.handle, n, 1 if self.scen.uniform_init else 0,
             self.scen.x0, ct.byref(w))
        self.weight = w.value
        return self.weight

    def set_feed_schedules(self, feeds):
        """bmc_set_feed_schedules from the kind / f0 / rate of each Feed."""
        arr = (_lib.FeedSchedule * len(feeds))()
        for k, fd in enumerate(feeds):
            arr[k].kind, arr[k].f0, arr[k].rate = fd.kind, fd.f0, fd.rate
        call("bmc_set_feed_schedules", self.handle, len(feeds), arr)

    def feed_time(self) -> float:
        t = ct.c_double()
        call("bmc_feed_time", self.handle, ct.byref(t))
        return t.value

    def set_weight(self, w: float):
        call("bmc_set_weight", self.handle, w)
        self.weight = w

    def set_gas(self, gas):
        """Two-phase flow: gas volumes, transition, Henry, kla, initial
        concentrations and feeds (bmc_gas_*)."""
        vol = np.ascontiguousarray(gas.net.volume, dtype=np.float64)
        r, c, v = transition_coo(gas.net)
        henry = np.zeros(8)
        henry[: len(gas.henry)] = gas.henry
        kla = np.ascontiguousarray(gas.kla, dtype=np.float64)
        call("bmc_gas_set", self.handle, _p(vol), len(v), _p(r), _p(c), _p(v), _p(henry), _p(kla))
        call("bmc_gas_set_concentrations", self.handle, _p(np.ascontiguousarray(gas.c0, dtype=np.float64)))
        if gas.feeds:
            arr = (Feed * len(gas.feeds))()
            for k, fd in enumerate(gas.feeds):
                arr[k].inlet = fd.inlet
                arr[k].outlet = fd.outlet
                arr[k].flow = fd.flow
                for sp in range(len(fd.conc)):
                    arr[k].conc[sp] = float(fd.conc[sp])
            call("bmc_gas_set_feeds", self.handle, len(gas.feeds), arr)

    def gas(self) -> dict:
        n, ns = self.scen.net.n_c, self.scen.n_species
        out = {k: np.zeros((n, ns)) for k in ("Cg", "Mg", "mtr")}
        call("bmc_gas_read", self.handle, _p(out["Cg"]), _p(out["Mg"]), _p(out["mtr"]))
        return out

    def add_flowmap(self, net):
        """Append a flow-map state of the same mesh (bmc_flowmap_add)."""
        vol = np.ascontiguousarray(net.volume, dtype=np.float64)
        nbr = np.ascontiguousarray(net.neighbors, dtype=np.uint64)
        outf = np.ascontiguousarray(net.out_flow, dtype=np.float64)
        cdf = np.ascontiguousarray(net.cdf, dtype=np.float64)
        r, c, v = transition_coo(net)
        call("bmc_flowmap_add", self.handle, _p(vol), _p(nbr), _p(outf), _p(cdf), len(v), _p(r), _p(c), _p(v))

    def add_flowmap_gas(self, map_index: int, gnet, kla=None):
        """Gas state of flow map `map_index` (bmc_flowmap_add_gas): gas
        volumes and transition of `gnet`, kla [n_c, n_s] (None: the gas
        phase's)."""
        vol = np.ascontiguousarray(gnet.volume, dtype=np.float64)
        r, c, v = transition_coo(gnet)
        k = None if kla is None else np.ascontiguousarray(kla, dtype=np.float64)
        call("bmc_flowmap_add_gas", self.handle, map_index, _p(vol), len(v), _p(r), _p(c), _p(v),
             None if k is None else _p(k))

    def set_shape(self, threads: int = 0, ppt: int = 0, blocks_per_sm: int = 0):
        call("bmc_set_shape", self.handle, threads, ppt, blocks_per_sm)

    def set_step_limit(self, limit: int):
        """Steps become no-ops once the step counter reaches `limit` (0: none)."""
        call("bmc_set_step_limit", self.handle, limit)

    def set_particles(self, parts: dict, next_id: int):
        m = self.scen.model
        ft = np.float64 if m.f64 else np.float32
        st = np.ascontiguousarray(parts["state"], dtype=ft)
        n = st.shape[1]
        arrs = [np.ascontiguousarray(parts[k], dtype=t) for k, t in
                (("pos", np.uint32), ("status", np.uint8), ("age_h", np.float32),
                 ("age_d", np.float32), ("id", np.uint32))]
        call("bmc_set_particles", self.handle, n, _p(st), *[_p(a) for a in arrs], next_id)

    # -- stepping ---------------------------------------------------------------
    def cycle(self, dt: float | None = None) -> dict:
        st = StepStats()
        call("bmc_cycle", self.handle, dt or self.scen.dt, ct.byref(st))
        return st.as_dict()

    def cycle_external(self, conc, sources=None, dt: float | None = None) -> tuple:
        """bmc_cycle_external: concentrations in, contributions out.  numpy
        arrays use host pointers; objects with a `data_ptr()` (device
        tensors) are passed as device pointers."""
        dt = self.scen.dt if dt is None else dt
        st = StepStats()
        if hasattr(conc, "data_ptr"):
            call("bmc_cycle_external", self.handle, dt, ct.c_void_p(conc.data_ptr()),
                 ct.c_void_p(sources.data_ptr()), 1, ct.byref(st))
            return sources, st.as_dict()
        c = np.ascontiguousarray(conc, dtype=np.float64)
        out = np.zeros_like(c) if sources is None else sources
        call("bmc_cycle_external", self.handle, dt, _p(c), _p(out), 0, ct.byref(st))
        return out, st.as_dict()

    def step(self, dt: float | None = None) -> dict:
        st = StepStats()
        call("bmc_step", self.handle, dt or self.scen.dt, ct.byref(st))
        return st.as_dict()

    def reserve(self, capacity: int):
        """Grow the container to at least `capacity` slots (bmc_reserve)."""
        call("bmc_reserve", self.handle, int(capacity))
        self.cap = max(self.cap, (int(capacity) + 1023) // 1024 * 1024)

    def step_read(self, conc: np.ndarray, dt: float | None = None) -> dict:
        """One step; the concentrations after it are written into `conc`
        (float64 [n_c, n_species], C-contiguous) in the same synchronisation."""
        n = self.scen.net.n_c * self.scen.n_species
        if conc.dtype != np.float64 or not conc.flags.c_contiguous or conc.size != n:
            raise ValueError(f"conc must be a C-contiguous float64 array of {n} values")
        st = StepStats()
        call("bmc_step_read", self.handle, dt or self.scen.dt, ct.byref(st), _p(conc))
        return st.as_dict()

    def step_enqueue(self, stats, conc: np.ndarray, dt: float | None = None):
        """bmc_step_enqueue: one step and the read-back of its counters into
        `stats` (a StepStats) and concentrations into `conc` (float64
        [n_c, n_species], C-contiguous), filled by the matching
        step_collect; the buffers must stay alive until then."""
        n = self.scen.net.n_c * self.scen.n_species
        if conc.dtype != np.float64 or not conc.flags.c_contiguous or conc.size != n:
            raise ValueError(f"conc must be a C-contiguous float64 array of {n} values")
        call("bmc_step_enqueue", self.handle, dt or self.scen.dt, ct.byref(stats), _p(conc))

    def step_collect(self):
        call("bmc_step_collect", self.handle)

    def step_timed(self, dt: float | None = None):
        """One step with per-kernel CUDA-event durations (ms): liquid, cycle,
        plan, divide, compact, merge."""
        st = StepStats()
        ms = (ct.c_float * 6)()
        call("bmc_step_timed", self.handle, dt or self.scen.dt, ct.byref(st), ms)
        return st.as_dict(), list(ms)

    def run(self, n_steps: int, dt: float | None = None) -> dict:
        st = StepStats()
        call("bmc_run", self.handle, dt or self.scen.dt, n_steps, ct.byref(st))
        return st.as_dict()

    def run_timed(self, n_steps: int, dt: float | None = None):
        """n_steps graph-replayed steps; device time (ms) from CUDA events
        recorded on the scenario's own stream around them."""
        st = StepStats()
        ms = ct.c_float()
        call("bmc_run_timed", self.handle, dt or self.scen.dt, n_steps, ct.byref(st), ct.byref(ms))
        return st.as_dict(), ms.value

    def run_async(self, n_steps: int, dt: float | None = None):
        call("bmc_run_async", self.handle, dt or self.scen.dt, n_steps)

    def synchronize(self):
        call("bmc_synchronize", self.handle)

    def stats(self) -> dict:
        st = StepStats()
        call("bmc_read_stats", self.handle, ct.byref(st))
        return st.as_dict()

    # -- readback -----------------------------------------------------------------
    def mass(self) -> np.ndarray:
        """Model::mass of each used slot, computed on the device."""
        n = self.stats()["n_used"]
        out = np.zeros(max(n, 1), dtype=np.float64)
        got = ct.c_uint64()
        call("bmc_read_mass", self.handle, max(n, 1), _p(out), ct.byref(got))
        return out[:got.value]

    def particles(self) -> dict:
        n = self.stats()["n_used"]
        m = self.scen.model
        ft = np.float64 if m.f64 else np.float32
        st = np.zeros((m.n_var, max(n, 1)), dtype=ft)
        pos = np.zeros(max(n, 1), np.uint32)
        status = np.zeros(max(n, 1), np.uint8)
        ah = np.zeros(max(n, 1), np.float32)
        ad = np.zeros(max(n, 1), np.float32)
        pid = np.zeros(max(n, 1), np.uint32)
        got = ct.c_uint64()
        call("bmc_read_particles", self.handle, max(n, 1), _p(st), _p(pos), _p(status), _p(ah),
             _p(ad), _p(pid), ct.byref(got))
        n = got.value
        return dict(state=st[:, :n], pos=pos[:n], status=status[:n], age_h=ah[:n], age_d=ad[:n],
                    id=pid[:n])

    def liquid(self) -> dict:
        shape = (self.scen.net.n_c, self.scen.n_species)
        C = np.zeros(shape)
        M = np.zeros(shape)
        S = np.zeros(shape)
        call("bmc_read_liquid", self.handle, _p(C), _p(M), _p(S))
        return dict(C=C, M=M, src=S)

    def repartition(self) -> np.ndarray:
        out = np.zeros(self.scen.net.n_c, dtype=np.uint64)
        call("bmc_repartition", self.handle, _p(out))
        return out

    def force_remove_dead(self):
        call("bmc_force_remove_dead", self.handle)

    def events(self, clear: bool = False) -> dict:
        """Event tallies since the last clear (EVENTS order, include/bmc.h)."""
        out = np.zeros(len(EVENTS), dtype=np.uint64)
        call("bmc_read_events", self.handle, _p(out), 1 if clear else 0)
        return {k: int(v) for k, v in zip(EVENTS, out)}

    # time-event probes: 0 leaving times, 1 division times (include/bmc.h)
    def probe_enable(self, capacity: int):
        call("bmc_probe_enable", self.handle, capacity)
        self.probe_capacity = capacity

    def probe_read(self, probe: int) -> tuple[np.ndarray, int]:
        """(stored values, events counted) of one probe."""
        cap = getattr(self, "probe_capacity", 0)
        out = np.zeros(max(cap, 1), dtype=np.float64)
        n = ct.c_uint64()
        call("bmc_probe_read", self.handle, probe, _p(out), cap, ct.byref(n))
        return out[:min(cap, n.value)].copy(), int(n.value)

    def probe_clear(self, probe: int):
        call("bmc_probe_clear", self.handle, probe)


def debug_draws(seed: int, ids: np.ndarray, step: int, purpose: int) -> np.ndarray:
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    out = np.zeros((len(ids), 4), dtype=np.float32)
    call("bmc_debug_draws", seed, _p(ids), len(ids), step, purpose, _p(out))
    return out


def transfer_bytes() -> tuple[int, int]:
    h, d = ct.c_uint64(), ct.c_uint64()
    call("bmc_transfer_bytes", ct.byref(h), ct.byref(d))
    return h.value, d.value


def set_device(device: int):
    call("bmc_set_device", device)


def launch_count() -> int:
    v = ct.c_uint64()
    call("bmc_launch_count", ct.byref(v))
    return v.value


class GpuBatch:
    """Many scenarios advanced by one set of launches per step."""

    def __init__(self, scenarios: list[GpuScenario]):
        self.members = scenarios
        arr = (ct.c_void_p * len(scenarios))(*[s.handle.value for s in scenarios])
        self.handle = ct.c_void_p()
        call("bmc_batch_create", arr, len(scenarios), ct.byref(self.handle))

    @classmethod
    def slots(cls, capacity: int, model) -> "GpuBatch":
        """An empty batch of `capacity` slots for `model` (a ModelSpec)."""
        b = cls.__new__(cls)
        b.members = [None] * capacity
        b.handle = ct.c_void_p()
        call("bmc_batch_create_slots", capacity, model.model_id, 1 if model.f64 else 0, ct.byref(b.handle))
        return b

    def set_slot(self, slot: int, scenario: GpuScenario | None):
        call("bmc_batch_set_slot", self.handle, slot, None if scenario is None else scenario.handle)
        self.members[slot] = scenario

    def set_shape(self, threads: int = 0, ppt: int = 0, blocks_per_sm: int = 0):
        call("bmc_batch_set_shape", self.handle, threads, ppt, blocks_per_sm)

    def run(self, n_steps: int, dt: float):
        call("bmc_batch_run", self.handle, dt, n_steps)

    def step_timed(self, dt: float) -> np.ndarray:
        """One step with per-kernel device times (ms): liquid, cycle, plan,
        divide, compact, merge."""
        ms = np.zeros(6, dtype=np.float32)
        call("bmc_batch_step_timed", self.handle, dt, _p(ms))
        return ms

    def synchronize(self):
        call("bmc_batch_synchronize", self.handle)

    def close(self):
        if self.handle:
            _lib.load().bmc_batch_destroy(self.handle)
            self.handle = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
