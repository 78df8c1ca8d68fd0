"""ctypes driver for the CPU restatement (oracle/bmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product.  It owns numpy arrays for
every buffer the C code reads or writes and mirrors the host-side set-up the
GPU library performs (weight, quantum exponents, feeds), so that both start
from identical inputs.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libbmc_oracle.so")

MAXO = 8


class OrcState(ct.Structure):
    _fields_ = [
        ("n_used", ct.c_uint64), ("phys_capacity", ct.c_uint64), ("inactive", ct.c_uint64),
        ("next_id", ct.c_uint64),
        ("state", ct.c_void_p), ("pos", ct.c_void_p), ("status", ct.c_void_p),
        ("age_h", ct.c_void_p), ("age_d", ct.c_void_p), ("id", ct.c_void_p),
        ("div_flag", ct.c_void_p), ("div_pos", ct.c_void_p), ("child_state", ct.c_void_p),
        ("child_pos", ct.c_void_p), ("gap_slot", ct.c_void_p), ("src_slot", ct.c_void_p),
        ("model", ct.c_int32), ("f64", ct.c_int32), ("n_var", ct.c_uint32), ("n_ctb", ct.c_uint32),
        ("params", ct.c_double * 16), ("weight", ct.c_double),
        ("n_c", ct.c_uint32), ("K", ct.c_uint32), ("n_s", ct.c_uint32),
        ("volume", ct.c_void_p), ("out_flow", ct.c_void_p), ("neighbors", ct.c_void_p),
        ("cdf", ct.c_void_p),
        ("n_outlets", ct.c_uint32), ("outlet_index", ct.c_uint32 * MAXO),
        ("outlet_flow", ct.c_double * MAXO), ("outlet_volume", ct.c_double * MAXO),
        ("C", ct.c_void_p), ("M", ct.c_void_p), ("src", ct.c_void_p), ("sink", ct.c_void_p),
        ("vinv", ct.c_void_p), ("in_ptr", ct.c_void_p), ("in_idx", ct.c_void_p),
        ("in_flow", ct.c_void_p),
        ("n_feeds", ct.c_uint32), ("feed_in", ct.c_uint32 * MAXO), ("feed_out", ct.c_int32 * MAXO),
        ("feed_flow", ct.c_double * MAXO), ("feed_conc", ct.c_double * (MAXO * 8)),
        ("draw_mode", ct.c_int32), ("seed", ct.c_uint64), ("step", ct.c_uint32),
        ("dead_ratio_threshold", ct.c_double), ("min_removal", ct.c_uint64),
        ("separable", ct.c_int32), ("q_exp", ct.c_int32 * 8), ("q_max", ct.c_int64),
        ("ctb_clamped", ct.c_uint64),
        ("quirk_tag3d", ct.c_int32),
        ("births", ct.c_uint64), ("exits", ct.c_uint64), ("moves", ct.c_uint64),
        ("overflow", ct.c_uint64), ("requested_divisions", ct.c_uint64),
        ("compacted", ct.c_int32), ("error", ct.c_int32),
        ("udf", ct.c_void_p),
        ("gas", ct.c_int32), ("gvinv", ct.c_void_p), ("g_in_ptr", ct.c_void_p),
        ("g_in_idx", ct.c_void_p), ("g_in_flow", ct.c_void_p), ("g_out_flow", ct.c_void_p),
        ("Cg", ct.c_void_p), ("Mg", ct.c_void_p), ("kla", ct.c_void_p), ("mtr", ct.c_void_p),
        ("henry", ct.c_double * 8), ("n_gfeeds", ct.c_uint32), ("gfeed_in", ct.c_uint32 * MAXO),
        ("gfeed_out", ct.c_int32 * MAXO), ("gfeed_flow", ct.c_double * MAXO),
        ("gfeed_conc", ct.c_double * (MAXO * 8)),
        ("feed_kind", ct.c_int32 * MAXO), ("feed_f0", ct.c_double * MAXO), ("feed_rate", ct.c_double * MAXO),
        ("t_rel", ct.c_double),
        ("probe_cap", ct.c_uint64), ("probe_buf", ct.c_void_p * 2), ("probe_n", ct.c_uint64 * 2),
    ]


class OrcUdfModel(ct.Structure):
    """orc_udf_model: a model library's host functions (bmc_udf_host_model)."""
    _fields_ = [("n_var", ct.c_uint32), ("n_ctb", ct.c_uint32), ("n_rates", ct.c_uint32),
                ("separable", ct.c_int32), ("rates", ct.c_void_p), ("update", ct.c_void_p),
                ("coef", ct.c_void_p), ("division", ct.c_void_p), ("init", ct.c_void_p),
                ("mass", ct.c_void_p), ("update_ctx", ct.c_void_p)]


def udf_host_model(path: str, f64: bool):
    """Open a model library and take its host entry points (host_model_udf);
    the library handle is returned with the table so it stays loaded."""
    L = ct.CDLL(path)
    f = L.host_model_udf
    f.argtypes = [ct.c_int32, ct.c_void_p]
    f.restype = ct.c_int
    m = OrcUdfModel()
    if f(1 if f64 else 0, ct.byref(m)) != 0:
        raise RuntimeError(f"{path}: precision not compiled in")
    return L, m


_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ct.CDLL(LIB_PATH)
        P = ct.POINTER(OrcState)
        L.orc_init_particles.argtypes = [P, ct.c_uint64, ct.c_uint32, ct.c_uint32]
        L.orc_total_mass.argtypes = [P]
        L.orc_total_mass.restype = ct.c_double
        L.orc_step.argtypes = [P, ct.c_double, ct.c_int]
        L.orc_run.argtypes = [P, ct.c_double, ct.c_uint32, ct.c_int]
        L.orc_cycle.argtypes = [P, ct.c_double, ct.c_int]
        L.orc_set_outlets.argtypes = [P]
        L.orc_post_cycle.argtypes = [P]
        L.orc_scalar_step.argtypes = [P, ct.c_double]
        L.orc_remove_inactive.argtypes = [P, ct.c_uint64]
        L.orc_find_next.argtypes = [P, ct.c_uint32, ct.c_double]
        L.orc_find_next.restype = ct.c_uint32
        L.orc_repartition.argtypes = [P, ct.c_void_p]
        L.orc_philox4x32_10.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_void_p]
        L.orc_draws.argtypes = [ct.c_uint64, ct.c_uint32, ct.c_uint32, ct.c_uint32, ct.c_void_p]
        L.orc_u01.argtypes = [ct.c_uint32]
        L.orc_u01.restype = ct.c_float
        L.orc_quantize.argtypes = [ct.c_double, ct.c_int32, ct.c_int64, ct.c_void_p]
        L.orc_quantize.restype = ct.c_int64
        for name in ("orc_sa_log", "orc_sa_exp", "orc_sa_erfinv"):
            getattr(L, name).argtypes = [ct.c_double]
            getattr(L, name).restype = ct.c_double
        L.orc_sa_truncnorm.argtypes = [ct.c_float] * 5
        L.orc_sa_truncnorm.restype = ct.c_float
        L.orc_particle_mass.argtypes = [P, ct.c_void_p]
        L.orc_probe_set.argtypes = [P, ct.c_int, ct.c_double]
        L.orc_probe_set.restype = ct.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def draws(seed: int, pid: int, step: int, purpose: int) -> np.ndarray:
    out = np.zeros(4, dtype=np.float32)
    lib().orc_draws(seed, pid, step, purpose, _ptr(out))
    return out


class Oracle:
    """One scenario on the CPU, laid out like the GPU container."""

    def __init__(self, scen, phys_capacity: int | None = None, draw_mode: int = 0,
                 quirk_tag3d: bool = False):
        self.scen = scen
        m = scen.model
        net = scen.net
        cap = phys_capacity or scen.capacity
        self.cap = cap
        ft = np.float64 if m.f64 else np.float32
        self.state = np.zeros(m.n_var * cap, dtype=ft)
        self.pos = np.zeros(cap, dtype=np.uint32)
        self.status = np.zeros(cap, dtype=np.uint8)
        self.age_h = np.zeros(cap, dtype=np.float32)
        self.age_d = np.zeros(cap, dtype=np.float32)
        self.id = np.zeros(cap, dtype=np.uint32)
        self.div_flag = np.zeros(cap, dtype=np.uint8)
        self.div_pos = np.zeros(cap, dtype=np.uint32)
        self.child_state = np.zeros(m.n_var * cap, dtype=ft)
        self.child_pos = np.zeros(cap, dtype=np.uint32)
        self.gap_slot = np.zeros(cap, dtype=np.uint32)
        self.src_slot = np.zeros(cap, dtype=np.uint32)
        ns = scen.n_species
        self.C = np.ascontiguousarray(scen.c0, dtype=np.float64).copy()
        self.vol = np.ascontiguousarray(net.volume, dtype=np.float64)
        self.vinv = 1.0 / self.vol
        self.M = (self.C * self.vol[:, None]).copy()
        self.src = np.zeros((net.n_c, ns))
        self.sink = np.zeros(net.n_c)
        self.out_flow = np.ascontiguousarray(net.out_flow, dtype=np.float64)
        self.neighbors = np.ascontiguousarray(net.neighbors, dtype=np.uint32)
        self.cdf = np.ascontiguousarray(net.cdf, dtype=np.float64)
        self.in_ptr = np.ascontiguousarray(net.in_ptr, dtype=np.uint32)
        self.in_idx = np.ascontiguousarray(net.in_idx, dtype=np.uint32)
        self.in_flow = np.ascontiguousarray(net.in_flow, dtype=np.float64)

        s = OrcState()
        s.phys_capacity = cap
        for name in ("state", "pos", "status", "age_h", "age_d", "id", "div_flag", "div_pos",
                     "child_state", "child_pos", "gap_slot", "src_slot", "C", "M", "src",
                     "sink", "vinv", "in_ptr", "in_idx", "in_flow", "neighbors", "cdf",
                     "out_flow"):
            setattr(s, name, _ptr(getattr(self, name)))
        s.volume = _ptr(self.vol)
        s.model = m.model_id
        s.f64 = 1 if m.f64 else 0
        s.n_var = m.n_var
        s.n_ctb = m.n_ctb
        for k in range(16):
            s.params[k] = float(m.params[k])
        s.n_c = net.n_c
        s.K = net.K
        s.n_s = ns
        s.n_feeds = len(scen.feeds)
        for f, fd in enumerate(scen.feeds):
            s.feed_in[f] = fd.inlet
            s.feed_out[f] = fd.outlet
            s.feed_flow[f] = fd.flow
            for sp in range(ns):
                s.feed_conc[f * 8 + sp] = float(fd.conc[sp])
            s.feed_kind[f] = getattr(fd, "kind", 0)
            s.feed_f0[f] = float(getattr(fd, "f0", 0.0))
            s.feed_rate[f] = float(getattr(fd, "rate", 0.0))
        s.draw_mode = draw_mode
        s.seed = scen.seed
        s.step = 0
        s.dead_ratio_threshold = scen.dead_ratio_threshold
        s.min_removal = scen.min_removal
        from bmc.scenarios import CTB_QMAX

        s.q_max = CTB_QMAX
        s.separable = 1 if m.separable else 0
        s.quirk_tag3d = 1 if quirk_tag3d else 0
        self._udf = None
        if getattr(m, "udf_path", None):
            self._udf = udf_host_model(m.udf_path, m.f64)
            assert self._udf[1].n_var == m.n_var and self._udf[1].n_ctb == m.n_ctb
            s.udf = ct.addressof(self._udf[1])
        if scen.gas is not None:
            self._setup_gas(s, scen.gas)
        self.s = s
        self.weight = None
        self._map_arrays = {}
        # no flow map applied yet: the first step applies map 0, as the
        # device's first switch does (its gas state included)
        self._map_cur = -1

    def _setup_gas(self, s, gas):
        """Gas phase arrays (kept alive on the object) and feeds."""
        gn = gas.net
        ns = self.scen.n_species
        self.gvol = np.ascontiguousarray(gn.volume, dtype=np.float64)
        self.gvinv = 1.0 / self.gvol
        self.g_in_ptr = np.ascontiguousarray(gn.in_ptr, dtype=np.uint32)
        self.g_in_idx = np.ascontiguousarray(gn.in_idx, dtype=np.uint32)
        self.g_in_flow = np.ascontiguousarray(gn.in_flow, dtype=np.float64)
        self.g_out_flow = np.ascontiguousarray(gn.out_flow, dtype=np.float64)
        self.Cg = np.ascontiguousarray(gas.c0, dtype=np.float64).copy()
        self.Mg = (self.Cg * self.gvol[:, None]).copy()
        self.kla = np.ascontiguousarray(gas.kla, dtype=np.float64)
        self.mtr = np.zeros_like(self.Cg)
        s.gas = 1
        for name in ("gvinv", "g_in_ptr", "g_in_idx", "g_in_flow", "g_out_flow", "Cg", "Mg", "kla", "mtr"):
            setattr(s, name, _ptr(getattr(self, name)))
        for sp in range(min(ns, 8)):
            s.henry[sp] = float(gas.henry[sp])
        s.n_gfeeds = len(gas.feeds)
        for f, fd in enumerate(gas.feeds):
            s.gfeed_in[f] = fd.inlet
            s.gfeed_out[f] = fd.outlet
            s.gfeed_flow[f] = fd.flow
            for sp in range(ns):
                s.gfeed_conc[f * 8 + sp] = float(fd.conc[sp])

    def reserve(self, capacity: int):
        """Grow the container to `capacity` slots keeping the live particles
        in their slots (the restatement of ParticlesContainer::_resize on
        growth, particles_container.hpp L603-L650)."""
        if capacity <= self.cap:
            return
        n = int(self.s.n_used)
        m = self.scen.model
        old_cap, cap = self.cap, capacity
        st = self.state.reshape(m.n_var, old_cap)
        new_state = np.zeros(m.n_var * cap, dtype=self.state.dtype)
        new_state.reshape(m.n_var, cap)[:, :n] = st[:, :n]
        self.state = new_state
        for name in ("pos", "status", "age_h", "age_d", "id"):
            a = getattr(self, name)
            b = np.zeros(cap, dtype=a.dtype)
            b[:n] = a[:n]
            setattr(self, name, b)
        for name in ("div_flag", "div_pos", "child_pos", "gap_slot", "src_slot"):
            setattr(self, name, np.zeros(cap, dtype=getattr(self, name).dtype))
        self.child_state = np.zeros(m.n_var * cap, dtype=self.state.dtype)
        for name in ("state", "pos", "status", "age_h", "age_d", "id", "div_flag", "div_pos",
                     "child_state", "child_pos", "gap_slot", "src_slot"):
            setattr(self.s, name, _ptr(getattr(self, name)))
        self.s.phys_capacity = cap
        self.cap = cap

    # -- set-up --------------------------------------------------------------
    def init_particles(self, n: int | None = None):
        n = self.scen.n_particles if n is None else n
        hi = self.scen.net.n_c if self.scen.uniform_init else 1
        lib().orc_init_particles(ct.byref(self.s), n, 0, hi)
        mass = lib().orc_total_mass(ct.byref(self.s))
        from bmc.scenarios import weight_from_mass
        self.set_weight(weight_from_mass(mass, self.scen.x0, self.scen.net.total_volume))
        return self.weight

    def set_weight(self, w: float):
        self.weight = w
        self.s.weight = w
        e = self.scen.quantum_exponents(w)
        for j in range(8):
            self.s.q_exp[j] = int(e[j])

    # -- flow-map cycle -----------------------------------------------------------
    def _use_map(self, m: int):
        """Point the domain at flow-map state m: volumes, out-flows,
        neighbours, cumulative probabilities, incoming flows, outlet
        volumes; masses are kept, so concentrations follow at the next
        liquid step (the reference's updateHydro + ScalarSimulation::
        setVolumes, apps/libs/simulation/src/simulation.cpp L95-L139)."""
        net = self.scen.flowmaps[m]
        keep = self._map_arrays.setdefault(m, {
            "volume": np.ascontiguousarray(net.volume, dtype=np.float64),
            "vinv": 1.0 / np.ascontiguousarray(net.volume, dtype=np.float64),
            "out_flow": np.ascontiguousarray(net.out_flow, dtype=np.float64),
            "neighbors": np.ascontiguousarray(net.neighbors, dtype=np.uint32),
            "cdf": np.ascontiguousarray(net.cdf, dtype=np.float64),
            "in_ptr": np.ascontiguousarray(net.in_ptr, dtype=np.uint32),
            "in_idx": np.ascontiguousarray(net.in_idx, dtype=np.uint32),
            "in_flow": np.ascontiguousarray(net.in_flow, dtype=np.float64),
        })
        for name, arr in keep.items():
            setattr(self.s, name, _ptr(arr))
        gas = self.scen.gas
        if gas is not None and gas.flowmaps:
            # the map's gas state (SimulationUnit::updateScalarHydro and
            # MassTransferModel::update): volumes, transition, kla; the gas
            # masses are kept
            gn = gas.flowmaps[m]
            gkeep = self._map_arrays.setdefault(("gas", m), {
                "gvinv": 1.0 / np.ascontiguousarray(gn.volume, dtype=np.float64),
                "g_in_ptr": np.ascontiguousarray(gn.in_ptr, dtype=np.uint32),
                "g_in_idx": np.ascontiguousarray(gn.in_idx, dtype=np.uint32),
                "g_in_flow": np.ascontiguousarray(gn.in_flow, dtype=np.float64),
                "g_out_flow": np.ascontiguousarray(gn.out_flow, dtype=np.float64),
                "kla": np.ascontiguousarray(gas.kla_maps[m] if gas.kla_maps else gas.kla, dtype=np.float64),
            })
            for name, arr in gkeep.items():
                setattr(self.s, name, _ptr(arr))
        for o in range(self.s.n_outlets):
            self.s.outlet_volume[o] = float(keep["volume"][self.s.outlet_index[o]])
        self.vol, self.vinv = keep["volume"], keep["vinv"]
        self._map_cur = m

    def _switch_map(self):
        fm = self.scen.flowmaps
        if not fm:
            return
        m = (int(self.s.step) // self.scen.n_per_flowmap) % len(fm)
        if m != self._map_cur:
            self._use_map(m)

    # -- stepping -------------------------------------------------------------
    def step(self, n_threads: int = 1):
        self._switch_map()
        lib().orc_step(ct.byref(self.s), self.scen.dt, n_threads)
        return self.stats()

    def run(self, n_steps: int, n_threads: int = 1):
        if self.scen.flowmaps:  # the map switch runs between steps
            for _ in range(n_steps):
                self.step(n_threads)
            return
        lib().orc_run(ct.byref(self.s), self.scen.dt, n_steps, n_threads)

    def cycle(self, n_threads: int = 1):
        """cycleProcess alone: leaving flows from the feeds' outlets, then the
        cycle (no liquid step, no feed sources)."""
        lib().orc_set_outlets(ct.byref(self.s))
        lib().orc_cycle(ct.byref(self.s), self.scen.dt, n_threads)

    def post_cycle(self):
        lib().orc_post_cycle(ct.byref(self.s))

    def stats(self) -> dict:
        s = self.s
        return dict(n_used=s.n_used, inactive=s.inactive, births=s.births, exits=s.exits,
                    moves=s.moves, overflow=s.overflow, compacted=s.compacted,
                    error=s.error, next_id=s.next_id, clamped=s.ctb_clamped)

    # -- views ----------------------------------------------------------------
    @property
    def n_used(self) -> int:
        return int(self.s.n_used)

    def particles(self) -> dict:
        n = self.n_used
        m = self.scen.model
        st = self.state.reshape(m.n_var, self.cap)[:, :n].copy()
        return dict(state=st, pos=self.pos[:n].copy(), status=self.status[:n].copy(),
                    age_h=self.age_h[:n].copy(), age_d=self.age_d[:n].copy(),
                    id=self.id[:n].copy())

    def repartition(self) -> np.ndarray:
        out = np.zeros(self.scen.net.n_c, dtype=np.uint64)
        lib().orc_repartition(ct.byref(self.s), _ptr(out))
        return out

    def mass(self) -> np.ndarray:
        """Model::mass of every used slot."""
        out = np.zeros(max(self.n_used, 1))
        lib().orc_particle_mass(ct.byref(self.s), _ptr(out))
        return out[:self.n_used]

    def force_remove_dead(self):
        """Every non-Idle particle removed (gap filling in slot order)."""
        inactive = int(np.count_nonzero(self.status[:self.n_used] != 0))
        self.s.inactive = inactive
        lib().orc_remove_inactive(ct.byref(self.s), inactive)

    # -- time-event probes (0: leaving times, 1: division times) ---------------
    def probe_enable(self, capacity: int):
        self._probe = [np.zeros(max(capacity, 1)), np.zeros(max(capacity, 1))]
        self.s.probe_cap = capacity
        for k in range(2):
            self.s.probe_buf[k] = _ptr(self._probe[k])
            self.s.probe_n[k] = 0

    def probe_set(self, probe: int, value: float) -> bool:
        """Probes::set: counts the event, stores the value while there is room."""
        return bool(lib().orc_probe_set(ct.byref(self.s), probe, value))

    def probe_read(self, probe: int) -> tuple[np.ndarray, int]:
        """(stored values, events counted) of one probe."""
        n = int(self.s.probe_n[probe])
        return self._probe[probe][:min(n, int(self.s.probe_cap))].copy(), n

    def probe_clear(self, probe: int):
        self._probe[probe][:] = 0.0
        self.s.probe_n[probe] = 0
