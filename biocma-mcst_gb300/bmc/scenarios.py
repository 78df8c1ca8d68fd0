"""Scenario descriptions: network + cell model + liquid state + feeds.

A :class:`Scenario` is plain data (numpy arrays); both the GPU library and
the CPU oracle are set up from the same object, so they see identical inputs.
The five workloads of the benchmark are built by :func:`workload`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .networks import Network, lattice_vortex, ring_network, single_compartment

MODEL_MONOD = 1
MODEL_OVERFLOW = 2
MODEL_FIXED_LENGTH = 3
MODEL_FIXED_LENGTH_GENERAL = 4
MODEL_SIMPLE_ACETATE = 5

MU_MAX = 0.77 / 3600.0  # 1/s


@dataclass
class ModelSpec:
    """Cell model as the ModelType concept describes it (n_var, n_c, FloatType)."""

    name: str
    model_id: int
    n_var: int
    n_ctb: int
    f64: bool
    params: np.ndarray  # float64[16]
    # separable models: [bound on |basis|]; general models: bound on
    # |contribution j| of one particle
    value_bound: np.ndarray
    separable: bool = True
    read_vars: int = 2  # state variables the update reads (the others are outputs)
    udf_path: str | None = None  # model library (runtime-loaded model) it comes from
    # variables of the particle dump (Model::names with get_number, the
    # reference's partial export) and their state indices; the mass column
    # is added by the exporter
    export_names: tuple = ()
    export_index: tuple = ()
    species: tuple = ()  # liquid scalar names (the exporter's misc/species_names)

    @property
    def itemsize(self) -> int:
        return 8 if self.f64 else 4


def monod(f64: bool = True, mu_max: float = MU_MAX, ks: float = 0.01, y: float = 0.5,
          m_div: float = 2.0, m_lo: float = 0.9, m_span: float = 0.2) -> ModelSpec:
    p = np.zeros(16)
    p[:6] = [mu_max, ks, y, m_div, m_lo, m_span]
    # contribution = -(mu / Y) * mass: the basis is the particle mass
    return ModelSpec("monod", MODEL_MONOD, 2, 1, f64, p, np.array([4.0 * m_div]),
                     export_names=("cycle_time",), export_index=(1,), species=("glucose",))


def overflow(f64: bool = True, mu_max: float = MU_MAX) -> ModelSpec:
    y_ox, y_of, y_ac, y_o, y_c, y_cof = 0.5, 0.15, 0.6, 0.6, 0.7, 0.3
    qs_max = mu_max / y_ox
    qo_max = 0.7 * qs_max
    m_div = 2.0
    p = np.zeros(16)
    p[:13] = [qs_max, 0.01, qo_max, 1e-4, y_ox, y_of, y_ac, y_o, y_c, m_div, y_cof, 0.9, 0.2]
    # every contribution is a rate of the compartment times the mass
    return ModelSpec("overflow", MODEL_OVERFLOW, 6, 4, f64, p, np.array([4.0 * m_div]),
                     export_names=("cycle_time", "mu", "q_s", "q_o2", "q_ac"), export_index=(1, 2, 3, 4, 5),
                     species=("glucose", "O2", "acetate", "CO2"))


def fixed_length(general: bool = False) -> ModelSpec:
    """The reference's FixedLength model (float state, one contribution).
    ``general`` runs it through the per-particle contribution path."""
    l_dot_max = np.float32(2e-6 / 3600.0)
    d_m = np.float32(0.6e-6)
    lin = np.float32(1000) * np.float32(math.pi) * d_m * d_m / np.float32(4.0)
    phi = float((l_dot_max * lin) / np.float32(0.5))
    p = np.zeros(16)
    if general:
        return ModelSpec("fixed_length_general", MODEL_FIXED_LENGTH_GENERAL, 2, 1, False, p,
                         np.array([4.0 * phi]), separable=False, export_names=("length",), export_index=(0,),
                         species=("glucose",))
    # contribution = -phi_s(C) per particle: basis 1; the dump exports the
    # length only (get_number, fixed_length.hpp L84-L97)
    return ModelSpec("fixed_length", MODEL_FIXED_LENGTH, 2, 1, False, p, np.array([1.0]),
                     export_names=("length",), export_index=(0,), species=("glucose",))


def simple_acetate() -> ModelSpec:
    """The reference's SimpleAcetate model: float state of 9 variables
    (length, l_max, a_p, a_max, a_e, a_e_s, a_e_a, phi_s, phi_a), glucose and
    acetate, two contributions per particle (general path), log-normal and
    truncated-normal draws at division."""
    a_max = np.float32(2e-6 / 3600.0)
    d_m = np.float32(0.6e-6)
    lin = np.float32(1000) * np.float32(math.pi) * d_m * d_m / np.float32(4.0)
    # |phi_s| <= a_max * lin * y_s, |phi_a| <= a_max * lin * max(1, y_s / y_a)
    bound = 4.0 * float(a_max) * float(lin) * 2.0
    p = np.zeros(16)
    return ModelSpec("simple_acetate", MODEL_SIMPLE_ACETATE, 9, 2, False, p, np.array([bound, bound]),
                     separable=False, read_vars=4,
                     export_names=("length", "l_max", "a_p", "a_max", "a_e", "a_e_s", "a_e_a", "phi_s", "phi_a"),
                     export_index=tuple(range(9)), species=("glucose", "acetate"))


FEED_CONSTANT = 0
FEED_LINEAR = 1
FEED_EXPONENTIAL = 2


@dataclass
class Feed:
    """A liquid feed (Simulation::Feed::FeedDescriptor): inlet, optional
    outlet, flow and inlet concentrations; kind selects the flow's time
    dependence: constant (`flow`), linear f0 + t * rate, or exponential
    f0 + exp(rate * t) at the relative time t."""
    inlet: int
    outlet: int  # -1 when the feed has no outlet
    flow: float  # m^3/s
    conc: np.ndarray  # kg/m^3 per species
    kind: int = FEED_CONSTANT
    f0: float = 0.0
    rate: float = 0.0


@dataclass
class GasPhase:
    """Gas phase of a two-phase scenario on the same mesh: gas flows and
    volumes (a Network), Henry constants per species, transfer coefficients
    kla [n_c, n_species] (1/s), initial concentrations and gas feeds."""

    net: Network
    henry: np.ndarray
    kla: np.ndarray
    c0: np.ndarray
    feeds: list = field(default_factory=list)
    # gas state of each flow map of the scenario (same order; empty: the gas
    # domain stays fixed while the maps cycle) and its kla (empty: `kla`)
    flowmaps: list = field(default_factory=list)
    kla_maps: list = field(default_factory=list)


@dataclass
class Scenario:
    name: str
    net: Network
    model: ModelSpec
    n_particles: int
    n_species: int
    c0: np.ndarray  # [n_c, n_species]
    feeds: list = field(default_factory=list)
    dt: float = 0.1
    n_steps: int = 100
    seed: int = 42
    x0: float = 0.5  # initial biomass concentration, kg/m^3 (sets the weight)
    alloc_factor: float = 1.5
    dead_ratio_threshold: float = 0.01
    min_removal: int = 0
    uniform_init: bool = True
    # flow-map cycle: states of the same mesh replayed in turn (flowmaps[0]
    # is `net`, the state the run starts on); empty: fixed domain
    flowmaps: list = field(default_factory=list)
    t_per_flowmap: float = 0.0
    gas: GasPhase | None = None  # two-phase flow

    @property
    def n_per_flowmap(self) -> int:
        """compute_n_per_flowmap (apps/core/src/global_initaliser.cpp L104-L114)."""
        if self.t_per_flowmap == 0 or len(self.flowmaps) <= 1:
            return 1
        return int(self.t_per_flowmap / self.dt) + 1

    @property
    def capacity(self) -> int:
        return int(math.ceil(self.n_particles * self.alloc_factor))

    def quantum_exponents(self, weight: float) -> np.ndarray:
        """Exponent e of the accumulator quantum 2^e per column, chosen so
        that the value bound is 2^QBITS quanta (ceil(log2) taken exactly)."""
        e = np.zeros(8, dtype=np.int32)
        cols = 1 if self.model.separable else self.model.n_ctb
        for j in range(cols):
            vmax = float(self.model.value_bound[j])
            if not self.model.separable:
                vmax *= weight
            m, ex = math.frexp(vmax)
            e[j] = (ex - 1 if m == 0.5 else ex) - QBITS
        return e

    def algorithmic_bytes(self) -> int:
        """Bytes per particle-step: state + u32 compartment + status + two f32
        ages, each read and written once."""
        return 2 * (self.model.n_var * self.model.itemsize + 4 + 1 + 8)


QBITS = 42  # a value at its bound is 2^QBITS quanta of the exact sums
CTB_QMAX = 1 << QBITS


def weight_from_mass(total_mass: float, x0: float, total_volume: float) -> float:
    """post_init_weight (apps/libs/mc/src/unit.cpp L233-L257): w = X0 V / m_tot."""
    return (x0 * total_volume) / total_mass


def workload(index: int, n_particles: int | None = None, n_steps: int | None = None,
             seed: int | None = None, f64: bool | None = None) -> Scenario:
    """Benchmark workloads (synthetic; no public dataset is involved).

    1: ring of 10 + 2 random links, 1 species, 1e5 particles, FP64 Monod,
       dt 0.1 s, 1000 steps, closed reactor.
    2: 8^3 lattice vortex, 4 species, 1e7 particles, FP64 overflow model,
       glucose inlet at 0, outlet at 511, D = 0.1/h, dt 0.05 s, 5000 steps.
    3: 16^3 lattice vortex, 5e7 particles, FP32 overflow model, dt 0.05 s,
       2000 steps.
    """
    if index == 1:
        net = ring_network(10, 2, 1e-3, 0.5, 0.5e-3, 2e-3, seed=42 if seed is None else seed,
                           max_courant=0.5, dt=0.1)
        model = monod(f64=True if f64 is None else f64)
        n_s = 1
        c0 = np.full((net.n_c, n_s), 5.0)
        return Scenario("ring10_monod_fp64", net, model, n_particles or 100_000, n_s, c0, [],
                        dt=0.1, n_steps=n_steps or 1000, seed=42 if seed is None else seed)
    if index in (2, 3):
        n = 8 if index == 2 else 16
        net = lattice_vortex(n, side=1.0, peak_velocity=0.5, noise=0.1,
                             seed=7 if seed is None else seed)
        use_f64 = (index == 2) if f64 is None else f64
        model = overflow(f64=use_f64)
        n_s = 4
        c0 = np.zeros((net.n_c, n_s))
        c0[:, 0] = 5.0
        c0[:, 1] = 8e-3
        flow = 0.1 / 3600.0 * net.total_volume
        conc = np.zeros(n_s)
        conc[0] = 20.0
        feeds = [Feed(0, net.n_c - 1, flow, conc)]
        npart = n_particles or (10_000_000 if index == 2 else 50_000_000)
        steps = n_steps or (5000 if index == 2 else 2000)
        name = "lattice512_overflow_fp64" if index == 2 else "lattice4096_overflow_fp32"
        return Scenario(name, net, model, npart, n_s, c0, feeds, dt=0.05, n_steps=steps,
                        seed=2024 if seed is None else seed)
    raise ValueError(f"unknown workload {index}")


def batch_scenario(k: int, seed: int = 1234, n_lo: float = 1e4, n_hi: float = 5e6,
                   nc_lo: float = 10, nc_hi: float = 2000, steps: int = 1000,
                   steps_lo: int | None = None, steps_hi: int | None = None,
                   particle_scale: float = 1.0) -> Scenario:
    """Scenario k of the batched workload: compartment count log-uniform on
    [10, 2000] (cubic lattice with a recirculation or a ring, chosen by the
    seed), particles log-uniform on [1e4, 5e6], mu_max uniform on
    [0.3, 1.0]/h, initial glucose uniform on [1, 20] g/L, FP32 Monod,
    dt 0.1 s, closed reactor.  With steps_lo/steps_hi the step count is
    log-uniform on that range (the served workload)."""
    rng = np.random.default_rng(seed * 100003 + k)
    n_c = int(round(math.exp(rng.uniform(math.log(nc_lo), math.log(nc_hi)))))
    n_p = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))) * particle_scale))
    mu = rng.uniform(0.3, 1.0) / 3600.0
    glc = rng.uniform(1.0, 20.0)
    dt = 0.1
    if rng.random() < 0.5:
        n = max(3, int(round(n_c ** (1.0 / 3.0))))
        net = lattice_vortex(n, side=1.0, peak_velocity=0.5, noise=0.1, seed=int(rng.integers(1 << 30)),
                             max_courant=0.5, dt=dt)
    else:
        net = ring_network(max(n_c, 3), 2, 1e-3, 0.5, 0.5e-3, 2e-3, seed=int(rng.integers(1 << 30)),
                           max_courant=0.5, dt=dt)
    if steps_lo is not None:
        steps = int(round(math.exp(rng.uniform(math.log(steps_lo), math.log(steps_hi)))))
    c0 = np.full((net.n_c, 1), glc)
    return Scenario(f"batch{k}", net, monod(f64=False, mu_max=mu), max(n_p, 1024), 1, c0, [],
                    dt=dt, n_steps=steps, seed=seed * 7919 + k)


def with_gas(scen: Scenario, kla: float = 0.05, henry: float = 0.03, gas_fraction: float = 0.1,
             gas_flow: float | None = None, seed: int = 17) -> Scenario:
    """Adds a gas phase to a scenario: a gas ring through the compartments
    (gas volume = gas_fraction x liquid volume), species 1 (O2 when present,
    else 0) transferred with the given kla and Henry constant, air-like gas
    inlet at compartment 0 and outlet at the last one."""
    import dataclasses

    n_c, ns = scen.net.n_c, scen.n_species
    rng = np.random.default_rng(seed)
    src = np.arange(n_c, dtype=np.int64)
    dst = (src + 1) % n_c
    # gas Courant number dt Q / V_gas of about 0.2 by default
    q = gas_flow if gas_flow is not None else 0.2 * float(np.min(scen.net.volume * gas_fraction)) / scen.dt
    flow = q * rng.uniform(0.8, 1.2, size=n_c) if n_c > 1 else np.zeros(0)
    if n_c > 1:
        gnet = Network(n_c, scen.net.volume * gas_fraction, src, dst, flow).finalize()
    else:
        gnet = Network(1, scen.net.volume * gas_fraction, np.zeros(0, np.int64), np.zeros(0, np.int64),
                       np.zeros(0)).finalize()
    o2 = 1 if ns > 1 else 0
    k = np.zeros((n_c, ns))
    k[:, o2] = kla
    h = np.zeros(ns)
    h[o2] = henry
    cg = np.zeros((n_c, ns))
    cg[:, o2] = 0.28  # kg/m3 of O2 in air
    conc = np.zeros(ns)
    conc[o2] = 0.28
    feeds = [Feed(0, n_c - 1, q, conc)]
    return dataclasses.replace(scen, gas=GasPhase(gnet, h, k, cg, feeds))


def small_ring(n_particles: int = 4096, n_c: int = 10, seed: int = 3, f64: bool = True,
               model: ModelSpec | None = None, n_steps: int = 20, dt: float = 0.1,
               feeds: bool = False) -> Scenario:
    """Small ring scenario for parity tests."""
    net = ring_network(n_c, 2, 1e-3, 0.5, 0.5e-3, 2e-3, seed=seed, max_courant=0.5, dt=dt)
    model = model or monod(f64=f64)
    n_s = max(1, model.n_ctb)
    c0 = np.zeros((n_c, n_s))
    c0[:, 0] = 5.0
    if n_s > 1:
        c0[:, 1] = 8e-3
    fl = []
    if feeds:
        conc = np.zeros(n_s)
        conc[0] = 20.0
        fl = [Feed(0, n_c - 1, 5e-5, conc)]
    return Scenario(f"small_ring{n_c}", net, model, n_particles, n_s, c0, fl, dt=dt,
                    n_steps=n_steps, seed=seed)


def zero_d(n_particles: int = 4096, seed: int = 5, model: ModelSpec | None = None,
           n_steps: int = 10, dt: float = 0.1, outlet: bool = True) -> Scenario:
    """0-D reactor (one compartment): move disabled, optional outlet."""
    net = single_compartment(1e-3)
    model = model or monod(f64=True)
    n_s = max(1, model.n_ctb)
    c0 = np.zeros((1, n_s))
    c0[:, 0] = 5.0
    fl = []
    if outlet:
        conc = np.zeros(n_s)
        conc[0] = 20.0
        fl = [Feed(0, 0, 2e-4, conc)]
    return Scenario("zero_d", net, model, n_particles, n_s, c0, fl, dt=dt, n_steps=n_steps,
                    seed=seed)
