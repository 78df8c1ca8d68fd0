"""The reference's particle cycle, compiled from its own headers, run beside
the oracle.  TEST INFRASTRUCTURE ONLY.

oracle/refbuild/ref_cycle.cpp compiles the reference's cycle functors
(kernels.hpp, model_kernel.hpp, contribution_kernel.hpp, move_kernel.hpp) and
its particle container (particles_container.hpp) unmodified against the
Kokkos stand-in into oracle/_ref/libbmc_ref.so (built where the reference
tree is present).  RefCycle starts that cycle from the oracle's initial
container and, every main-loop iteration, hands it

* the concentrations the oracle's cycle read (the oracle's liquid step runs
  first: the reference's liquid step needs Eigen, which is not here),
* the draws the oracle gives every container slot (its Philox draws keyed by
  the particle's id: move test, destination, exit; the division draws),

then compares the two containers slot by slot.  What is compared and how:

* particle counts, statuses, ages: equal;
* state variables: equal (bit for bit), except the variables a division does
  not set in a newborn (SimpleAcetate's a_e ... phi_a, which the reference
  takes from its division buffer's previous contents and the next update
  overwrites before anything reads them);
* compartments of Idle particles: equal (the reference's move kernel also
  moves particles that already left; their compartments are never read);
* event counts: births, exits, and moves when no particle that left is
  still in the container;
* contributions: the oracle's exact sums against the exact sum of the
  operands the reference's scatter received, within the rounding of the
  float weight the reference multiplies by.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

import oracle as _orc

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libbmc_ref.so")
# the same cycle built with the reference's probes on (use_probe, a buffer of
# 10,000 values per probe)
REF_PROBE_LIB = os.path.join(HERE, "_ref", "libbmc_ref_probe.so")
REF_PROBE_CAPACITY = 10000
VP = ct.c_void_p
_LIBS = {}

# draw kinds of the stand-in's random pool: 0 float uniform, 1 double
# uniform, 2 standard normal; SimpleAcetate::division draws two log-normal
# factors (normals), then two truncated normals (double uniforms)
DIV_KINDS = {3: (0, 0, 0, 0), 5: (2, 2, 1, 1)}
# state variables a division sets in the newborn
DIV_SET_VARS = {3: 2, 5: 4}


def normalized(p: dict, births: int, model_id: int) -> dict:
    """A container as the comparison sees it: newborns' variables that the
    division does not set zeroed, compartments of non-Idle slots replaced by
    0xFFFFFFFF."""
    st = np.array(p["state"], dtype=np.float32, copy=True)
    n = st.shape[1]
    if births:
        st[DIV_SET_VARS[model_id]:, n - births:] = 0.0
    pos = np.where(np.asarray(p["status"]) == 0, np.asarray(p["pos"], np.uint32), np.uint32(0xFFFFFFFF))
    return dict(state=st, pos=pos.astype(np.uint32), status=np.asarray(p["status"], np.uint8),
                age_h=np.asarray(p["age_h"], np.float32), age_d=np.asarray(p["age_d"], np.float32))


def digest(p: dict, births: int, model_id: int) -> str:
    """SHA-256 (first 32 hex digits) of the normalized container's bytes."""
    import hashlib

    q = normalized(p, births, model_id)
    h = hashlib.sha256()
    for k in ("state", "pos", "status", "age_h", "age_d"):
        h.update(np.ascontiguousarray(q[k]).tobytes())
    return h.hexdigest()[:32]


def available(probes: bool = False) -> bool:
    return os.path.exists(REF_PROBE_LIB if probes else REF_LIB)


def ref_lib(probes: bool = False):
    if probes not in _LIBS:
        L = ct.CDLL(REF_PROBE_LIB if probes else REF_LIB)
        L.ref_cycle_new.restype = VP
        L.ref_cycle_new.argtypes = [ct.c_int32, ct.c_uint32, ct.c_uint32, ct.c_uint32, VP, VP, VP, VP, ct.c_uint32,
                                    VP, VP, VP, ct.c_uint64, VP, VP, VP, VP, ct.c_double, ct.c_uint64, ct.c_double,
                                    ct.c_uint32]
        L.ref_cycle_free.argtypes = [VP]
        L.ref_cycle_step.restype = ct.c_int32
        L.ref_cycle_step.argtypes = [VP, ct.c_double, VP, VP, VP, VP, VP, VP, VP, VP, VP, VP]
        L.ref_cycle_read.restype = ct.c_uint64
        L.ref_cycle_read.argtypes = [VP, ct.c_uint64, VP, VP, VP, VP, VP]
        L.ref_cycle_misses.restype = ct.c_long
        L.ref_cycle_misses.argtypes = [VP]
        L.ref_cycle_set_leaving.argtypes = [VP, ct.c_uint32, VP]
        L.ref_cycle_step_stream.restype = ct.c_int32
        L.ref_cycle_step_stream.argtypes = [VP, ct.c_double, VP, ct.c_uint64, VP, VP, VP, VP]
        if hasattr(L, "ref_assert_failures"):  # the pin library's (not the probe build's)
            L.ref_assert_failures.restype = ct.c_long
        L.ref_cycle_probe.restype = ct.c_uint64
        L.ref_cycle_probe.argtypes = [VP, ct.c_int32, VP, ct.c_uint64, VP]
        _LIBS[probes] = L
    return _LIBS[probes]


def _p(a: np.ndarray):
    return ct.c_void_p(a.ctypes.data)


def draw_tables(o) -> dict:
    """The draws of every slot of the oracle's container for its next step."""
    L = _orc.lib()
    n = o.n_used
    ids = np.ascontiguousarray(o.id[:n])
    d0 = np.zeros((max(n, 1), 4), np.float32)
    L.orc_draw_table.argtypes = [ct.c_uint64, VP, ct.c_uint64, ct.c_uint32, ct.c_uint32, VP]
    L.orc_division_draw_table.argtypes = [ct.c_uint64, VP, ct.c_uint64, ct.c_uint32, VP]
    step = int(o.s.step)
    L.orc_draw_table(o.scen.seed, _p(ids), n, step, 0, _p(d0))
    div = np.zeros((max(n, 1), 4))
    if o.scen.model.model_id == 5:
        L.orc_division_draw_table(o.scen.seed, _p(ids), n, step, _p(div))
    return dict(move0=np.ascontiguousarray(d0[:, 0]), move1=np.ascontiguousarray(d0[:, 1]),
                exit=np.ascontiguousarray(d0[:, 2]), div=div)


class RefCycle:
    """The reference's compiled cycle holding a copy of the oracle's
    container (after init_particles)."""

    def __init__(self, o, particles_per_team: int = 64, probes: bool = False):
        """probes: run the cycle built with the reference's probes on."""
        self.L = ref_lib(probes)
        sc = o.scen
        net = sc.net
        m = sc.model
        if m.model_id not in DIV_KINDS or m.f64:
            raise ValueError("the reference-cycle comparison runs FixedLength and SimpleAcetate")
        self.o = o
        self.model = m.model_id
        self.n_var = m.n_var
        self.n_ctb = m.n_ctb
        self.n_c = net.n_c
        p = o.particles()
        n = len(p["pos"])
        outs = [(fd.outlet, fd.flow) for fd in sc.feeds if fd.outlet >= 0]
        self._keep = dict(
            vol=np.ascontiguousarray(net.volume, np.float64),
            out_flow=np.ascontiguousarray(net.out_flow, np.float64),
            nbr=np.ascontiguousarray(net.neighbors, np.uint64),
            cdf=np.ascontiguousarray(net.cdf, np.float64),
            oi=np.array([i for i, _ in outs] or [0], np.uint64),
            of=np.array([f for _, f in outs] or [0.0], np.float64),
            ov=np.array([net.volume[i] for i, _ in outs] or [0.0], np.float64),
            state=np.ascontiguousarray(p["state"], np.float32),
            pos=np.ascontiguousarray(p["pos"], np.uint64),
            age_h=np.ascontiguousarray(p["age_h"]),
            age_d=np.ascontiguousarray(p["age_d"]),
            kinds=np.array(DIV_KINDS[self.model], np.int32),
        )
        k = self._keep
        self.h = self.L.ref_cycle_new(self.model, net.n_c, net.K, sc.n_species, _p(k["vol"]), _p(k["out_flow"]),
                                         _p(k["nbr"]), _p(k["cdf"]), len(outs), _p(k["oi"]), _p(k["of"]),
                                         _p(k["ov"]), n, _p(k["state"]), _p(k["pos"]), _p(k["age_h"]),
                                         _p(k["age_d"]), float(o.weight), int(o.s.min_removal),
                                         float(o.s.dead_ratio_threshold), particles_per_team)
        if not self.h:
            raise RuntimeError("reference cycle not created")

    def close(self):
        if self.h:
            self.L.ref_cycle_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def misses(self) -> int:
        return int(self.L.ref_cycle_misses(self.h))

    def particles(self) -> dict:
        L = self.L
        n = int(L.ref_cycle_read(self.h, 0, None, None, None, None, None))
        cap = max(n, 1)
        st = np.zeros((self.n_var, cap), np.float32)
        pos = np.zeros(cap, np.uint64)
        status = np.zeros(cap, np.uint8)
        ah = np.zeros(cap, np.float32)
        ad = np.zeros(cap, np.float32)
        if n:
            L.ref_cycle_read(self.h, cap, _p(st), _p(pos), _p(status), _p(ah), _p(ad))
        return dict(state=st[:, :n], pos=pos[:n].astype(np.uint32), status=status[:n], age_h=ah[:n], age_d=ad[:n])

    def step(self) -> dict:
        """One main-loop iteration: the oracle's, then the reference's cycle
        with the oracle's concentrations and draws.  Returns the comparison
        (counts of disagreeing values, zero when the two agree)."""
        o = self.o
        inactive_before = int(o.s.inactive)
        tab = draw_tables(o)
        o.step()
        conc = np.ascontiguousarray(o.C, np.float64)
        # the outlets' flows this step's cycle used (scheduled feeds change them)
        n_out = int(o.s.n_outlets)
        if n_out:
            flows = np.array([o.s.outlet_flow[k] for k in range(n_out)], np.float64)
            self.L.ref_cycle_set_leaving(self.h, n_out, _p(flows))
        stats = np.zeros(8, np.uint64)
        ex = np.zeros(self.n_ctb * self.n_c)
        ab = np.zeros(self.n_ctb * self.n_c)
        sc = np.zeros(self.n_ctb * self.n_c, np.float32)
        rc = self.L.ref_cycle_step(self.h, o.scen.dt, _p(conc), _p(tab["move0"]), _p(tab["move1"]),
                                      _p(tab["exit"]), _p(tab["div"]), _p(self._keep["kinds"]), _p(stats), _p(ex),
                                      _p(ab), _p(sc))
        if rc != 0:
            raise RuntimeError("reference cycle refused the step (empty container)")
        return self.compare(stats, ex.reshape(self.n_ctb, self.n_c), ab.reshape(self.n_ctb, self.n_c),
                            sc.reshape(self.n_ctb, self.n_c), inactive_before)

    def run_free(self, n_steps: int, seed: int) -> int:
        """Free-running: n_steps main-loop iterations of the reference's
        cycle drawing from its own xorshift1024* stream (seeded with `seed`),
        coupled to the oracle's liquid step, which receives the exact sums of
        the reference's contribution operands.  The oracle's own particles
        are not used.  Returns the births counted."""
        o = self.o
        L = _orc.lib()
        L.orc_liquid_step.argtypes = [VP, ct.c_double]
        stats = np.zeros(8, np.uint64)
        ex = np.zeros(self.n_ctb * self.n_c)
        ab = np.zeros_like(ex)
        sc = np.zeros(self.n_ctb * self.n_c, np.float32)
        births = 0
        for _ in range(n_steps):
            L.orc_liquid_step(ct.byref(o.s), o.scen.dt)
            conc = np.ascontiguousarray(o.C, np.float64)
            if self.L.ref_cycle_step_stream(self.h, o.scen.dt, _p(conc), seed, _p(stats), _p(ex), _p(ab),
                                               _p(sc)) != 0:
                break
            o.src[:, :self.n_ctb] = ex.reshape(self.n_ctb, self.n_c).T
            births += int(stats[1])
        return births

    def compare(self, stats, exact, absum, scatter, inactive_before) -> dict:
        o = self.o
        os_ = o.stats()
        r = self.particles()
        q = o.particles()
        n = len(r["pos"])
        out = dict(n_ref=n, n_oracle=o.n_used)
        if n != o.n_used:
            out["count"] = 1
            return out
        births = int(os_["births"])
        newborn = np.zeros(n, bool)
        newborn[n - births:] = True
        vs = DIV_SET_VARS[self.model]
        bad_state = 0
        for v in range(self.n_var):
            a = q["state"][v].astype(np.float32).view(np.uint32)
            b = r["state"][v].view(np.uint32)
            diff = a != b
            if v >= vs:
                diff &= ~newborn
            bad_state += int(diff.sum())
        idle = q["status"] == 0
        out.update(
            status=int((q["status"] != r["status"]).sum()),
            state=bad_state,
            pos=int(((q["pos"] != r["pos"]) & idle).sum()),
            age_h=int((q["age_h"].view(np.uint32) != r["age_h"].view(np.uint32)).sum()),
            age_d=int((q["age_d"].view(np.uint32) != r["age_d"].view(np.uint32)).sum()),
            births=int(stats[1]) - births,
            exits=int(stats[2]) - int(os_["exits"]),
            overflow=int(stats[4]) + int(os_["overflow"]),
        )
        if inactive_before == 0:
            out["moves"] = int(stats[3]) - int(os_["moves"])
        # contributions: [species j][compartment p]
        src = np.asarray(o.src).reshape(self.n_c, -1)[:, :self.n_ctb].T
        tol = 2.0 ** -22 * absum + 1e-300
        out["contrib"] = int((np.abs(src - exact) > tol).sum())
        with np.errstate(divide="ignore", invalid="ignore"):
            out["scatter_rel_dev"] = float(np.nanmax(np.where(absum > 0, np.abs(scatter - exact) / absum, 0.0)))
            out["scatter_vs_oracle"] = float(np.nanmax(np.where(absum > 0, np.abs(scatter - src) / absum, 0.0)))
        out["digest_ref"] = digest(r, int(stats[1]), self.model)
        out["digest_oracle"] = digest(q, births, self.model)
        out["exact"] = exact
        out["scatter"] = scatter
        out["absum"] = absum
        out["src"] = src
        out["births_n"] = births
        out["exits_n"] = int(os_["exits"])
        out["moves_n"] = int(os_["moves"])
        out["compacted"] = int(os_["compacted"])
        return out


    def probe(self, k: int) -> tuple[np.ndarray, bool]:
        """Values probe k (0 leaving times, 1 division times) holds and
        whether it needs exporting (Probes::get, need_export)."""
        out = np.zeros(REF_PROBE_CAPACITY)
        full = ct.c_int32()
        n = int(self.L.ref_cycle_probe(self.h, k, _p(out), len(out), ct.byref(full)))
        return out[:min(n, len(out))].copy(), bool(full.value)
