"""Time records in the dataset layout of the reference's exporters
(records/time, concentration_liquid, volume_liquid, number_particle,
tallies, gas fields for two-phase runs)."""
import numpy as np
import pytest

from bmc import export, scenarios


class FakeScenario:
    """What Records reads from a device scenario, from the CPU restatement."""

    def __init__(self, oracle_mod, sc):
        self.scen = sc
        self.o = oracle_mod.Oracle(sc)
        self.o.init_particles()
        self.last = {}
        self.ev = dict.fromkeys(export.TALLIES, 0)

    def run(self, n):
        for _ in range(n):
            self.last = self.o.step()
            self.ev["NewParticle"] += int(self.o.s.requested_divisions)
            self.ev["Exit"] += self.last["exits"]
            self.ev["Move"] += self.last["moves"]
            self.ev["Overflow"] += self.last["overflow"]

    def events(self, clear=False):
        out = dict(self.ev)
        if clear:
            self.ev = dict.fromkeys(export.TALLIES, 0)
        return out

    def force_remove_dead(self):
        self.o.force_remove_dead()

    def particles(self):
        return self.o.particles()

    def mass(self):
        return self.o.mass()

    @property
    def weight(self):
        return float(self.o.s.weight)

    def liquid(self):
        return {"C": self.o.C.copy()}

    def gas(self):
        return {"Cg": self.o.Cg.copy(), "Mg": self.o.Mg.copy(), "mtr": self.o.mtr.copy()}

    def repartition(self):
        p = self.o.particles()
        idle = p["status"] == 0
        return np.bincount(p["pos"][idle], minlength=self.scen.net.n_c).astype(np.uint64)

    def stats(self):
        st = {k: 0 for k in ("births", "exits", "moves", "overflow")}
        st.update(self.last)
        st["n_used"], st["inactive"] = int(self.o.s.n_used), int(self.o.s.inactive)
        st["step"] = int(self.o.s.step)
        return st

    def probe_enable(self, cap):
        self.o.probe_enable(cap)
        self.probe_capacity = cap

    def probe_read(self, k):
        return self.o.probe_read(k)

    def probe_clear(self, k):
        self.o.probe_clear(k)


def test_layout_and_save_roundtrip(oracle_mod, tmp_path):
    sc = scenarios.small_ring(3000, feeds=True)
    rec = export.Records(FakeScenario(oracle_mod, sc)).run(10, dump_interval=4)
    a = rec.arrays()
    n_exp = 1 + 3  # first state, after 4, 8 and 10 steps
    assert a["records/time"].shape == (n_exp,)
    assert np.allclose(a["records/time"], [0.0, 4 * sc.dt, 8 * sc.dt, 10 * sc.dt])
    assert a["records/concentration_liquid"].shape == (n_exp, sc.net.n_c, sc.n_species)
    assert a["records/volume_liquid"].shape == (n_exp, sc.net.n_c)
    assert a["records/number_particle"].shape == (n_exp, sc.net.n_c)
    assert a["records/tallies"].shape == (n_exp, len(export.TALLIES))
    assert np.all(a["records/tallies"][0] == 0)  # nothing before the first step
    col = {k: a["records/tallies"][:, i] for i, k in enumerate(export.TALLIES)}
    assert col["Move"].sum() == a["final_result/events/move"] > 0
    assert col["Exit"].sum() == a["final_result/events/total_exit"] > 0
    assert col["NewParticle"].sum() == a["final_result/events/total_division"]
    assert np.all(col["Death"] == 0) and np.all(col["ChangeWeight"] == 0)
    assert a["records/number_particle"][-1].sum() == a["final_result/number_particles"]
    assert np.array_equal(a["final_result/concentration_liquid"], a["records/concentration_liquid"][-1])
    assert a["initial_parameters/final_time"] == pytest.approx(10 * sc.dt)
    assert a["initial_parameters/initial_weight"] > 0.0
    assert a["misc/species_names"].tolist() == [b"glucose"]
    path = rec.save(str(tmp_path / "run"))
    back = export.load(path)
    for k, v in a.items():
        assert np.array_equal(back[k], v), k


def test_particle_dumps_in_the_reference_layout(oracle_mod):
    """biological_model/<k>/ after every export: each exported variable and
    the mass per live particle, their sums per compartment, both ages."""
    sc = scenarios.small_ring(3000, feeds=True, model=scenarios.overflow(f64=True))
    f = FakeScenario(oracle_mod, sc)
    a = export.Records(f).run(6, dump_interval=3).arrays()
    for k in range(3):
        base = f"biological_model/{k}/"
        n = len(a[base + "mass"])
        assert n == a["records/number_particle"][k].sum()
        for name in ("cycle_time", "mu", "q_s", "q_o2", "q_ac", "mass"):
            assert a[base + name].shape == (n,) and a[base + name].dtype == np.float64
            assert a[base + "spatial/" + name].shape == (sc.net.n_c,)
            assert np.isclose(a[base + "spatial/" + name].sum(), a[base + name].sum())
        assert a[base + "age_hydro"].shape == (n,) and a[base + "age"].shape == (n,)
    # the overflow model's mass is its first state variable
    assert np.array_equal(a["biological_model/2/mass"], f.o.particles()["state"][0])
    plain = export.Records(FakeScenario(oracle_mod, sc), dump_particles=False).run(6, dump_interval=3).arrays()
    assert not any(k.startswith("biological_model/") for k in plain)


@pytest.mark.gpu
def test_gpu_particle_dumps_match_the_restatement(oracle_mod):
    from bmc.sim import GpuScenario

    for model in (scenarios.overflow(f64=True), scenarios.fixed_length()):
        sc = scenarios.small_ring(4000, feeds=True, model=model)
        sc.feeds[0].flow = 2e-3  # exits: the dumps remove them first
        g = GpuScenario(sc)
        a = export.Records(g).run(8, dump_interval=4).arrays()
        f = FakeScenario(oracle_mod, sc)
        f.o = oracle_mod.Oracle(sc, phys_capacity=g.cap)
        f.o.init_particles()
        f.o.set_weight(g.weight)
        b = export.Records(f).run(8, dump_interval=4).arrays()
        keys = [k for k in a if k.startswith("biological_model/")]
        assert keys and sorted(keys) == sorted(k for k in b if k.startswith("biological_model/"))
        for k in keys:
            assert np.array_equal(a[k].view(np.uint64), b[k].view(np.uint64)), (model.name, k)


def test_volumes_follow_the_flow_maps(oracle_mod):
    """With flow maps, each export carries the volumes of the map the last
    step ran on (the reference exports the current state's volumes)."""
    import sys
    import os

    sys.path.insert(0, os.path.dirname(__file__))
    from test_flowmap import gas_flowmap_scenario

    sc = gas_flowmap_scenario(n_particles=3000)  # 3 maps, 4 steps each
    f = FakeScenario(oracle_mod, sc)
    a = export.Records(f, dump_particles=False).run(12, dump_interval=2).arrays()
    for k, done in enumerate(range(0, 13, 2)):
        m = ((done - 1) // 4) % 3 if done > 0 else 0
        assert np.array_equal(a["records/volume_liquid"][k], sc.flowmaps[m].volume), done
        assert np.array_equal(a["records/volume_gas"][k], sc.gas.flowmaps[m].volume), done


def _probe_scenario():
    sc = scenarios.zero_d(3000, model=scenarios.monod(f64=True, m_div=1.0), outlet=True)
    sc.feeds[0].flow = 1e-3
    return sc


def test_probes_exported_as_the_reference_exporter(oracle_mod):
    """A full buffer goes to probes/<name> at the next export and is emptied;
    the end of the run exports whatever is left (save_probes(force))."""
    sc = _probe_scenario()
    small = FakeScenario(oracle_mod, sc)
    small.probe_enable(300)
    a = export.Records(small).run(12, dump_interval=3).arrays()
    big = FakeScenario(oracle_mod, sc)
    big.probe_enable(1 << 20)
    b = export.Records(big).run(12, dump_interval=3).arrays()
    for name in export.PROBES:
        full = b[f"probes/{name}"]
        part = a[f"probes/{name}"]
        assert len(full) > 300 and 0 < len(part) <= len(full)
    # division times are in slot order: what the small buffers kept is a
    # sequence of stretches of the complete list
    div = b["probes/DivisionTime"]
    assert set(a["probes/DivisionTime"].tolist()) <= set(div.tolist())


@pytest.mark.gpu
def test_gpu_probe_records_match_the_restatement(oracle_mod):
    from bmc.sim import GpuScenario

    sc = _probe_scenario()
    g = GpuScenario(sc, capacity=4096)
    g.probe_enable(1 << 18)
    a = export.Records(g).run(10, dump_interval=5).arrays()
    f = FakeScenario(oracle_mod, sc)
    f.o = oracle_mod.Oracle(sc, phys_capacity=g.cap)
    f.o.init_particles()
    f.o.set_weight(g.weight)
    f.probe_enable(1 << 18)
    b = export.Records(f).run(10, dump_interval=5).arrays()
    assert np.array_equal(a["probes/DivisionTime"], b["probes/DivisionTime"])
    assert np.array_equal(np.sort(a["probes/LeavingTime"]), np.sort(b["probes/LeavingTime"]))
    assert len(a["probes/DivisionTime"]) > 0 and len(a["probes/LeavingTime"]) > 0


@pytest.mark.gpu
def test_gpu_records_match_the_scenario():
    from bmc.sim import GpuScenario

    sc = scenarios.with_gas(scenarios.small_ring(5000, n_c=12, feeds=True,
                                                 model=scenarios.overflow(f64=True)), kla=0.05, henry=0.03)
    g = GpuScenario(sc)
    rec = export.Records(g).run(9, dump_interval=3)
    a = rec.arrays()
    assert a["records/concentration_gas"].shape == (4, 12, sc.n_species)
    assert np.array_equal(a["records/concentration_liquid"][-1], g.liquid()["C"])
    assert np.array_equal(a["records/number_particle"][-1], g.repartition())
    assert a["final_result/number_particles"] == g.stats()["n_used"] - g.stats()["inactive"]
