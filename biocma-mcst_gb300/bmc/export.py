"""Time records of a run, in the dataset layout of the reference's exporters.

The reference writes, every `dump_interval` main-loop iterations, into an
HDF5 file (apps/core/src/dataexporter/main_exporter.cpp L52-L150,
partial_exporter.cpp L25-L160, host_export_handler.cpp L70-L115):

  records/time                  [n_export]
  records/concentration_liquid  [n_export, n_compartments, n_species]
  records/volume_liquid         [n_export, n_compartments]
  records/concentration_gas     [n_export, n_compartments, n_species]  (two-phase)
  records/volume_gas            [n_export, n_compartments]             (two-phase)
  records/mtr                   [n_export, n_compartments, n_species]  (two-phase)
  records/number_particle       [n_export, n_compartments]
  records/tallies               [n_export, n_tallies]
  probes/LeavingTime            [n_leaving]   (with time-event probes on)
  probes/DivisionTime           [n_division]
  biological_model/<k>/<variable>, spatial/<variable>, mass, spatial/mass,
                     age_hydro, age   (particle dump k, at every export)

plus `initial_parameters/*` and `final_result/*` (the live particle count,
event totals, the final liquid and gas fields).  records/tallies holds the
reference's event counts (MC::EventType order) accumulated since the
previous export, which clears them (host_export_handler.cpp L118-L122);
final_result/events/* are totals over the run (the reference reads its
counters after the last export cleared them, so its values cover only the
steps after the last export).  `Records`
collects the same arrays from a device scenario (read-backs between graph
runs) and writes them under the same names: with h5py to an HDF5 file,
without it (this image) to a NumPy archive whose keys are the dataset paths.
"""
from __future__ import annotations

import numpy as np

TALLIES = ("NewParticle", "Exit", "Move", "Death", "Overflow", "ChangeWeight")
# probe names of the reference's exporter (map_probe_name, probe.hpp L21-L22),
# in the order of the library's probe indices
PROBES = ("LeavingTime", "DivisionTime")


class Records:
    """Accumulates the records of one scenario (a GpuScenario, or any object
    with `liquid()`, `repartition()`, `stats()`, `scen`, and `gas()` for a
    two-phase scenario)."""

    def __init__(self, g, dump_particles: bool = True, export_age: bool = True):
        """dump_particles and export_age: the reference's dump_particle_state
        and export_age build flags (both on in its default build)."""
        self.g = g
        self.dump_particles = dump_particles
        self.export_age = export_age
        self.n_dumps = 0
        self.dumps: dict[str, np.ndarray] = {}
        self.rows: dict[str, list] = {}
        sc = g.scen
        # MainExporter::write_initial and its constructor (main_exporter.cpp
        # L17-L50); final_time is set by run(); one host thread drives the
        # device, one process
        names = tuple(sc.model.species) or tuple(f"species_{k}" for k in range(sc.n_species))
        self.initial = {
            "initial_parameters/number_particles": sc.n_particles,
            "initial_parameters/initial_weight": float(g.weight) if getattr(g, "weight", None) else 0.0,
            "initial_parameters/initial_biomass_concentration": sc.x0,
            "initial_parameters/number_compartment": sc.net.n_c,
            "initial_parameters/final_time": 0.0,
            "initial_parameters/delta_time": sc.dt,
            "initial_parameters/n_map": max(1, len(getattr(sc, "flowmaps", []) or [])),
            "initial_parameters/t_per_flow_map": getattr(sc, "t_per_flowmap", 0.0),
            "misc/species_names": np.array([n.encode() for n in names[:sc.n_species]]),
            "misc/n_node_thread": 1,
            "misc/n_rank": 1,
        }
        self.final: dict[str, float] = {}
        self.totals = dict.fromkeys(TALLIES, 0)

    def _append(self, name: str, value):
        self.rows.setdefault(name, []).append(np.asarray(value))

    def record(self, t: float, volume=None):
        """One export: the time, the liquid field, the volumes (the current
        flow map's when given), the particle count per compartment and the
        tallies of the last step."""
        sc = self.g.scen
        # the flow map the domain holds: the one the last step ran on
        fm = getattr(sc, "flowmaps", None) or []
        m = None
        if fm:
            step = int(self.g.stats()["step"])
            m = ((step - 1) // sc.n_per_flowmap) % len(fm) if step > 0 else 0
        if volume is None:
            volume = fm[m].volume if m is not None else sc.net.volume
        self._append("records/time", float(t))
        self._append("records/concentration_liquid", self.g.liquid()["C"])
        self._append("records/volume_liquid", np.asarray(volume, dtype=float))
        if getattr(sc, "gas", None) is not None:
            gas = self.g.gas()
            gfm = getattr(sc.gas, "flowmaps", None) or []
            gvol = gfm[m].volume if (gfm and m is not None) else sc.gas.net.volume
            self._append("records/concentration_gas", gas["Cg"])
            self._append("records/volume_gas", np.asarray(gvol, dtype=float))
            self._append("records/mtr", gas["mtr"])
        self._append("records/number_particle", self.g.repartition().astype(np.uint64))
        ev = self.g.events(clear=True)
        self._append("records/tallies", np.array([ev[k] for k in TALLIES], dtype=np.uint64))
        for k in TALLIES:
            self.totals[k] += ev[k]
        self.save_probes()
        if self.dump_particles:
            self.save_particle_state()

    def save_particle_state(self):
        """The reference's particle dump (save_particle_state, append_properties,
        apps/core/src/post_process.cpp L64-L74, L146-L163; get_properties,
        apps/core/public/core/post_process.hpp L85-L104, L170-L240): after
        force_remove_dead, under biological_model/<k>/ (k counts the dumps)
        each exported model variable and the mass (Model::mass, computed on
        the device) per particle in float64, their sums per compartment under
        spatial/<name>, and with export_age both ages (age_hydro = ages(i, 0),
        age = ages(i, 1))."""
        g = self.g
        g.force_remove_dead()
        p = g.particles()
        mass = np.asarray(g.mass(), dtype=np.float64)
        m = g.scen.model
        n_c = g.scen.net.n_c
        pos = p["pos"].astype(np.int64)
        base = f"biological_model/{self.n_dumps}/"
        cols = [(name, p["state"][k].astype(np.float64))
                for name, k in zip(m.export_names, m.export_index) if name != "mass"]
        cols.append(("mass", mass))
        for name, v in cols:
            self.dumps[base + name] = v
            self.dumps[base + "spatial/" + name] = np.bincount(pos, weights=v, minlength=n_c)
        if self.export_age:
            self.dumps[base + "age_hydro"] = p["age_h"].astype(np.float64)
            self.dumps[base + "age"] = p["age_d"].astype(np.float64)
        self.n_dumps += 1

    def save_probes(self, force: bool = False):
        """The reference's save_probes (apps/core/src/post_process.cpp
        L30-L60, called at every export and, forced, at the end of the run):
        each probe whose buffer is full, or every probe with `force`, has its
        stored values appended to probes/<name> and is emptied.  Nothing
        while the scenario's probes are off."""
        cap = getattr(self.g, "probe_capacity", 0)
        if not cap:
            return
        for k, name in enumerate(PROBES):
            values, n = self.g.probe_read(k)
            if n >= cap or force:
                self.rows.setdefault(f"probes/{name}", []).append(values)
                self.g.probe_clear(k)

    def run(self, n_steps: int, dump_interval: int, t0: float = 0.0):
        """Advance n_steps in graph-replayed runs of dump_interval steps,
        recording the first state and after every run (the reference records
        the first and the last state as well, main_exporter.cpp L58)."""
        dt = self.g.scen.dt
        self.initial["initial_parameters/final_time"] = t0 + n_steps * dt
        self.record(t0)
        done = 0
        while done < n_steps:
            k = min(dump_interval, n_steps - done)
            self.g.run(k)
            done += k
            self.record(t0 + done * dt)
        self.save_probes(force=True)
        st = self.g.stats()
        ev = self.g.events(clear=True)  # steps after the last export (none here)
        tot = {k: self.totals[k] + ev[k] for k in TALLIES}
        self.final = {
            "final_result/number_particles": st["n_used"] - st["inactive"],
            "final_result/events/move": tot["Move"],
            "final_result/events/total_division": tot["NewParticle"],
            "final_result/events/total_death": tot["Death"],
            "final_result/events/total_exit": tot["Exit"],
            "final_result/concentration_liquid": self.g.liquid()["C"],
        }
        if getattr(self.g.scen, "gas", None) is not None:
            self.final["final_result/concentration_gas"] = self.g.gas()["Cg"]
        return self

    def arrays(self) -> dict:
        out = {k: (np.concatenate(v) if k.startswith("probes/") else np.stack(v)) for k, v in self.rows.items()}
        out.update(self.dumps)
        out.update({k: np.asarray(v) for k, v in self.initial.items()})
        out.update({k: np.asarray(v) for k, v in self.final.items()})
        return out

    def save(self, path: str) -> str:
        """Write the records: HDF5 when h5py is importable, else a NumPy
        archive (`path` gets the .npz suffix) with the dataset paths as keys."""
        data = self.arrays()
        try:
            import h5py  # noqa: F401
        except ImportError:
            if not path.endswith(".npz"):
                path = path + ".npz"
            np.savez_compressed(path, **data)
            return path
        import h5py

        with h5py.File(path, "w") as f:
            for k, v in data.items():
                f.create_dataset(k, data=v)
        return path


def load(path: str) -> dict:
    """Read records written by `Records.save` (either form)."""
    if path.endswith(".npz"):
        with np.load(path) as z:
            return {k: z[k] for k in z.files}
    import h5py

    out = {}
    with h5py.File(path, "r") as f:
        f.visititems(lambda k, v: out.__setitem__(k, v[()]) if hasattr(v, "shape") else None)
    return out
