"""Writes tests/golden/ref_probes.json from the reference's own cycle built
with its probes on.

The reference's cycle records, when compiled with use_probe, the residence
time of every particle leaving through an outlet (ProbeType::LeavingTime)
and the time since its last division of every particle asking to divide
(ProbeType::DivisionTime) into buffers of probe_buffer_size values
(apps/libs/simulation/public/simulation/probe.hpp).  `make -C oracle/refbuild
REF=<reference tree>` builds that cycle (oracle/_ref/libbmc_ref_probe.so,
the same driver as the cycle pins with the configuration's use_probe set);
__graft_entry__.build() runs it where the tree is present.  For each
non-emulating scenario of make_ref_cycle_golden.py, the reference's cycle
runs beside the oracle (oracle/ref_cycle.py, probes=True) from the same
initial container with the oracle's concentrations and draws; every step the
values each reference probe holds must equal the oracle's probe bit for bit
(the stand-in runs the reference's teams one after another, so both record
in slot order), and the script records per step the count of values and
the SHA-256 of their float64 bytes.

    python tests/golden/make_ref_probes_golden.py
"""
import hashlib
import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "biocma-mcst_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import ref_cycle  # noqa: E402

STEPS = 40


def cycle_cases():
    spec = importlib.util.spec_from_file_location("make_ref_cycle_golden",
                                                  os.path.join(HERE, "make_ref_cycle_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return [(n, b, kw) for n, b, kw in m.cases() if not kw.get("quirk_tag3d")]


def probe_digest(values: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(values, np.float64).tobytes()).hexdigest()


def run_case(name, build, kw, steps=STEPS):
    sc = build()
    o = oracle.Oracle(sc, phys_capacity=8 * sc.n_particles, **kw)
    o.init_particles()
    o.probe_enable(ref_cycle.REF_PROBE_CAPACITY)
    R = ref_cycle.RefCycle(o, probes=True)
    rec = []
    for k in range(steps):
        R.step()
        row = {}
        for p, label in ((0, "leaving"), (1, "division")):
            rv, _ = R.probe(p)
            ov, _ = o.probe_read(p)
            if not (len(rv) == len(ov) and np.array_equal(rv.view(np.uint64), ov.view(np.uint64))):
                raise SystemExit(f"{name} step {k}: the {label} probes of the oracle and the reference differ")
            row[label] = [len(rv), probe_digest(rv)]
        rec.append(row)
    R.close()
    return rec


def main():
    oracle.build()
    if not ref_cycle.available(probes=True):
        raise SystemExit("oracle/_ref/libbmc_ref_probe.so is not built (make -C oracle/refbuild REF=...)")
    out = {"steps": STEPS, "capacity": ref_cycle.REF_PROBE_CAPACITY, "cases": {}}
    for name, build, kw in cycle_cases():
        out["cases"][name] = run_case(name, build, kw)
        last = out["cases"][name][-1]
        print(name, "leaving", last["leaving"][0], "division", last["division"][0])
    with open(os.path.join(HERE, "ref_probes.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
