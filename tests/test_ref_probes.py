"""The oracle's time-event probes against the reference's own cycle built with
its probes on.

tests/golden/ref_probes.json records, per scenario and step, how many values
each probe of the reference's compiled cycle held (its use_probe build:
oracle/refbuild, oracle/_ref/libbmc_ref_probe.so) and the SHA-256 of their
float64 bytes, when run beside the oracle from the same container with the
oracle's concentrations and draws (tests/golden/make_ref_probes_golden.py).
Here the oracle runs the same scenarios alone and must hold the same values
every step: leaving times (ages(i, 0) at an exit) and division times
(ages(i, 1) at a division request), in slot order.  The GPU's probes equal
the oracle's (tests/test_gpu_probes.py), so these records tie them to the
reference as well.  Where the reference's probe build is present, a live run
compares the values themselves.
"""
import hashlib
import importlib.util
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _gen():
    spec = importlib.util.spec_from_file_location("make_ref_probes_golden",
                                                  os.path.join(HERE, "golden", "make_ref_probes_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "ref_probes.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def gen(oracle_mod):
    return _gen()


def test_records_exercise_both_probes(golden):
    last = [c[-1] for c in golden["cases"].values()]
    assert sum(r["leaving"][0] for r in last) > 3000
    assert sum(r["division"][0] for r in last) > 5000
    assert golden["capacity"] == 10000


@pytest.mark.parametrize("name", ["fixed_ring", "acetate_ring", "acetate_ring_scheduled_outlet",
                                  "fixed_ring_compact_every_step", "acetate_0d", "acetate_lattice"])
def test_oracle_probes_equal_the_reference(oracle_mod, golden, gen, name):
    build, kw = {n: (b, k) for n, b, k in gen.cycle_cases()}[name]
    sc = build()
    o = oracle_mod.Oracle(sc, phys_capacity=8 * sc.n_particles, **kw)
    o.init_particles()
    o.probe_enable(golden["capacity"])
    for k, rec in enumerate(golden["cases"][name]):
        o.step()
        for p, label in ((0, "leaving"), (1, "division")):
            values, _ = o.probe_read(p)
            n, digest = rec[label]
            assert len(values) == n, f"{name} step {k}: {label} count"
            assert hashlib.sha256(np.ascontiguousarray(values, np.float64).tobytes()).hexdigest() == digest, \
                f"{name} step {k}: {label} values"


def test_live_reference_probes_when_built(oracle_mod, gen):
    import ref_cycle

    if not ref_cycle.available(probes=True):
        pytest.skip("reference probe build not present here")
    name, build, kw = gen.cycle_cases()[1]
    rec = gen.run_case(name, build, kw, steps=12)  # raises on any difference
    assert rec[-1]["division"][0] > 0
