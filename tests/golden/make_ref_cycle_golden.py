"""Writes tests/golden/ref_cycle.json from the reference's own particle cycle.

Needs the reference tree (to build oracle/_ref/libbmc_ref.so:
`make -C oracle/refbuild REF=<reference tree>`, which __graft_entry__.build()
runs where the tree is present).  For each scenario below the reference's
compiled cycle (its cycle functors and particle container; see
oracle/refbuild/ref_cycle.cpp) runs beside the oracle from the same initial
container, with the oracle's concentrations and per-slot draws
(oracle/ref_cycle.py).  Every step the two containers are compared and the
script stops on any disagreement; it records, per step, what the reference
produced:

* the digest of its normalized container (oracle/ref_cycle.py `digest`),
  the particle count and the births, exits and moves its events counted;
* per contribution and compartment, the exact sum of the operands its
  scatter received (float64 bits), the sum of their magnitudes and its float
  scatter result (float32 bits).

Two more runs drive the reference with an oracle that emulates the scatter's
chunk early return (contribution_kernel.hpp Tag3D: a 32-particle chunk stops
at its first non-Idle particle); there the oracle's sources must equal the
reference's float scatter to float rounding until the first compaction
(afterwards the reference's last chunk also reads stale slots past the
container's end, which the emulation does not model).

    python tests/golden/make_ref_cycle_golden.py
"""
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
from bmc import networks, scenarios  # noqa: E402

STEPS = 40


def cases():
    """(name, scenario builder, Oracle keyword arguments); a builder returns
    a fresh Scenario."""

    def fixed_ring():
        return scenarios.small_ring(3000, model=scenarios.fixed_length(), feeds=True)

    def acetate_ring():
        return scenarios.small_ring(3000, model=scenarios.simple_acetate(), feeds=True, seed=11)

    def fixed_ring_compact_every_step():
        sc = scenarios.small_ring(2500, model=scenarios.fixed_length(), feeds=True, seed=7)
        sc.feeds[0].flow = 4e-4  # many exits
        sc.dead_ratio_threshold = 0.0
        sc.min_removal = 0
        return sc

    def acetate_0d():
        sc = scenarios.zero_d(2000, model=scenarios.simple_acetate(), outlet=True, seed=9)
        sc.feeds[0].flow = 5e-4
        return sc

    def acetate_lattice():
        sc = scenarios.small_ring(4000, model=scenarios.simple_acetate(), feeds=True, seed=13)
        net = networks.lattice_vortex(4, side=0.1, peak_velocity=0.05, noise=0.2, seed=5, max_courant=0.5, dt=sc.dt)
        sc.net = net
        sc.c0 = np.tile(sc.c0[:1], (net.n_c, 1))
        sc.feeds[0].outlet = net.n_c - 1
        sc.feeds[0].flow = 2e-5
        return sc

    def acetate_ring_scheduled_outlet():
        # the outlet's flow grows linearly from 1e-5 to 4e-4 m^3/s over the 40 steps
        sc = scenarios.small_ring(3000, model=scenarios.simple_acetate(), feeds=True, seed=17)
        fd = sc.feeds[0]
        fd.kind, fd.f0, fd.rate = scenarios.FEED_LINEAR, 1e-5, 1e-4
        return sc

    return [("fixed_ring", fixed_ring, {}), ("acetate_ring", acetate_ring, {}),
            ("acetate_ring_scheduled_outlet", acetate_ring_scheduled_outlet, {}),
            ("fixed_ring_compact_every_step", fixed_ring_compact_every_step, {}), ("acetate_0d", acetate_0d, {}),
            ("acetate_lattice", acetate_lattice, {}), ("fixed_ring_chunk_quirk", fixed_ring, {"quirk_tag3d": True}),
            ("acetate_ring_chunk_quirk", acetate_ring, {"quirk_tag3d": True})]


# float accumulation bound of the reference's scatter against exact sums,
# relative to the operands' magnitude sum
SCATTER_TOL = 1e-4


KEYS = ("count", "status", "state", "pos", "age_h", "age_d", "births", "exits", "overflow", "moves", "contrib")


def run_case(name, build, kw, steps=STEPS):
    sc = build()
    o = oracle.Oracle(sc, phys_capacity=8 * sc.n_particles, **kw)
    o.init_particles()
    R = ref_cycle.RefCycle(o)
    quirk = bool(kw.get("quirk_tag3d"))
    rec = dict(quirk=quirk, steps=[], totals=dict(births=0, exits=0, moves=0, compactions=0))
    compacted = False
    for k in range(steps):
        r = R.step()
        bad = {a: r[a] for a in KEYS if r.get(a) and not (quirk and a == "contrib")}
        if quirk and not compacted:
            dev = np.abs(r["src"] - r["scatter"]) > SCATTER_TOL * r["absum"] + 1e-300
            if dev.any():
                bad["chunk_quirk"] = int(dev.sum())
        compacted = compacted or bool(r["compacted"])
        if bad or r["digest_ref"] != r["digest_oracle"]:
            raise SystemExit(f"{name} step {k}: the oracle and the reference disagree: {bad}")
        rec["steps"].append(dict(
            digest=r["digest_ref"], n=r["n_ref"], births=r["births_n"], exits=r["exits_n"], moves=r["moves_n"],
            compacted=r["compacted"],
            exact=[int(v) for v in np.asarray(r["exact"], np.float64).ravel().view(np.uint64)],
            absum=[int(v) for v in np.asarray(r["absum"], np.float32).ravel().view(np.uint32)],
            scatter=[int(v) for v in np.asarray(r["scatter"], np.float32).ravel().view(np.uint32)]))
        t = rec["totals"]
        t["births"] += r["births_n"]
        t["exits"] += r["exits_n"]
        t["moves"] += r["moves_n"]
        t["compactions"] += r["compacted"]
    misses = R.misses()
    if misses:
        raise SystemExit(f"{name}: {misses} draws had no slot")
    R.close()
    return rec


def main():
    oracle.build()
    if not ref_cycle.available():
        raise SystemExit("oracle/_ref/libbmc_ref.so is not built (make -C oracle/refbuild REF=...)")
    out = {"steps": STEPS, "scatter_tol": SCATTER_TOL, "cases": {}}
    for name, build, kw in cases():
        out["cases"][name] = run_case(name, build, kw)
        print(name, out["cases"][name]["totals"])
    out["assert_failures"] = int(ref_cycle.ref_lib().ref_assert_failures())
    with open(os.path.join(HERE, "ref_cycle.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
