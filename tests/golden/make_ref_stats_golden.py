"""Writes tests/golden/ref_stats.json: free-running statistics of the
reference's own particle cycle.

Needs the reference's compiled cycle (oracle/_ref/libbmc_ref.so, built where
the reference tree is present).  For each of 32 seeds the reference's cycle
functors and particle container (oracle/refbuild/ref_cycle.cpp) run the
SimpleAcetate 10-ring scenario of tests/test_statistics.py
(`reference_scenario`) for its 200 steps, drawing from their own
xorshift1024* stream (the generator family of the reference's Kokkos pool),
coupled to the oracle's liquid step, which receives the exact sums of the
reference's contribution operands (the reference's liquid step needs Eigen,
absent here).  The summary statistics of each finished run
(tests/stat_bands.py `summary`) are recorded; the tests compare the GPU and
the oracle, drawing from Philox, with them.

    python tests/golden/make_ref_stats_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "biocma-mcst_gb300"), os.path.join(ROOT, "oracle"), ROOT, os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import ref_cycle  # noqa: E402
from stat_bands import N_SEEDS, seeded, summary  # noqa: E402
from test_statistics import REFERENCE_SEED0, reference_scenario  # noqa: E402


def run(seed: int) -> list:
    sc = seeded(reference_scenario(), seed)
    o = oracle.Oracle(sc, phys_capacity=(sc.capacity + 1023) // 1024 * 1024)
    o.init_particles()
    n0 = o.n_used
    R = ref_cycle.RefCycle(o)
    births = R.run_free(sc.n_steps, seed)
    v = summary(R.particles(), o.C, sc.net.n_c, n0, n0 + births)
    R.close()
    return [float(x) for x in v]


def main():
    oracle.build()
    if not ref_cycle.available():
        raise SystemExit("oracle/_ref/libbmc_ref.so is not built (make -C oracle/refbuild REF=...)")
    rows = [run(REFERENCE_SEED0 + k) for k in range(N_SEEDS)]
    out = {"seeds": [REFERENCE_SEED0 + k for k in range(N_SEEDS)], "summaries": rows,
           "assert_failures": int(ref_cycle.ref_lib().ref_assert_failures())}
    with open(os.path.join(HERE, "ref_stats.json"), "w") as f:
        json.dump(out, f)
    a = np.array(rows)
    print("live", a[:, 20].mean(), "births", a[:, 21].mean())


if __name__ == "__main__":
    main()
