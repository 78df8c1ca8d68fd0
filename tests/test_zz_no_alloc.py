"""bmc_repartition_static: the allocation-free repartition entry point.

It serves callers that cannot allocate device memory where they ask for the
per-compartment particle counts: programs whose device memory is all handed
out in advance (a capped caching pool allocator, a serving loop admitting
work against an HBM budget), where an extra cudaMalloc fails, or that cannot
afford the device-wide synchronisation of cudaMalloc / cudaFree while other
streams run.  Its counters live in a static device array shared by every
call.  This test calls it through the C-ABI twice in a row, on scenarios of
different sizes (so the clearing of the shared array is exercised), and
checks each result against bmc_repartition, which allocates its counters.
Counts are integers: the comparison is exact.  The file is named so that
pytest collects it last.
"""
import ctypes as ct

import numpy as np
import pytest

from bmc import networks, scenarios

pytestmark = pytest.mark.gpu


def _counts(fn, g):
    out = np.zeros(g.scen.net.n_c, dtype=np.uint64)
    rc = getattr(g.lib, fn)(g.handle, ct.c_void_p(out.ctypes.data))
    assert rc == 0, g.lib.bmc_last_error()
    return out


def test_static_repartition_matches_allocating_one():
    from bmc.sim import GpuScenario

    big = scenarios.workload(2, n_particles=200_000)
    small = scenarios.small_ring(50_000, feeds=True)
    ga = GpuScenario(big)
    gb = GpuScenario(small)
    ga.run(3)
    gb.run(3)
    first = _counts("bmc_repartition_static", ga)  # 512 compartments
    assert np.array_equal(first, _counts("bmc_repartition", ga))
    assert int(first.sum()) == ga.stats()["n_used"] - ga.stats()["inactive"]
    second = _counts("bmc_repartition_static", gb)  # 10 compartments, after the larger call
    assert np.array_equal(second, _counts("bmc_repartition", gb))
    assert int(second.sum()) == gb.stats()["n_used"] - gb.stats()["inactive"]
    ga.close()
    gb.close()


def test_static_repartition_rejects_too_many_compartments():
    from bmc.sim import GpuScenario

    n_c = 65537
    net = networks.Network(n_c, np.full(n_c, 1e-3), np.zeros(0, np.int64), np.zeros(0, np.int64),
                           np.zeros(0), meta={"kind": "isolated"}).finalize()
    sc = scenarios.Scenario("isolated", net, scenarios.monod(), 4096, 1, np.full((n_c, 1), 5.0))
    g = GpuScenario(sc)
    out = np.zeros(n_c, dtype=np.uint64)
    rc = g.lib.bmc_repartition_static(g.handle, ct.c_void_p(out.ctypes.data))
    assert rc == -4  # BMC_E_CAPACITY
    assert b"65536" in g.lib.bmc_last_error()
    g.close()
