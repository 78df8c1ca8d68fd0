"""Pins of the CPU restatement (the oracle) against published and
reference-derived known answers (tests/golden/)."""
import ctypes as ct
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_philox_known_answers(oracle_mod):
    for case in load("philox_kat.json"):
        out = oracle_mod.philox(case["ctr"], case["key"])
        assert [int(x) for x in out] == case["out"]


def test_u01_open_interval(oracle_mod):
    L = oracle_mod.lib()
    assert L.orc_u01(0) == 2.0 ** -24
    assert L.orc_u01(0xFFFFFFFF) == 1.0 - 2.0 ** -24
    assert 0.0 < L.orc_u01(0x80000000) < 1.0


def _oracle_for_row(oracle_mod, cdf, nbr):
    from bmc import scenarios

    sc = scenarios.small_ring(64, n_c=10)
    o = oracle_mod.Oracle(sc)
    K = len(cdf)
    o.cdf_row = np.zeros((10, K))
    o.cdf_row[:] = np.asarray(cdf)
    o.nbr_row = np.zeros((10, K), dtype=np.uint32)
    o.nbr_row[:] = np.asarray(nbr, dtype=np.uint32)
    o.s.cdf = o.cdf_row.ctypes.data
    o.s.neighbors = o.nbr_row.ctypes.data
    o.s.K = K
    return o


def test_move_search_hand_derived(oracle_mod):
    g = load("move_cases.json")
    o = _oracle_for_row(oracle_mod, g["cdf"], g["neighbors"])
    for case in g["cases"]:
        assert oracle_mod.lib().orc_find_next(ct.byref(o.s), 4, case["u"]) == case["next"]
    o = _oracle_for_row(oracle_mod, g["cdf4"], g["neighbors4"])
    for case in g["cases4"]:
        assert oracle_mod.lib().orc_find_next(ct.byref(o.s), 2, case["u"]) == case["next"]


def test_leave_probability_hand_derived():
    # probability_leaving<fast_tag>: dt * flow / volume > u, in double, u a float
    for case in load("move_cases.json")["leave"]:
        u = float(np.float32(case["u"]))
        assert ((case["dt"] * case["q"]) / case["v"] > u) == case["leave"]


def test_quantize_exact_sums(oracle_mod):
    L = oracle_mod.lib()
    cl = ct.c_int(0)
    e = -60
    vals = np.random.default_rng(1).normal(size=1000) * 2.0 ** -30
    q = [L.orc_quantize(float(v), e, 1 << 42, ct.byref(cl)) for v in vals]
    assert cl.value == 0
    # each quantum is the nearest multiple of 2^e
    for v, qi in zip(vals, q):
        assert abs(v * 2.0 ** -e - qi) <= 0.5
    # clamping
    assert L.orc_quantize(1.0, -60, 1 << 42, ct.byref(cl)) == 1 << 42 and cl.value == 1


def test_container_counts(oracle_mod):
    """apps/libs/mc/tests/test_container.cpp: divisions fill the buffer and
    merge appends them; removal of inactive particles shrinks n_used."""
    from bmc import scenarios

    g = load("container_counts.json")
    n = g["size"]
    sc = scenarios.zero_d(n_particles=n, outlet=False)
    o = oracle_mod.Oracle(sc, phys_capacity=int(math.ceil(n * g["allocation_factor_cuda"])))
    assert o.cap == n * g["allocation_factor_cuda"]
    o.init_particles()
    o.div_flag[: g["ndiv"]] = 1
    o.s.exits = 0
    o.post_cycle()
    assert o.n_used == g["after_merge"]
    assert o.s.births == g["ndiv"]
    # fresh container: kill to_remove particles, then remove them
    o = oracle_mod.Oracle(sc, phys_capacity=int(math.ceil(n * g["allocation_factor_cuda"])))
    o.init_particles()
    o.status[: g["to_remove"]] = 3
    oracle_mod.lib().orc_remove_inactive(ct.byref(o.s), g["to_remove"])
    assert o.n_used == g["after_remove"]
    assert (o.status[: o.n_used] == 0).all()
