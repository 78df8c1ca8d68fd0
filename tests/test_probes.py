"""Time-event probes of the CPU restatement (the reference's
Simulation::Probes, apps/libs/simulation/public/simulation/probe.hpp
L38-L146, with use_probe).

The buffer semantics are checked with the sequences of the reference's own
apps/libs/simulation/tests/test_probes.cpp (test_probes_set / _get /
_clear): a value is stored while the buffer has room and set reports it,
the buffer needs exporting once the count reaches its size, get returns the
stored values in order, clear empties it.  Then a stepped scenario: every
division request and every exit of a step is one event of its probe."""
import numpy as np
import pytest

from bmc import scenarios

LEAVING, DIVISION = 0, 1


def _oracle(oracle_mod, cap):
    sc = scenarios.zero_d(2000, model=scenarios.monod(f64=True, m_div=1.0), outlet=True)
    sc.feeds[0].flow = 1e-3
    o = oracle_mod.Oracle(sc, phys_capacity=2048)
    o.init_particles()
    o.probe_enable(cap)
    return o


def need_export(o, probe):
    return o.probe_read(probe)[1] >= int(o.s.probe_cap)


def test_set_as_the_reference_test(oracle_mod):
    """test_probes_set: buffer of 2."""
    o = _oracle(oracle_mod, 2)
    assert o.probe_set(DIVISION, 1.0)
    assert not need_export(o, DIVISION)
    assert o.probe_set(DIVISION, 2.0)
    assert need_export(o, DIVISION)
    assert not o.probe_set(DIVISION, 3.0)


def test_get_as_the_reference_test(oracle_mod):
    """test_probes_get: buffer of 10, one value too many."""
    o = _oracle(oracle_mod, 10)
    for i in range(10):
        assert o.probe_set(LEAVING, float(i))
    assert not o.probe_set(LEAVING, 55.0)
    assert need_export(o, LEAVING)
    values, count = o.probe_read(LEAVING)
    assert count == 11 and len(values) == 10
    assert np.array_equal(values, np.arange(10.0))


def test_clear_as_the_reference_test(oracle_mod):
    """test_probes_clear: buffer of 20, cleared and filled again."""
    o = _oracle(oracle_mod, 20)
    for i in range(20):
        assert o.probe_set(DIVISION, 2.0 * i)
    assert need_export(o, DIVISION)
    values, _ = o.probe_read(DIVISION)
    assert len(values) == 20 and values[2] == 4.0
    o.probe_clear(DIVISION)
    assert not need_export(o, DIVISION)
    assert o.probe_read(DIVISION) == (pytest.approx(np.zeros(0)), 0)
    for i in range(20):
        assert o.probe_set(DIVISION, 2.0 * i)
    assert need_export(o, DIVISION)
    assert o.probe_read(DIVISION)[0][2] == 4.0


def test_stepped_scenario_records_every_event(oracle_mod):
    """Division requests (refused ones included: the container is small)
    and exits of every step are events; the values are ages of the step:
    positive multiples of dt in float, leaving times at least one step."""
    o = _oracle(oracle_mod, 1 << 20)
    req = exits = overflow = 0
    for _ in range(8):
        o.step()
        st = o.stats()
        req += int(o.s.requested_divisions)
        exits += st["exits"]
        overflow += st["overflow"]
    assert overflow > 0 and exits > 0 and req > 0
    div, n_div = o.probe_read(DIVISION)
    left, n_left = o.probe_read(LEAVING)
    assert n_div == req == len(div)
    assert n_left == exits == len(left)
    dt = np.float32(o.scen.dt)
    for v in (div, left):
        assert np.all(v >= float(dt) * 0.999) and np.all(v <= 8 * float(dt) * 1.001)


def test_probes_off_record_nothing(oracle_mod):
    o = _oracle(oracle_mod, 0)
    o.run(4)
    for p in (LEAVING, DIVISION):
        assert o.probe_read(p) == (pytest.approx(np.zeros(0)), 0)
