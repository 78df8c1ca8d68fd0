"""Serving form: requests admitted over time into a continuously re-formed
batch give, each, exactly the result the same request gives alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    ui = {8: np.uint64, 4: np.uint32}[a.dtype.itemsize]
    return a.shape == b.shape and bool(np.all((a.view(ui) == b.view(ui)) | (np.isnan(a) & np.isnan(b))))


def test_served_results_equal_alone():
    from bmc import serve
    from bmc.sim import GpuScenario

    reqs = serve.poisson_requests(rate=200.0, duration=0.15, seed=11, steps_lo=5, steps_hi=60,
                                  particle_scale=0.004)
    assert len(reqs) >= 10
    out = {}

    def keep(r, g):
        out[r.rid] = (g.particles(), g.liquid(), g.stats())

    srv = serve.Server(hbm_budget=2e9, chunk_steps=7)
    stats = srv.serve(reqs, on_finish=keep)
    assert stats["completed"] == len(reqs)
    assert srv.used == 0
    for r in reqs:
        assert r.latency is not None and r.latency >= 0
        g = GpuScenario(r.scen)
        g.run(r.steps)
        p_alone, l_alone = g.particles(), g.liquid()
        p_mix, l_mix, st = out[r.rid]
        assert st["step"] == r.steps
        for k in ("pos", "status", "id"):
            assert np.array_equal(p_alone[k], p_mix[k]), (r.rid, k)
        for k in ("state", "age_h", "age_d"):
            assert same_bits(p_alone[k], p_mix[k]), (r.rid, k)
        for k in ("C", "M", "src"):
            assert same_bits(l_alone[k], l_mix[k]), (r.rid, k)
        g.close()


def test_admission_respects_budget():
    from bmc import serve

    reqs = serve.poisson_requests(rate=400.0, duration=0.05, seed=3, steps_lo=3, steps_hi=10,
                                  particle_scale=0.004)
    biggest = max(serve.scenario_bytes(r.scen) for r in reqs)
    srv = serve.Server(hbm_budget=biggest * 2.5, chunk_steps=4)
    peak = {"used": 0}
    orig = srv.serve

    stats = srv.serve(reqs, on_finish=lambda r, g: peak.__setitem__("used", max(peak["used"], srv.used)))
    assert stats["completed"] == len(reqs)
    assert peak["used"] <= srv.budget
    del orig
