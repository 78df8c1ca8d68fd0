"""The reference's SimpleAcetate model (apps/libs/models/public/models/
simple_acetate.hpp): its draw functions (own logarithm and exponential from
IEEE operations, the reference's Winitzki erfinv, truncated-normal and
log-normal draws) against numpy/scipy, the model's invariants in the CPU
restatement, and the GPU kernels against the restatement bit for bit."""
import math

import numpy as np
import pytest

from bmc import scenarios


def test_log_and_exp_are_accurate(oracle_mod):
    L = oracle_mod.lib()
    rng = np.random.default_rng(3)
    xs = np.concatenate([10.0 ** rng.uniform(-300, 300, 4000), rng.uniform(0.5, 2.0, 4000),
                         [1.0, 2.0, 0.5, 5e-324, 1.7976931348623157e308]])
    for x in xs:
        got, ref = L.orc_sa_log(float(x)), math.log(float(x))
        assert abs(got - ref) <= 4e-16 * max(1.0, abs(ref)), x
    for x in rng.uniform(-700, 700, 4000):
        got, ref = L.orc_sa_exp(float(x)), math.exp(float(x))
        assert abs(got - ref) <= 2e-15 * ref, x
    assert L.orc_sa_exp(-800.0) == 0.0 and math.isinf(L.orc_sa_exp(800.0))
    assert math.isinf(L.orc_sa_log(0.0)) and math.isnan(L.orc_sa_log(-1.0))


def test_winitzki_erfinv_within_its_published_error(oracle_mod):
    special = pytest.importorskip("scipy.special")
    L = oracle_mod.lib()
    for x in np.linspace(-0.999, 0.999, 2001):
        got, ref = L.orc_sa_erfinv(float(x)), float(special.erfinv(x))
        assert abs(got - ref) <= 6e-3 * max(1.0, abs(ref)), x  # the approximation, not the code


def test_truncated_normal_stays_within_its_bounds(oracle_mod):
    L = oracle_mod.lib()
    lm = np.float32(2e-6)
    sd = np.float32(float(lm) / 10.0)
    lo, hi = 0.7 * float(lm), 1.3 * float(lm)
    u = (np.arange(1, 1 << 12, dtype=np.float64) / (1 << 12)).astype(np.float32)
    v = np.array([L.orc_sa_truncnorm(float(x), float(lm), float(sd), float.fromhex("0x1.61de2p-10"),
                                     float.fromhex("0x1.ff4f1p-1")) for x in u])
    assert np.all(np.diff(v) >= 0)  # a quantile function
    assert v.min() >= lo * 0.995 and v.max() <= hi * 1.005  # Winitzki's error at the tails
    assert abs(np.median(v) - float(lm)) < 0.01 * float(lm)


def test_model_invariants_in_the_restatement(oracle_mod):
    sc = scenarios.small_ring(20000, model=scenarios.simple_acetate(), feeds=True)
    o = oracle_mod.Oracle(sc)
    o.init_particles()
    st = o.particles()["state"]
    lm = 2e-6
    assert st[0].min() >= 0.7 * lm / 2 * 0.99 and st[0].max() <= 1.3 * lm * 1.01
    assert np.all(st[2] == np.float32(2e-6 / 3600.0) / np.float32(2.0))
    births = 0
    for _ in range(200):
        births += o.step()["births"]
    assert births > 1000
    st = o.particles()["state"]
    assert np.all(np.isfinite(st))
    assert np.all(st[4] == st[5] + st[6])  # a_e = uptake of glucose + acetate
    assert np.all(st[7] <= 0)  # glucose is consumed
    assert np.all(o.src[:, 0] <= 0)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [None, (256, 2, 0)])
def test_gpu_simple_acetate_matches_oracle(oracle_mod, shape):
    from test_gpu_parity import assert_same_liquid, assert_same_particles, assert_same_stats, make_pair

    sc = scenarios.small_ring(20000, model=scenarios.simple_acetate(), feeds=True)
    g, o = make_pair(oracle_mod, sc)
    if shape:
        g.set_shape(*shape)
    assert_same_particles(g, o, "init")
    births = 0
    for k in range(60):
        gs, os_ = g.step(), o.step()
        assert_same_stats(gs, os_, f"step {k}")
        assert_same_liquid(g, o, f"step {k}")
        births += gs["births"]
    assert births > 0
    assert_same_particles(g, o, "end")


def test_lognormal_division_draw_keeps_the_mean(oracle_mod):
    """a_p of a daughter ~ LogNormal(log(a_e) - s^2/2, s), s = 0.2
    (simple_acetate.hpp L226-L233): its mean is the mother's a_e.  The
    draw is exp(mu + s sqrt2 erfinv(2u - 1)); over a fine grid of u the mean
    must come out at a_e to within the erfinv approximation."""
    L = oracle_mod.lib()
    a_e, s = 3.7e-10, 0.2
    mu = L.orc_sa_log(a_e) - s * s / 2
    u = (np.arange(20000) + 0.5) / 20000
    z = np.array([math.sqrt(2.0) * L.orc_sa_erfinv(2 * x - 1) for x in u])
    z = np.clip(z, -5 * math.sqrt(2.0), 5 * math.sqrt(2.0))
    draws = np.array([L.orc_sa_exp(mu + s * v) for v in z])
    assert abs(draws.mean() / a_e - 1.0) < 5e-3
    assert abs(np.log(draws).std() - s) < 5e-3
