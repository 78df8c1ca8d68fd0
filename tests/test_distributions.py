"""The draw transformations of the path and the feed arithmetic, checked the
way the reference's own tests check them.

* apps/libs/mc/tests/test_rng_2.cpp: moments of the distributions drawn from
  the pool, each within 5 % relative of its theoretical value (the test's
  full-size tolerance; 0 when the theoretical moment is 0), bounds of the
  truncated normal (2, 2/3, [0, 4]), mean and variance of `norminv` on
  uniform draws (|mean| < 0.1, |var - 1| < 0.1).  Here the uniforms are the
  Philox draws of the path (four per particle id and step) and the
  transformations are the ones the models use: the standard normal by the
  reference's inverse-CDF form (the SimpleAcetate division's log-normal
  factor), the log-normal exp(mu + sigma z), the truncated normal of
  prng_extension.hpp (the SimpleAcetate l_max draws) and norminv.  Only the
  distributions the path draws are restated (the reference's skew-normal is
  drawn by no model on it).
* apps/libs/simulation/tests/test_feed.cpp: a constant feed keeps its flow,
  a linear feed is f0 + t df and an exponential feed f0 + exp(alpha t), to
  1e-12, at t = 0, 0.1, ... as the main loop accumulates it.
"""
import ctypes as ct
import math

import numpy as np
import pytest

N_IDS = 1_000_000  # 4e6 uniforms, 2e6 standard normals per draw lane pair
TOL = 0.05


def p(a):
    return ct.c_void_p(a.ctypes.data)


@pytest.fixture(scope="module")
def L(oracle_mod):
    L = oracle_mod.lib()
    L.orc_draw_table.argtypes = [ct.c_uint64, ct.c_void_p, ct.c_uint64, ct.c_uint32, ct.c_uint32, ct.c_void_p]
    L.orc_std_normal_table.argtypes = [ct.c_void_p, ct.c_uint64, ct.c_void_p]
    L.orc_truncnorm_table.argtypes = [ct.c_void_p, ct.c_uint64, ct.c_float, ct.c_float, ct.c_float, ct.c_float,
                                      ct.c_void_p]
    L.orc_pin_norminv_f.restype = ct.c_float
    L.orc_pin_norminv_f.argtypes = [ct.c_float, ct.c_float, ct.c_float]
    L.orc_feed_flow.restype = ct.c_double
    L.orc_feed_flow.argtypes = [ct.c_int32, ct.c_double, ct.c_double, ct.c_double, ct.c_double]
    return L


@pytest.fixture(scope="module")
def uniforms(L):
    ids = np.arange(N_IDS, dtype=np.uint32)
    d = np.zeros((N_IDS, 4), np.float32)
    L.orc_draw_table(1407, p(ids), N_IDS, 0, 1, p(d))
    return d.ravel()


def check_moment(empirical, theoretical, name, tol=TOL):
    err = abs(empirical - theoretical) / abs(theoretical) if theoretical != 0 else abs(empirical)
    assert err < tol, (name, empirical, theoretical, err)


def moments(x):
    x = np.asarray(x, np.float64)
    m = x.mean()
    v = (x * x).mean() - m * m
    sk = ((x ** 3).mean() - 3 * m * v - m ** 3) / v ** 1.5
    return m, v, sk


def test_uniform_draws_are_uniform(uniforms):
    m, v, sk = moments(uniforms)
    check_moment(m, 0.5, "mean")
    check_moment(v, 1.0 / 12.0, "variance")
    check_moment(sk, 0.0, "skewness")
    assert uniforms.min() > 0.0 and uniforms.max() < 1.0


def test_standard_normal_moments(L, uniforms):
    z = np.zeros(len(uniforms))
    L.orc_std_normal_table(p(uniforms), len(uniforms), p(z))
    m, v, sk = moments(z)
    check_moment(m, 0.0, "mean")
    check_moment(v, 1.0, "variance")
    check_moment(sk, 0.0, "skewness")
    assert np.isfinite(z).all()


def test_lognormal_moments(L, uniforms):
    """LogNormal(0, 1): mean e^(1/2), variance (e - 1) e, skewness
    (e + 2) sqrt(e - 1)."""
    z = np.zeros(len(uniforms))
    L.orc_std_normal_table(p(uniforms), len(uniforms), p(z))
    x = np.exp(z)
    m, v, sk = moments(x)
    e = math.e
    check_moment(m, math.exp(0.5), "mean")
    check_moment(v, (e - 1.0) * e, "variance")
    # the sample skewness of a log-normal converges slowly: 4e6 draws hold it
    # to a few per cent, as the reference's 4e7 hold it to its 5 %
    check_moment(sk, (e + 2.0) * math.sqrt(e - 1.0), "skewness", tol=0.1)


def test_truncated_normal_bounds_and_moments(L, uniforms):
    """TruncatedNormal(2, 2/3, [0, 4]) (test_truncated): every draw in
    [0, 4]; symmetric about 2 with variance sigma^2 (1 - 2 b phi(b) / (2
    Phi(b) - 1)), b = 3."""
    u = uniforms[:400_000].copy()
    y = np.zeros(len(u), np.float32)
    L.orc_truncnorm_table(p(u), len(u), 2.0, 2.0 / 3.0, 0.0, 4.0, p(y))
    assert y.min() >= 0.0 and y.max() <= 4.0
    b = 3.0
    phi = math.exp(-b * b / 2) / math.sqrt(2 * math.pi)
    big_phi = 0.5 * math.erfc(-b / math.sqrt(2))
    var = (2.0 / 3.0) ** 2 * (1 - 2 * b * phi / (2 * big_phi - 1))
    m, v, sk = moments(y)
    check_moment(m, 2.0, "mean")
    check_moment(v, var, "variance")
    check_moment(sk, 0.0, "skewness")


def test_norminv_mean_and_variance(L, uniforms):
    u = uniforms[:200_000]
    x = np.array([L.orc_pin_norminv_f(float(v), 0.0, 1.0) for v in u])
    assert abs(x.mean()) < 0.1
    assert abs(x.var(ddof=1) - 1.0) < 0.1


@pytest.mark.parametrize("kind,rate,expected", [
    (0, 0.0, lambda t: 1.0),
    (1, 0.1, lambda t: 1.0 + t * 0.1),
    (2, 0.1, lambda t: 1.0 + math.exp(t * 0.1)),
])
def test_feed_updates_as_the_reference_test(L, kind, rate, expected):
    """test_update_constant / _linear / _exp: f0 = 1, dt = 0.1, 12 updates at
    t accumulated by the main loop's sum of steps."""
    t = 0.0
    for _ in range(12):
        y = L.orc_feed_flow(kind, 1.0, 1.0, rate, t)
        assert abs(y - expected(t)) < 1e-12, (kind, t, y)
        t += 0.1
