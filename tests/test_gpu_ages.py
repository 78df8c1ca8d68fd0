"""The age step of the cycle kernels on the device.

The reference keeps ages in float and advances them with a double time
step, `ages(i, 0) += d_t` (MoveFunctor, apps/libs/simulation/public/
simulation/kernels/move_kernel.hpp L356), which rounds the sum to double and
then to float.  The kernels evaluate that with float and integer operations;
here they are held against numpy's float32(float64(a) + dt) on ages stepped
from zero, random ages, ages at powers of two, and time steps near half an
ulp of the ages (the rounding ties), bit for bit.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_age_add(a: np.ndarray, dt: float) -> np.ndarray:
    from bmc import _lib

    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.zeros_like(a)
    _lib.call("bmc_debug_age_add", ct.c_void_p(a.ctypes.data), len(a), dt, ct.c_void_p(out.ctypes.data))
    return out


def reference(a: np.ndarray, dt: float) -> np.ndarray:
    return (a.astype(np.float64) + dt).astype(np.float32)


@pytest.mark.parametrize("dt", [0.05, 0.1, 0.01, 1e-3, 1.0 / 3.0, 0.0625, 123.456])
def test_age_step_bit_exact(dt):
    rng = np.random.default_rng(int(dt * 1e6) % 1000)
    stepped = np.zeros(200_000, np.float32)
    for k in range(1, stepped.size):  # ages advanced step by step from zero
        stepped[k] = np.float32(np.float64(stepped[k - 1]) + dt)
    rand = rng.integers(0, 0x5F000000, size=2_000_000, dtype=np.uint32).view(np.float32)
    k = rng.integers(-30, 30, size=200_000)
    pow2 = np.ldexp(np.float32(1.0), k).astype(np.float32)
    below = np.nextafter(pow2, np.float32(0.0))
    a = np.concatenate([stepped, rand, pow2, below])
    got = device_age_add(a, dt)
    assert np.array_equal(got.view(np.uint32), reference(a, dt).view(np.uint32))


def test_age_step_at_rounding_ties():
    rng = np.random.default_rng(5)
    for _ in range(20):
        e = int(rng.integers(-20, 20))
        a = np.ldexp(1.0 + rng.integers(0, 1 << 23, size=100_000) / 2.0 ** 23, e).astype(np.float32)
        ulp = 2.0 ** (e - 23)
        dt = ulp * (0.5 * int(rng.integers(1, 8))) + 2.0 ** (e - 53) * int(rng.integers(-16, 17))
        if dt <= 0:
            dt = ulp / 2
        got = device_age_add(a, dt)
        assert np.array_equal(got.view(np.uint32), reference(a, dt).view(np.uint32)), dt


def test_float_quantisation_forms_agree():
    """The scaled-conversion quantisation of the cycle kernels equals the
    IEEE-field form and rint(v * 2^-e) (the oracle's quantisation) on
    random values, rounding ties, subnormals, zeros, clamped magnitudes,
    infinities and NaN, for quantum exponents across the float range."""
    from bmc import _lib

    rng = np.random.default_rng(17)
    qmax = 1 << 42
    for e in (-160, -126, -125, -90, -64, -40, -20, 0, 20, 100, 126, 127):
        v = np.concatenate([
            (rng.standard_normal(200000) * np.exp2(rng.uniform(-40, 50, 200000) + e)).astype(np.float32),
            # exact ties: odd multiples of half a quantum
            np.clip((rng.integers(-2**22, 2**22, 20000) * 2 + 1) * 2.0 ** (e - 1), -3e38, 3e38).astype(np.float32),
            np.array([0.0, -0.0, 1e-45, -1e-45, 1.1754942e-38, np.inf, -np.inf, np.nan, 3.4e38, -3.4e38],
                     np.float32)])
        out = np.zeros(2 * len(v), np.int64)
        _lib.call("bmc_debug_quantize", ct.c_void_p(v.ctypes.data), len(v), e, ct.c_void_p(out.ctypes.data))
        fast, bits = out[0::2], out[1::2]
        assert np.array_equal(fast, bits), e
        fin = np.isfinite(v)
        ref = np.rint(np.ldexp(v[fin].astype(np.float64), -e))
        ref = np.clip(ref, -qmax, qmax).astype(np.int64)
        sub = np.abs(v[fin]) < np.float32(1.1754944e-38)  # subnormal inputs quantise to 0 on the device
        assert np.array_equal(np.where(sub, 0, ref), fast[fin]), e
