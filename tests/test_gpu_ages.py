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
