"""The FP64 form's Newton-refined quotient, reciprocal and square root (the forms its face-flux and
sweep kernels use in place of the IEEE division and root) against the IEEE operations, on the device,
through the C-ABI. The bar is two units in the last place, over the magnitudes the path meets
(densities, pressures, sums of squares with their 1e-6 regularisation, tangential velocities near the
Roe flux's 1e-8 regularisation) and a wide range of exponents besides."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ULP = 2


def ulps(a, b):
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    assert np.all(np.signbit(a) == np.signbit(b))
    return np.abs(a.view(np.int64) - b.view(np.int64))


def _samples(rng, n):
    wide = 10.0 ** rng.uniform(-30.0, 30.0, n)
    path = 10.0 ** rng.uniform(-9.0, 6.0, n)
    near_one = rng.uniform(0.5, 2.0, n)
    x = np.concatenate([wide, path, near_one])
    return x * rng.choice([-1.0, 1.0], x.size)


def test_quotient_reciprocal_and_root_within_two_ulp(gpu_lib):
    rng = np.random.default_rng(7)
    x, y = _samples(rng, 1 << 18), _samples(rng, 1 << 18)
    # the device's IEEE operations are numpy's, bit for bit
    assert np.array_equal(gpu_lib.fp64_arith_check(3, x, y), x / y)
    assert np.array_equal(gpu_lib.fp64_arith_check(4, np.abs(x)), np.sqrt(np.abs(x)))
    assert ulps(gpu_lib.fp64_arith_check(0, x, y), x / y).max() <= MAX_ULP
    assert ulps(gpu_lib.fp64_arith_check(2, y), 1.0 / y).max() <= MAX_ULP
    assert ulps(gpu_lib.fp64_arith_check(1, np.abs(x)), np.sqrt(np.abs(x))).max() <= MAX_ULP
