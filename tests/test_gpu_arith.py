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


def test_split_into_an_fp32_pair(gpu_lib):
    # the mixed form's residual norm splits FP64 values into FP32 pairs by integer operations: the
    # pair holds 47 bits (hi truncated to 24, the rest rounded to 23), zeros and signs exactly
    rng = np.random.default_rng(11)
    w = 10.0 ** rng.uniform(-20.0, 20.0, 1 << 16) * rng.choice([-1.0, 1.0], 1 << 16)
    assert np.max(np.abs(gpu_lib.fp64_arith_check(5, w) - w) / np.abs(w)) <= 2.0 ** -47
    edge = np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 1.5 * 2.0 ** 127])
    assert np.array_equal(gpu_lib.fp64_arith_check(5, edge), edge)


def test_integer_conversions_equal_the_conversion_instructions(gpu_lib):
    # FP64 -> FP32 (round to nearest, ties to even) -> FP64 by integer operations against the
    # conversion instructions and numpy, bit for bit: random values over the whole FP32 range,
    # halfway cases (ties), the largest finite FP32 and just above, FP32 subnormal results, zeros
    rng = np.random.default_rng(17)
    x = 10.0 ** rng.uniform(-44.0, 38.5, 1 << 17) * rng.choice([-1.0, 1.0], 1 << 17)
    f = rng.uniform(1.0, 2.0, 1 << 14).astype(np.float32).astype(np.float64)
    ulp = np.spacing(f.astype(np.float32)).astype(np.float64)
    ties = np.concatenate([f + 0.5 * ulp, f - 0.25 * ulp, f + 0.5 * ulp * (1 + 2.0 ** -28)])
    edge = np.array([0.0, -0.0, float(np.finfo(np.float32).max), 3.4028235677973366e38, 1e39, -1e39,
                     2.0 ** -149, 2.0 ** -150, 1.5 * 2.0 ** -150, 2.0 ** -126, 2.0 ** -127, 1e-300, np.inf, -np.inf])
    for v in (x, ties, edge):
        got = gpu_lib.fp64_arith_check(6, v)
        want = gpu_lib.fp64_arith_check(7, v)
        assert np.array_equal(got.view(np.int64), want.view(np.int64))
        with np.errstate(over="ignore"):
            assert np.array_equal(got.view(np.int64), v.astype(np.float32).astype(np.float64).view(np.int64))
