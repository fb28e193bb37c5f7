"""Accuracy of the shared FP32 transcendentals (path-tracer_gb300/csrc/pt_fmath.h)
against double precision, and their special values."""
import numpy as np
import pytest

import oracle


def ulp_error(got, want):
    got = got.astype(np.float64)
    spacing = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    spacing = np.maximum(spacing, np.float64(np.finfo(np.float32).smallest_subnormal))
    return np.abs(got - want) / spacing


rng = np.random.default_rng(12345)


@pytest.mark.parametrize("lo,hi", [(0.0, 6.2831855), (-20.0, 20.0), (0.0, 1e-3)])
def test_sin_cos(lo, hi):
    x = rng.uniform(lo, hi, 200000).astype(np.float32)
    assert ulp_error(oracle.fmath("sin", x), np.sin(x.astype(np.float64))).max() <= 2.0
    c = oracle.fmath("cos", x)
    want = np.cos(x.astype(np.float64))
    # absolute error near zeros of cos is what matters for the shader
    assert np.abs(c - want).max() <= 2.5e-7
    assert ulp_error(c[np.abs(want) > 0.01], want[np.abs(want) > 0.01]).max() <= 2.0


def test_acos():
    x = np.concatenate([rng.uniform(-1, 1, 200000), [-1, -0.5, 0, 0.5, 1]]).astype(np.float32)
    got = oracle.fmath("acos", x)
    want = np.arccos(x.astype(np.float64))
    assert ulp_error(got, want).max() <= 2.0
    assert np.isnan(oracle.fmath("acos", np.array([1.5, np.nan], np.float32))).all()


def test_atan2():
    y = rng.normal(size=200000).astype(np.float32)
    x = rng.normal(size=200000).astype(np.float32)
    got = oracle.fmath("atan2", x, y)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert ulp_error(got, want).max() <= 3.0
    # C99 signed-zero conventions
    z = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0], np.float32)
    xs = np.array([0.0, 0.0, -0.0, -0.0, 0.0, 0.0], np.float32)
    np.testing.assert_array_equal(oracle.fmath("atan2", xs, z), np.arctan2(z, xs).astype(np.float32))


def test_pow_for_diffuse_roughness():
    r = np.concatenate([rng.uniform(0, 1, 200000), [1e-30, 1e-40, 0.5, 1.0]]).astype(np.float32)
    got = oracle.fmath("pow", r, np.full_like(r, 0.1))
    want = np.power(r.astype(np.float64), 0.1)
    err = ulp_error(got, want)
    # exp2 of a rounded float exponent: a few ulp for normal inputs, more for subnormals
    assert err[r >= 1e-6].max() <= 4.0
    assert err.max() <= 12.0
    assert oracle.fmath("pow", np.array([0.0], np.float32), np.array([0.1], np.float32))[0] == 0.0


def test_log2_exp2():
    x = np.exp(rng.uniform(-80, 80, 100000)).astype(np.float32)
    assert ulp_error(oracle.fmath("log2", x), np.log2(x.astype(np.float64))).max() <= 3.0
    t = rng.uniform(-140, 127, 100000).astype(np.float32)
    got = oracle.fmath("exp2", t)
    want = np.exp2(t.astype(np.float64))
    ok = want > 2.0 ** -126
    assert ulp_error(got[ok], want[ok]).max() <= 2.0


def test_sincos_equals_sin_and_cos():
    """The kernels take sin and cos of one argument through one shared reduction; the bits must be
    those of the separate functions the oracle uses."""
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(-10, 10, 200000), rng.uniform(0, 2 * np.pi, 200000),
                        np.array([0.0, -0.0, np.pi / 4, np.pi / 2, np.pi, 2 * np.pi])]).astype(np.float32)
    np.testing.assert_array_equal(oracle.fmath("sincos_sin", x).view(np.uint32), oracle.fmath("sin", x).view(np.uint32))
    np.testing.assert_array_equal(oracle.fmath("sincos_cos", x).view(np.uint32), oracle.fmath("cos", x).view(np.uint32))
