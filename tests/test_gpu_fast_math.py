"""Error bounds of the reciprocal and square root of the fast precisions.

fp64_fast replaces IEEE division and the library square root by
Newton-Raphson refinements of the hardware estimates (physics_fast.cuh:
`rcp_t`, two Newton steps from rcp.approx.ftz.f64; `sqrt_t`, one Newton step
folded into x*y0 plus one residual correction from rsqrt.approx.ftz.f64).
The FP32 form uses one Newton step from rcp.approx.ftz.f32 and the hardware
square-root approximation.  These tests evaluate them on the GPU over a
log-spaced sweep of the whole normal range (plus random mantissas) and bound
their error in units in the last place against the correctly rounded
values, which CUDA's IEEE division and square root return (checked here
too, against numpy's).  They also pin the flush-to-zero edges, where the
hardware estimates treat subnormal values as zero: the solver never feeds
them (densities, pressures and sound speeds of a state are normal numbers).
"""
import numpy as np
import pytest

ib = pytest.importorskip("ibtfo_gb300")

pytestmark = pytest.mark.gpu


def sweep64(lo_exp, hi_exp, n=200_001, seed=3):
    rng = np.random.default_rng(seed)
    e = np.linspace(lo_exp, hi_exp, n)
    x = np.ldexp(1.0 + rng.random(n), np.floor(e).astype(np.int64))
    return np.concatenate([x, np.ldexp(1.0, np.arange(lo_exp, hi_exp + 1))])


def ulp_err(y, ref):
    return np.abs(y - ref) / np.spacing(np.abs(ref))


def test_ieee_reference_matches_numpy():
    x = sweep64(-1000, 1000, n=50_001)
    assert np.array_equal(ib.fast_math_eval("div_f64", x), 1.0 / x)
    assert np.array_equal(ib.fast_math_eval("libsqrt_f64", x), np.sqrt(x))


def test_rcp_f64_within_one_ulp():
    x = sweep64(-1021, 1020)  # 1/x stays a normal number
    x = np.concatenate([x, -x])
    y = ib.fast_math_eval("rcp_f64", x)
    ref = ib.fast_math_eval("div_f64", x)
    err = ulp_err(y, ref)
    assert err.max() <= 1.0, f"rcp_t: {err.max():.3f} ulp at x = {x[err.argmax()]!r}"
    # most values are the correctly rounded one
    assert (y == ref).mean() > 0.9


def test_sqrt_f64_within_one_ulp():
    x = sweep64(-1022, 1023)
    y = ib.fast_math_eval("sqrt_f64", x)
    ref = ib.fast_math_eval("libsqrt_f64", x)
    err = ulp_err(y, ref)
    assert err.max() <= 1.0, f"sqrt_t: {err.max():.3f} ulp at x = {x[err.argmax()]!r}"
    assert (y == ref).mean() > 0.9


def test_f64_edges():
    tiny = np.array([5e-324, 1e-310, 2.0 ** -1023])  # subnormal
    # sqrt_t hands zero, subnormal, negative and non-finite values to the library square root
    special = np.concatenate([tiny, [0.0, -0.0, -1.0, np.inf, np.nan]])
    ys = ib.fast_math_eval("sqrt_f64", special)
    ref = ib.fast_math_eval("libsqrt_f64", special)
    assert np.array_equal(ys, ref, equal_nan=True)
    # rcp_t: the estimate flushes a subnormal input to zero, so the result is not finite
    assert not np.isfinite(ib.fast_math_eval("rcp_f64", tiny)).any()
    # and a result below the normal range flushes to zero
    big = np.array([2.0 ** 1023, 1.5 * 2.0 ** 1023])
    assert np.array_equal(ib.fast_math_eval("rcp_f64", big), np.zeros(2))


def sweep32(n=200_001, seed=5):
    rng = np.random.default_rng(seed)
    e = np.linspace(-125, 125, n)
    x = np.ldexp(1.0 + rng.random(n), np.floor(e).astype(np.int64)).astype(np.float32)
    return x.astype(np.float64)


def test_fp32_rcp_and_sqrt():
    x = sweep32()
    ref_div = ib.fast_math_eval("div_f32", x).astype(np.float32)
    assert np.array_equal(ref_div, (np.float32(1.0) / x.astype(np.float32)))
    y = ib.fast_math_eval("rcp_f32", x).astype(np.float32)
    err = ulp_err(y, ref_div)
    assert err.max() <= 1.0, f"FP32 rcp_t: {err.max():.3f} ulp"
    ref_sqrt = ib.fast_math_eval("libsqrt_f32", x).astype(np.float32)
    assert np.array_equal(ref_sqrt, np.sqrt(x.astype(np.float32)))
    ys = ib.fast_math_eval("sqrt_f32", x).astype(np.float32)
    err = ulp_err(ys, ref_sqrt)
    assert err.max() <= 2.0, f"FP32 sqrt_t: {err.max():.3f} ulp"
