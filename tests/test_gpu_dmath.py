"""The table-driven binary64 log and exp that setvset's Ganser drag
iteration uses in place of pow (f3d_dmath_eval), against an evaluation in
extended precision (numpy longdouble: 64-bit significand on x86, IEEE quad
on Arm).

Bounds: exp within 3 ulp of the exact value; log within 3 ulp plus 1.2e-16
absolute (the breakpoint tables hold log c to half an ulp of values up to
ln 2, which bounds the absolute error of results near 0; the iteration
only exponentiates the log, so absolute accuracy is what it needs)."""
import numpy as np
import pytest

import fall3d_gb300 as F

pytestmark = pytest.mark.gpu


def _ulp(v):
    return np.spacing(np.abs(v.astype(np.float64)))


def test_log_accuracy():
    rng = np.random.default_rng(5)
    x = np.concatenate([
        10.0 ** rng.uniform(-12, 12, 200000),          # Reynolds-number range and beyond
        1.0 + rng.uniform(-1e-3, 1e-3, 20000),          # around 1 (both sides of the binade)
        np.array([1.0, 2.0, 0.5, 3305.0, 1e-300, 1e300, 5e-324, np.nextafter(1.0, 0.0)]),
    ])
    y = F.dmath_eval(0, x)
    t = np.log(x.astype(np.longdouble))
    err = np.abs(y.astype(np.longdouble) - t)
    bound = 3 * _ulp(t) + 1.2e-16
    assert np.all(err <= bound), (x[np.argmax(err / bound)], np.max(err / bound))
    assert abs(y[np.where(x == 1.0)[0][0]]) < 1e-17


def test_exp_accuracy():
    rng = np.random.default_rng(6)
    a = np.concatenate([
        rng.uniform(-30, 30, 200000),                   # the iteration's range
        rng.uniform(-700, 700, 20000),
        rng.uniform(-1e-6, 1e-6, 5000),
        np.array([0.0, 1.0, -1.0, 700.0, -700.0, 709.0, -745.0, 0.5 * np.log(2.0)]),
    ])
    y = F.dmath_eval(1, a)
    t = np.exp(a.astype(np.longdouble))
    finite = np.isfinite(t) & (t < np.finfo(np.float64).max) & (t > np.finfo(np.float64).tiny)
    err = np.abs(y[finite].astype(np.longdouble) - t[finite])
    bound = 3 * _ulp(t[finite])
    assert np.all(err <= bound), (a[finite][np.argmax(err / bound)], np.max(err / bound))
    assert y[np.where(a == 0.0)[0][0]] == 1.0


def test_pow_as_used_by_the_drag_iteration():
    # R^0.6567 / R = exp(0.6567 L - L), L = log R, over the Reynolds range
    rng = np.random.default_rng(7)
    R = 10.0 ** rng.uniform(-6, 7, 100000)
    L = F.dmath_eval(0, R)
    P = F.dmath_eval(1, 0.6567 * L - L)
    t = R.astype(np.longdouble) ** np.longdouble(0.6567) / R.astype(np.longdouble)
    rel = np.abs(P.astype(np.longdouble) - t) / t
    assert float(np.max(rel)) < 4e-15


def test_rejects_bad_op():
    with pytest.raises(F.F3DError):
        F.dmath_eval(3, np.ones(4))


def test_quotient_from_reciprocal_is_the_ieee_quotient():
    """op 2: RN(a/b) from RN(1/b) by Markstein's correction, as the plain
    form's limiter (m/dx) and diffz (c/rho) divide: bit for bit the IEEE
    quotient, across magnitudes, signed zeros, subnormals and non-finite
    operands (the guarded ones take the division)."""
    rng = np.random.default_rng(8)
    n = 2_000_000
    with np.errstate(over="ignore"):  # magnitudes past the binary64 range become infinities
        a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-310, 310, n) * rng.uniform(1.0, 10.0, n)
        b = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-310, 310, n) * rng.uniform(1.0, 10.0, n)
    # the operands of the sweeps: concentrations over densities and grid spacings
    a[: n // 4] = 10.0 ** rng.uniform(-40, 3, n // 4)
    b[: n // 4] = rng.uniform(0.05, 1.4, n // 4)
    a[n // 4: n // 2] = rng.uniform(0.0, 1e-6, n // 4)
    b[n // 4: n // 2] = rng.choice([0.01, 0.025, 0.1, 1000.0, 2500.0], n // 4)
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                        np.inf, -np.inf, np.nan, 1.0, 3.0, 2.0 ** -900, 2.0 ** 900])
    sa, sb = np.meshgrid(special, special)
    a = np.concatenate([a, sa.ravel()])
    b = np.concatenate([b, sb.ravel()])
    x = np.empty(2 * a.size)
    x[0::2], x[1::2] = a, b
    y = F.dmath_eval(2, x)
    with np.errstate(all="ignore"):
        t = a / b
    nan = np.isnan(t)
    assert np.array_equal(np.isnan(y), nan)
    bad = np.nonzero(y[~nan].view(np.uint64) != t[~nan].view(np.uint64))[0]
    assert bad.size == 0, (bad.size, a[~nan][bad[:3]], b[~nan][bad[:3]])
