"""The cubic spline entry points against the reference's own spline.c,
compiled unchanged into oracle/_ref/libspline_ref.so by oracle/Makefile:
coefficients and values must be bit-identical (both compiled without FP
contraction), including the flags, the end conditions (default and known
slopes), extrapolation and the segment hint."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "libspline_ref.so")


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF):
        pytest.skip("reference spline not built (needs the reference sources)")
    lib = C.CDLL(REF)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.spline.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, dp, dp, dp, dp,
                           dp, ip]
    lib.seval.argtypes = [C.c_int, C.c_double, dp, dp, dp, dp, dp, ip]
    lib.seval.restype = C.c_double
    lib.deriv.argtypes = [C.c_int, C.c_double, dp, dp, dp, dp, ip]
    lib.deriv.restype = C.c_double
    lib.sinteg.argtypes = [C.c_int, C.c_double, dp, dp, dp, dp, dp, ip]
    lib.sinteg.restype = C.c_double
    return lib


def P(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ref_coeffs(ref, x, y, e1, e2, s1, s2):
    n = len(x)
    b, c, d = np.zeros(n), np.zeros(n), np.zeros(n)
    flag = C.c_int(-1)
    ref.spline(n, e1, e2, s1, s2, P(x), P(y), P(b), P(c), P(d), C.byref(flag))
    return b, c, d, flag.value


CASES = [(2, 0, 0), (3, 0, 0), (4, 0, 0), (4, 1, 1), (7, 1, 0), (25, 0, 1), (200, 0, 0),
         (200, 1, 1)]


@pytest.mark.parametrize("n,e1,e2", CASES)
def test_coefficients_and_values_bit_identical(pkg, ref, n, e1, e2):
    rng = np.random.default_rng(n * 10 + e1 * 2 + e2)
    x = np.cumsum(rng.uniform(0.05, 1.0, n))
    y = np.sin(x) + 0.1 * rng.normal(size=n)
    s1, s2 = 0.7, -1.3
    b, c, d, flag = ref_coeffs(ref, x.copy(), y.copy(), e1, e2, s1, s2)
    sp = pkg.Spline(x, y, e1, e2, s1, s2)
    assert sp.iflag == flag == 0
    assert np.array_equal(sp.b, b) and np.array_equal(sp.c, c) and np.array_equal(sp.d, d)
    # values, slopes, integrals: inside, at knots, outside; the hint carried
    us = np.concatenate([rng.uniform(x[0] - 1, x[-1] + 1, 50), x, [x[0] - 2.0, x[-1] + 3.0]])
    last_ref, last_ours = C.c_int(0), C.c_int(0)
    for u in us:
        for f_ref, f_ours in (
                (lambda: ref.seval(n, u, P(x), P(y), P(b), P(c), P(d), C.byref(last_ref)),
                 lambda: sp(u)),
                (lambda: ref.deriv(n, u, P(x), P(b), P(c), P(d), C.byref(last_ref)),
                 lambda: sp.deriv(u)),
                (lambda: ref.sinteg(n, u, P(x), P(y), P(b), P(c), P(d), C.byref(last_ref)),
                 lambda: sp.integral(u))):
            last_ref.value = sp.last.value
            vr = f_ref()
            vo = f_ours()
            assert vr == vo and last_ref.value == sp.last.value, (u, vr, vo)


def test_flags(pkg, ref):
    x = np.array([0.0, 1.0, 1.0, 2.0])
    y = np.zeros(4)
    assert pkg.Spline(x, y).iflag == 2 == ref_coeffs(ref, x, y, 0, 0, 0, 0)[3]
    assert pkg.Spline(x[:1], y[:1]).iflag == 1 == ref_coeffs(ref, x[:1], y[:1], 0, 0, 0, 0)[3]


def test_reproduces_a_cubic_exactly(pkg):
    """The default end conditions match third derivatives, so a cubic is
    reproduced to rounding."""
    x = np.linspace(-1.0, 2.0, 9)
    f = lambda t: 1.0 - 2.0 * t + 0.5 * t ** 2 + 0.25 * t ** 3
    sp = pkg.Spline(x, f(x))
    for u in (-0.7, 0.1, 1.33, 1.99):
        assert abs(sp(u) - f(u)) < 1e-12
        assert abs(sp.deriv(u) - (-2.0 + u + 0.75 * u ** 2)) < 1e-11
    F = lambda t: t - t ** 2 + t ** 3 / 6 + t ** 4 / 16
    assert abs(sp.integral(1.5) - (F(1.5) - F(-1.0))) < 1e-11
