"""Accuracy of the portable transcendentals (pmath.h) against glibc, on the
argument ranges the path tracer uses and beyond."""
import numpy as np
import pytest


def ulp_diff(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-2**31) - ia, ia)
    ib = np.where(ib < 0, np.int64(-2**31) - ib, ib)
    return np.abs(ia - ib)


rs = np.random.default_rng(0)


def test_sincos(oracle):
    x = np.concatenate([rs.uniform(0, 2 * np.pi, 200000), rs.uniform(-100, 100, 50000),
                        np.array([0.0, -0.0, np.pi, 2 * np.pi, 1e-30, -1e-30])]).astype(np.float32)
    s, c = oracle.pm_eval("sincos", x)
    ls, lc = oracle.pm_eval("sincos", x, libm=True)
    # compare in absolute terms near zeros of sin/cos, ulps elsewhere
    assert np.max(np.abs(s.astype(np.float64) - np.sin(x.astype(np.float64)))) < 3e-7
    assert np.max(np.abs(c.astype(np.float64) - np.cos(x.astype(np.float64)))) < 3e-7
    big = np.abs(ls) > 0.1
    assert ulp_diff(s[big], ls[big]).max() <= 2
    big = np.abs(lc) > 0.1
    assert ulp_diff(c[big], lc[big]).max() <= 2
    s, c = oracle.pm_eval("sincos", np.array([np.inf, np.nan], np.float32))
    assert np.isnan(s).all() and np.isnan(c).all()


def test_atan2(oracle):
    y = np.concatenate([rs.normal(size=200000), np.array([0, -0.0, 0, -0.0, 1, -1, np.inf, -np.inf])]).astype(np.float32)
    x = np.concatenate([rs.normal(size=200000), np.array([1, 1, -1, -1, 0, 0, np.inf, -np.inf])]).astype(np.float32)
    a = oracle.pm_eval("atan2", y, x)
    b = oracle.pm_eval("atan2", y, x, libm=True)
    assert ulp_diff(a, b).max() <= 2
    assert np.array_equal(np.signbit(a), np.signbit(b))


def test_acos(oracle):
    x = np.concatenate([rs.uniform(-1, 1, 300000), np.array([-1, 1, 0, -0.0, 0.5, -0.5, 0.99999994])]).astype(np.float32)
    a = oracle.pm_eval("acos", x)
    b = oracle.pm_eval("acos", x, libm=True)
    assert ulp_diff(a, b).max() <= 3
    assert np.isnan(oracle.pm_eval("acos", np.array([1.5, np.nan], np.float32))).all()


@pytest.mark.parametrize("y", [0.33333, 5.0, 1 / 2.2, 2.2, -1.5, 3.0, 0.5])
def test_pow_tracer_domains(oracle, y):
    x = np.concatenate([rs.uniform(0, 2, 200000), np.ldexp(rs.uniform(0.5, 1, 2000), -rs.integers(1, 40, 2000)),
                        np.array([0.0, 1.0, 2.0, 2.0 ** -32, 1e-38, 1e-45])]).astype(np.float32)
    yy = np.full_like(x, y)
    a = oracle.pm_eval("pow", x, yy)
    b = oracle.pm_eval("pow", x, yy, libm=True)
    finite = np.isfinite(b) & (b != 0) & (np.abs(b) > 1e-37)
    assert ulp_diff(a[finite], b[finite]).max() <= 8
    assert np.array_equal(a[~finite] == 0, b[~finite] == 0)


def test_pow_special_cases(oracle):
    cases = [(0.0, 2.0), (-0.0, 3.0), (0.0, -1.0), (-0.0, -3.0), (-2.0, 3.0), (-2.0, 2.0), (-2.0, 0.5),
             (1.0, np.nan), (np.nan, 0.0), (np.inf, 2.0), (np.inf, -2.0), (-np.inf, 3.0), (0.5, np.inf),
             (2.0, -np.inf), (-1.0, np.inf), (8.0, 1 / 3)]
    x = np.array([c[0] for c in cases], np.float32)
    y = np.array([c[1] for c in cases], np.float32)
    a = oracle.pm_eval("pow", x, y)
    b = oracle.pm_eval("pow", x, y, libm=True)
    same = (np.isnan(a) & np.isnan(b)) | (a == b) | (ulp_diff(a, b) <= 8)
    assert same.all(), list(zip(cases, a, b))
    assert np.array_equal(np.signbit(a[np.isfinite(a)]), np.signbit(b[np.isfinite(a)]))
