"""Portable exp/log/cbrt (wr_math.h): accuracy on the host, identity on the device."""
import math

import numpy as np
import pytest


def _ulp_error(got, exact):
    import mpmath as mp
    if exact == 0:
        return 0.0 if got == 0 else math.inf
    m, k = mp.frexp(exact)
    return float(abs(mp.mpf(got) - exact) / mp.ldexp(1, max(int(k) - 53, -1074)))


def _samples(rng, kind, n):
    if kind == "exp":
        parts = [rng.uniform(-708, 709.7, n), rng.uniform(-1, 1, n), rng.uniform(-1e-8, 1e-8, n),
                 rng.uniform(-60, 60, n)]
    elif kind == "log":
        parts = [10 ** rng.uniform(-307, 307, n), rng.uniform(0.99, 1.01, n), 1 + rng.uniform(-1e-9, 1e-9, n),
                 10 ** rng.uniform(-323, -308, n)]
    else:
        parts = [10 ** rng.uniform(-300, 300, n), -(10 ** rng.uniform(-30, 30, n)), 10 ** rng.uniform(-320, -308, n)]
    return np.concatenate(parts)


@pytest.mark.parametrize("fn,bound", [("exp", 0.51), ("log", 0.51), ("cbrt", 1.0)])
def test_accuracy_vs_mpmath(oracle_port, fn, bound):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 120
    ref = {"exp": mp.exp, "log": mp.log, "cbrt": lambda v: mp.sign(v) * mp.cbrt(abs(v))}[fn]
    f = getattr(oracle_port, fn)
    rng = np.random.default_rng(11)
    worst = 0.0
    for x in _samples(rng, fn, 1500):
        x = float(x)
        worst = max(worst, _ulp_error(f(x), ref(mp.mpf(x))))
    assert worst < bound, worst


def test_special_values(oracle_port):
    o = oracle_port
    inf, nan = math.inf, math.nan
    assert o.exp(0.0) == 1.0 and o.exp(-0.0) == 1.0
    assert o.exp(inf) == inf and o.exp(-inf) == 0.0 and math.isnan(o.exp(nan))
    assert o.exp(710.0) == inf and o.exp(-746.0) == 0.0
    assert o.exp(1.0) == math.exp(1.0)
    assert 0 < o.exp(-740.0) < 2.3e-308  # subnormal result
    assert o.log(1.0) == 0.0 and o.log(0.0) == -inf and math.isnan(o.log(-1.0))
    assert o.log(inf) == inf and math.isnan(o.log(nan))
    assert o.log(2.0) == math.log(2.0) and o.log(10.0) == math.log(10.0)
    assert o.log(5e-324) == pytest.approx(-744.4400719213812, rel=1e-15)
    assert o.cbrt(27.0) == 3.0 and o.cbrt(-8.0) == -2.0 and o.cbrt(0.0) == 0.0
    assert math.copysign(1.0, o.cbrt(-0.0)) == -1.0


def test_agreement_with_c_library(oracle_port):
    """Nearly correctly rounded, so the C library's results are reproduced almost
    always; differences are single-ulp."""
    rng = np.random.default_rng(5)
    xs = rng.uniform(-50, 50, 20000)
    same = sum(oracle_port.exp(float(x)) == math.exp(float(x)) for x in xs)
    assert same / len(xs) > 0.99
    ys = 10 ** rng.uniform(-30, 30, 20000)
    same = sum(oracle_port.log(float(y)) == math.log(float(y)) for y in ys)
    assert same / len(ys) > 0.99


@pytest.mark.gpu
@pytest.mark.parametrize("fn", [0, 1, 2])
def test_device_equals_host_bitwise(wr, gpu, oracle_port, fn):
    import ctypes
    rng = np.random.default_rng(17 + fn)
    kind = ("exp", "log", "cbrt")[fn]
    x = np.ascontiguousarray(np.concatenate([_samples(rng, kind, 50000),
                                             np.array([0.0, -0.0, math.inf, -math.inf, math.nan, 1.0, 5e-324])]))
    out = np.zeros_like(x)
    L = wr.lib()
    L.wr_diag_math.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    assert L.wr_diag_math(len(x), x.ctypes.data, fn, wr.MATH_PORTABLE, out.ctypes.data) == 1
    f = (oracle_port.exp, oracle_port.log, oracle_port.cbrt)[fn]
    host = np.array([f(float(v)) for v in x])
    assert out.view(np.uint64).tolist() == host.view(np.uint64).tolist()


def _div_cases(rng, n):
    a = 10 ** rng.uniform(-300, 300, n) * rng.choice([-1.0, 1.0], n)
    b = 10 ** rng.uniform(-300, 300, n) * rng.choice([-1.0, 1.0], n)
    ma = rng.integers(2**52, 2**53, n).astype(np.float64) * 2.0**-52
    mb = rng.integers(2**52, 2**53, n).astype(np.float64) * 2.0**-52
    special = np.array([0.0, -0.0, 1.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308,
                        1.7976931348623157e308, 3.0, 0.1])
    sa, sb = np.meshgrid(special, special)
    return (np.concatenate([a, ma, mb, np.nextafter(ma, 3.0), sa.ravel()]),
            np.concatenate([b, mb, ma, mb, sb.ravel()]))


def test_integer_division_is_ieee_on_host(oracle_port):
    """wr_div_int (the device division) computed on the host equals a / b."""
    import ctypes
    f = oracle_port.lib.wro_div_int
    f.restype, f.argtypes = ctypes.c_double, [ctypes.c_double, ctypes.c_double]
    a, b = _div_cases(np.random.default_rng(23), 20000)
    with np.errstate(all="ignore"):
        want = a / b
    got = np.array([f(float(x), float(y)) for x, y in zip(a, b)])
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), (a[~same][:3], b[~same][:3])


@pytest.mark.gpu
def test_integer_division_is_ieee_on_device(wr, gpu):
    import ctypes
    a, b = _div_cases(np.random.default_rng(29), 400000)
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    out = np.zeros_like(a)
    L = wr.lib()
    L.wr_diag_div.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert L.wr_diag_div(len(a), a.ctypes.data, b.ctypes.data, out.ctypes.data) == 1
    with np.errstate(all="ignore"):
        want = a / b
    same = (out.view(np.uint64) == want.view(np.uint64)) | (np.isnan(out) & np.isnan(want))
    assert same.all(), (a[~same][:3], b[~same][:3])
