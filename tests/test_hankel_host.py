"""Accuracy of the device Hankel evaluator (bem2d_gb300/csrc/hankel.cuh).

The evaluator is header-only and compiles for the host too; this builds it
with g++ and checks H0, H1 against mpmath (50 digits) and against the POSIX
libm Bessel functions that stand in for GSL in the oracle.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def hk(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("hk") / "libhk.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared",
                    "-I" + os.path.join(ROOT, "bem2d_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "hankel_host.cpp"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)

    def f(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        o = np.zeros((len(x), 4))
        lib.hankel01_d_host(ctypes.c_int(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                            o.ctypes.data_as(ctypes.c_void_p))
        return o[:, 0] + 1j * o[:, 1], o[:, 2] + 1j * o[:, 3]
    return f


def test_against_mpmath(hk):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    rng = np.random.default_rng(7)
    x = np.concatenate([10 ** rng.uniform(-9, 4.3, 1500), np.linspace(3.95, 4.05, 21),
                        np.linspace(7.95, 8.05, 21), [4.0, 8.0]])
    h0, h1 = hk(x)
    e0 = max(abs(complex(h0[i]) - complex(mp.hankel1(0, xi))) / abs(mp.hankel1(0, xi))
             for i, xi in enumerate(x))
    e1 = max(abs(complex(h1[i]) - complex(mp.hankel1(1, xi))) / abs(mp.hankel1(1, xi))
             for i, xi in enumerate(x))
    # stated accuracy of the FP64 evaluator: 1e-15 relative to |H|
    assert e0 < 1e-15 and e1 < 1e-15, (e0, e1)


def test_against_libm(hk):
    """POSIX libm j0/j1/y0/y1 (the oracle's stand-in for GSL)."""
    libm = ctypes.CDLL("libm.so.6")
    f = {}
    for name in ("j0", "j1", "y0", "y1"):
        fn = getattr(libm, name)
        fn.restype = ctypes.c_double
        fn.argtypes = [ctypes.c_double]
        f[name] = np.vectorize(fn)
    x = np.linspace(1e-3, 2e4, 40001)
    h0, h1 = hk(x)
    r0 = np.abs(h0 - (f["j0"](x) + 1j * f["y0"](x))) / np.abs(h0)
    r1 = np.abs(h1 - (f["j1"](x) + 1j * f["y1"](x))) / np.abs(h1)
    assert r0.max() < 4e-15 and r1.max() < 4e-15, (r0.max(), r1.max())


@pytest.fixture(scope="module")
def hkff(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("hkff") / "libhkff.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=on",
                    "-I" + os.path.join(ROOT, "bem2d_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "hankel_ff_host.cpp"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)

    def f(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        o = np.zeros((len(x), 4))
        lib.hankel01_ff_host(ctypes.c_int(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                             o.ctypes.data_as(ctypes.c_void_p))
        return o[:, 0] + 1j * o[:, 1], o[:, 2] + 1j * o[:, 3]

    def b(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        o = np.zeros((len(x), 4))
        lib.bessel01_ff_host(ctypes.c_int(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                             o.ctypes.data_as(ctypes.c_void_p))
        return o

    def lg(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        o = np.zeros(len(x))
        lib.log_ff_host(ctypes.c_int(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                        o.ctypes.data_as(ctypes.c_void_p))
        return o
    f.bessel = b
    f.log = lg
    f.path = out
    return f


def _ff_round(x):
    """x rounded to the nearest float-float (as the evaluators receive it)."""
    hi = x.astype(np.float32).astype(np.float64)
    return hi + (x - hi).astype(np.float32).astype(np.float64)


def test_float_float_small_argument_against_mpmath(hkff):
    """bessel01_ff over 1e-7 <= x <= 40, with the small-argument branch
    (x <= 4: series form and the float-float logarithm) and the join at 4:
    J0, Y0, J1, Y1 within 3e-14 of max(1, |value|) and ff_log within 1e-13
    absolute, both at the float-float-rounded argument."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(5)
    x = _ff_round(np.concatenate([10 ** rng.uniform(-7, np.log10(40), 800),
                                  np.linspace(3.99, 4.01, 41), np.linspace(0.85, 0.95, 21)]))
    o = hkff.bessel(x)
    ref = np.array([[float(mp.besselj(0, mp.mpf(v))), float(mp.bessely(0, mp.mpf(v))),
                     float(mp.besselj(1, mp.mpf(v))), float(mp.bessely(1, mp.mpf(v)))]
                    for v in x])
    err = np.abs(o - ref) / np.maximum(1.0, np.abs(ref))
    assert err.max() < 3e-14, (err.max(axis=0), x[err.argmax() // 4])
    lg = hkff.log(x)
    lref = np.array([float(mp.log(mp.mpf(v))) for v in x])
    assert np.abs(lg - lref).max() < 1e-13


def test_float_float_against_mpmath(hkff):
    """The float-float far-field evaluator (used from k|x - y| = 4 on) against
    mpmath at 50 digits, on every interval of the piecewise fit and across
    its joins (4, 8, 16, 64): relative error of H0 and H1 within 3e-14 plus
    x * 2^-48 (x itself is held as a float-float, ~48 bits, so the phase
    x - pi/4 carries an absolute error of that size)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    rng = np.random.default_rng(3)
    x = np.concatenate([np.linspace(4.0, 8.0, 201), 10 ** rng.uniform(np.log10(4), 4, 600),
                        np.linspace(7.99, 8.01, 11), np.linspace(15.99, 16.01, 11),
                        np.linspace(63.99, 64.01, 11)])
    h0, h1 = hkff(x)
    r0 = np.array([complex(mp.hankel1(0, mp.mpf(float(v)))) for v in x])
    r1 = np.array([complex(mp.hankel1(1, mp.mpf(float(v)))) for v in x])
    bound = 3e-14 + x * 2.0 ** -48
    e0 = np.abs(h0 - r0) / np.abs(r0) / bound
    e1 = np.abs(h1 - r1) / np.abs(r1) / bound
    assert e0.max() < 1 and e1.max() < 1, (e0.max(), e1.max())


def test_float_float_dot2_against_exact(hkff):
    """ff_dot2(a, b, c, d) = a b + c d in float-float (the far field's complex
    products, normal factors and squared distance): within 2^-46 (|a b| +
    |c d|) of the exact value of the float-float inputs (rational
    arithmetic), including near-total cancellation, and the result
    normalised (|lo| <= ulp(hi))."""
    from fractions import Fraction
    lib = ctypes.CDLL(hkff.path)
    rng = np.random.default_rng(11)
    n = 4000

    def ffs(m):
        hi = (rng.standard_normal(m) * 10.0 ** rng.uniform(-3, 3, m)).astype(np.float32)
        lo = (hi.astype(np.float64) * rng.uniform(-2 ** -25, 2 ** -25, m)).astype(np.float32)
        return hi, lo
    a, b, c, d = ffs(n), ffs(n), ffs(n), ffs(n)
    # a quarter of the cases: c d = -a b up to the low parts (cancellation)
    k = n // 4
    c[0][:k], c[1][:k] = -a[0][:k], np.zeros(k, dtype=np.float32)
    d[0][:k], d[1][:k] = b[0][:k], (b[0][:k].astype(np.float64) * 2 ** -30).astype(np.float32)
    v = np.stack([a[0], a[1], b[0], b[1], c[0], c[1], d[0], d[1]], axis=1).astype(np.float32)
    v = np.ascontiguousarray(v)
    out = np.zeros((n, 2), dtype=np.float32)
    lib.dot2_ff_host(ctypes.c_int(n), v.ctypes.data_as(ctypes.c_void_p),
                     out.ctypes.data_as(ctypes.c_void_p))
    worst = 0.0
    for i in range(n):
        F = [Fraction(float(x)) for x in v[i]]
        ab = (F[0] + F[1]) * (F[2] + F[3])
        cd = (F[4] + F[5]) * (F[6] + F[7])
        exact = ab + cd
        got = Fraction(float(out[i, 0])) + Fraction(float(out[i, 1]))
        scale = abs(ab) + abs(cd)
        if scale:
            worst = max(worst, float(abs(got - exact) / scale))
        assert abs(float(out[i, 1])) <= np.spacing(np.float32(abs(out[i, 0]))) or out[i, 0] == 0
    assert worst <= 2.0 ** -46, worst
