"""Accuracy of the complex-argument Hankel evaluator
(bem2d_gb300/csrc/hankel_c.cuh), which replaces the reference's AMOS zbesh
calls for complex wavenumbers (lib/bem2d_mathroutines.cpp:44-75).

The evaluator is header-only and compiles for the host too; this builds it
with g++ and checks H0, H1 over its domain (Re z > 0, -pi/3 <= arg z <= pi/2)
against mpmath (working precision raised with |z|, so that its own J + iY
cancellation does not show) and against scipy.special.hankel1, which is
AMOS's zbesh.  Stated bound: relative error <= 4e-15 (1 + |z|/50).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def hkc(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("hkc") / "libhkc.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared",
                    "-I" + os.path.join(ROOT, "bem2d_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "hankel_host.cpp"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)

    def f(z):
        z = np.ascontiguousarray(np.asarray(z, dtype=np.complex128))
        o = np.zeros((len(z), 4))
        lib.hankel01_c_host(ctypes.c_int(len(z)), z.ctypes.data_as(ctypes.c_void_p),
                            o.ctypes.data_as(ctypes.c_void_p))
        return o[:, 0] + 1j * o[:, 1], o[:, 2] + 1j * o[:, 3]
    f.lib = lib
    return f


def domain_points(n, seed):
    """|z| log-uniform in [1e-6, 500], arg z uniform in [-pi/3, pi/2], plus the
    piece boundaries (|z| = 1.5, 3, 7, 14) and the edges of the angle range."""
    rng = np.random.default_rng(seed)
    r = 10 ** rng.uniform(-6, np.log10(500), n)
    a = rng.uniform(-np.pi / 3, np.pi / 2, n)
    rb = np.repeat([1.5, 1.5 * (1 + 1e-12), 3.0, 3.0 * (1 + 1e-12), 7.0, 7.0 * (1 + 1e-12),
                    14.0, 14.0 * (1 + 1e-12)], 5)
    ab = np.tile([-np.pi / 3, -0.46, 0.0, 0.8, np.pi / 2], 8)
    z = np.concatenate([r * np.exp(1j * a), rb * np.exp(1j * ab)])
    return z[z.imag < 60]  # beyond, |H| < e^-60: underflow territory, not accuracy


def rel_err(got, ref, z):
    return np.abs(got - ref) / np.abs(ref) / (1 + np.abs(z) / 50)


def test_against_mpmath(hkc):
    mp = pytest.importorskip("mpmath")
    z = domain_points(300, 11)
    h0, h1 = hkc(z)
    r0 = np.empty(len(z), complex)
    r1 = np.empty(len(z), complex)
    for i, zi in enumerate(z):
        with mp.workdps(int(30 + abs(zi))):
            zz = mp.mpc(zi.real, zi.imag)
            r0[i] = complex(mp.hankel1(0, zz))
            r1[i] = complex(mp.hankel1(1, zz))
    e = max(rel_err(h0, r0, z).max(), rel_err(h1, r1, z).max())
    assert e < 4e-15, e


def test_against_amos(hkc):
    """scipy.special.hankel1 is AMOS zbesh (kode 1), the routine the reference
    links for complex wavenumbers."""
    sp = pytest.importorskip("scipy.special")
    z = domain_points(20000, 12)
    h0, h1 = hkc(z)
    e = max(rel_err(h0, sp.hankel1(0, z), z).max(), rel_err(h1, sp.hankel1(1, z), z).max())
    assert e < 1e-14, e


def test_real_axis_matches_real_evaluator(hkc):
    """On the real axis the complex evaluator agrees with the real one
    (hankel.cuh), an independent method (fitted polynomials)."""
    x = np.concatenate([10 ** np.linspace(-5, 2.5, 400), [1.5, 3.0, 7.0, 14.0]])
    h0, h1 = hkc(x.astype(complex))
    o = np.zeros((len(x), 4))
    hkc.lib.hankel01_d_host(ctypes.c_int(len(x)), x.ctypes.data_as(ctypes.c_void_p),
                            o.ctypes.data_as(ctypes.c_void_p))
    r0, r1 = o[:, 0] + 1j * o[:, 1], o[:, 2] + 1j * o[:, 3]
    e = max(rel_err(h0, r0, x).max(), rel_err(h1, r1, x).max())
    assert e < 1e-14, e


def test_trap_domain(hkc):
    """Arguments of the reference's resonance scan (resonances/trapresonance.cpp:
    k in [4, 8] + i[-2, 0], distances up to the trapping domain's diameter)."""
    sp = pytest.importorskip("scipy.special")
    kr, ki, d = np.meshgrid(np.linspace(4, 8, 21), np.linspace(-2, 0, 11),
                            np.linspace(1e-4, 3.0, 61))
    z = ((kr + 1j * ki) * d).ravel()
    h0, h1 = hkc(z)
    e = max(rel_err(h0, sp.hankel1(0, z), z).max(), rel_err(h1, sp.hankel1(1, z), z).max())
    assert e < 1e-14, e


def test_against_reference_fixture(hkc):
    """The reference's own BesselH0 / BesselH1 of a complex argument
    (lib/bem2d_mathroutines.cpp:44-75) as recorded in tests/golden/hankel_ck.npz
    by the reference build (its zbesh served by a binary128 evaluator that
    make_golden.py checks against scipy's AMOS)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "hankel_ck.npz"))
    h0, h1 = hkc(z["z"])
    e = max(rel_err(h0, z["h0"], z["z"]).max(), rel_err(h1, z["h1"], z["z"]).max())
    assert e < 4e-15, e
