"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/liboracle.so (the C restatement in bem2d_oracle.c) and adds the
dense linear algebra the reference delegates to LAPACK, through scipy's
LAPACK bindings with the same drivers the reference calls:
  SolveSystem  zgetrf + zgetrs     lib/bem2d_mathroutines.cpp:323-351
  L2NormCond   zgesvd (no vectors) lib/bem2d_mathroutines.cpp:208-266
  ChangeBasis  zpotrf + 2 ztrsm    lib/bem2d_mathroutines.cpp:534-588
  NumRange     zheev per angle     lib/bem2d_mathroutines.cpp:590-653
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

KERNELS = {"single": 0, "double": 1, "conjdouble": 2, "combined": 3}


def _k(k, eta):
    """(Re k, Im k, eta): a complex k selects the oracle's binary128 Hankel
    functions (the reference's AMOS branch); eta defaults to Re k."""
    kc = complex(k)
    return kc.real, kc.imag, (kc.real if eta is None else float(eta))


class _Geom(ctypes.Structure):
    _fields_ = [("n_elem", ctypes.c_int32),
                ("kind", ctypes.c_void_p), ("param", ctypes.c_void_p),
                ("index", ctypes.c_void_p), ("next", ctypes.c_void_p),
                ("prev", ctypes.c_void_p),
                ("n_unk", ctypes.c_int32),
                ("unk_elem", ctypes.c_void_p), ("unk_kind", ctypes.c_void_p),
                ("unk_param", ctypes.c_void_p)]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run `make -C oracle port`")
        _LIB = ctypes.CDLL(path)
    return _LIB


def _geom(g):
    a = g.arrays()
    s = _Geom(len(a["kind"]), a["kind"].ctypes.data, a["param"].ctypes.data,
              a["index"].ctypes.data, a["next"].ctypes.data,
              a["prev"].ctypes.data, len(a["unk_elem"]),
              a["unk_elem"].ctypes.data, a["unk_kind"].ctypes.data,
              a["unk_param"].ctypes.data)
    return s, a  # keep the arrays alive with the struct


def gauss(n):
    x = np.zeros(n)
    w = np.zeros(n)
    rc = lib().orc_gauss(ctypes.c_int(n), x.ctypes.data_as(ctypes.c_void_p),
                         w.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return x, w


def discrete_kernel(g, kernel="combined", k=10.0, eta=None, quad=(3, 5, 0.15),
                    alpha=1.0, beta=0.0, threads=0):
    """beta*Id + alpha*DiscreteKernel(g, quad, kernel) as complex128 (n x n);
    k real or complex."""
    s, keep = _geom(g)
    n = s.n_unk
    out = np.zeros((n, n), dtype=np.complex128, order="F")
    kr, ki, eta = _k(k, eta)
    L, N, sigma = quad
    rc = lib().orc_discrete_kernel_c(
        ctypes.byref(s), ctypes.c_int(L), ctypes.c_int(N), ctypes.c_double(sigma),
        ctypes.c_int(KERNELS[kernel]), ctypes.c_double(kr), ctypes.c_double(ki),
        ctypes.c_double(eta),
        ctypes.c_double(alpha), ctypes.c_double(beta),
        out.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(threads))
    assert rc == 0, rc
    return out


def discrete_kernel_rows(g, rows, kernel="combined", k=10.0, eta=None,
                         quad=(3, 5, 0.15), alpha=1.0, beta=0.0, threads=0):
    """Selected rows of beta*Id + alpha*DiscreteKernel (len(rows) x n)."""
    s, keep = _geom(g)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    out = np.zeros((len(rows), s.n_unk), dtype=np.complex128)
    eta = float(k) if eta is None else float(eta)
    L, N, sigma = quad
    rc = lib().orc_discrete_kernel_rows(
        ctypes.byref(s), ctypes.c_int(L), ctypes.c_int(N), ctypes.c_double(sigma),
        ctypes.c_int(KERNELS[kernel]), ctypes.c_double(k), ctypes.c_double(eta),
        ctypes.c_double(alpha), ctypes.c_double(beta), ctypes.c_int(len(rows)),
        rows.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
        ctypes.c_int(threads))
    assert rc == 0, rc
    return out


def eval_ident(g, N=5):
    s, keep = _geom(g)
    n = s.n_unk
    out = np.zeros((n, n), dtype=np.complex128, order="F")
    rc = lib().orc_eval_ident(ctypes.byref(s), ctypes.c_int(N),
                              out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return out


def rhs(g, k, direction, eta=None, N=5, fun=2, scale=2.0):
    """scale * DotProdBasFuns(g, quad, CombinedPlaneWave(direction, k, eta));
    k real or complex."""
    s, keep = _geom(g)
    out = np.zeros(s.n_unk, dtype=np.complex128)
    kr, ki, eta = _k(k, eta)
    rc = lib().orc_rhs_c(ctypes.byref(s), ctypes.c_int(N), ctypes.c_int(fun),
                       ctypes.c_double(kr), ctypes.c_double(ki), ctypes.c_double(direction[0]),
                       ctypes.c_double(direction[1]), ctypes.c_double(eta),
                       ctypes.c_double(scale), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return out


def system(g, k, direction, eta=None, quad=(3, 5, 0.15), threads=0):
    """SoundSoftScattering::Discretize: A = Id + 2K(combined), b = 2<f,phi>."""
    A = discrete_kernel(g, "combined", k, eta, quad, alpha=2.0, beta=1.0,
                        threads=threads)
    b = rhs(g, k, direction, eta, quad[1])
    return A, b


def solve(A, b):
    """SolveSystem: LAPACK zgetrf + zgetrs."""
    from scipy.linalg import lu_factor, lu_solve
    return lu_solve(lu_factor(A, check_finite=False), b, check_finite=False)


def change_basis(K, M):
    """ChangeBasis(K, M): M = U^H U, returns U^{-H} K U^{-1}."""
    from scipy.linalg import cholesky, solve_triangular
    U = cholesky(M, lower=False, check_finite=False)
    T = solve_triangular(U, K.T, trans="T", lower=False, check_finite=False).T  # K U^{-1}
    return solve_triangular(U, T, trans="C", lower=False, check_finite=False)


def norm_cond(A):
    """L2NormCond: singular values by zgesvd (no vectors)."""
    from scipy.linalg import svd
    s = svd(A, compute_uv=False, lapack_driver="gesvd", check_finite=False)
    return s[0], s[0] / s[-1]


def numrange_lmax(A, thetas):
    """lambda_max of the Hermitian part of e^{i theta} A per angle (zheev)."""
    from scipy.linalg import eigh
    out = []
    for th in thetas:
        m = np.exp(1j * th) * A
        H = 0.5 * (m + m.conj().T)
        out.append(eigh(H, eigvals_only=True, driver="ev", check_finite=False)[-1])
    return np.array(out)


def potential(g, coeffs, points, kernel="single", k=10.0, eta=0.0, N=5):
    """EvalKernel: sum_u c_u int K(p, y) phi_u(y) ds(y) at the points; k real
    or complex."""
    s, keep = _geom(g)
    c = np.ascontiguousarray(coeffs, dtype=np.complex128)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2)
    out = np.zeros(len(pts), dtype=np.complex128)
    kr, ki, eta = _k(k, eta)
    rc = lib().orc_potential_c(ctypes.byref(s), ctypes.c_int(N), ctypes.c_int(KERNELS[kernel]),
                             ctypes.c_double(kr), ctypes.c_double(ki), ctypes.c_double(eta),
                             c.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(len(pts)),
                             pts.ctypes.data_as(ctypes.c_void_p),
                             out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return out
