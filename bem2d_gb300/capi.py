"""ctypes binding of the C ABI (include/bem2d_gpu.h) for tests and the bench.

Loads bem2d_gb300/libbem2d_gpu.so and fails loudly if it is missing or if no
GPU is present: there is no CPU fallback.  Arrays may be numpy (host) or
torch CUDA tensors (device); the library takes either.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import geometry as G

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbem2d_gpu.so")

OK = 0
ERR = {-1: "ARG", -2: "CUDA", -3: "NOMEM", -4: "NONFINITE", -5: "NOCONV",
       -6: "TIMEOUT", -7: "UNSUPPORTED"}
KERNEL = {"single": 0, "double": 1, "conjdouble": 2, "combined": 3}
FUN = {"planewave": 0, "normalplanewave": 1, "combinedplanewave": 2}
PREC = {"fp64": 0, "mixed": 1, "mixed_tf32": 2}

# symbols declared in include/bem2d_gpu.h
EXPORTS = ["bem2d_ctx_create", "bem2d_ctx_destroy", "bem2d_ctx_last_error",
           "bem2d_ctx_stream", "bem2d_ctx_set_stream", "bem2d_ctx_launch_count",
           "bem2d_gauss", "bem2d_discrete_kernel", "bem2d_discrete_kernel_mixed",
           "bem2d_eval_ident",
           "bem2d_dot_prod_basfuns", "bem2d_solve_system", "bem2d_scattering_solve",
           "bem2d_fma_peak", "bem2d_ctx_enable_timers", "bem2d_ctx_timer",
           "bem2d_change_basis", "bem2d_l2_norm_cond", "bem2d_l2_norm_cond_prec",
           "bem2d_num_range",
           "bem2d_eval_kernel", "bem2d_solve_system_noalloc",
           "bem2d_sweep_solve", "bem2d_hermitian_eigenvalues", "bem2d_singular_values",
           "bem2d_eigenvalues", "bem2d_debug_panel_timeout", "bem2d_noalloc_scratch_fits",
           "bem2d_debug_tc_update", "bem2d_matmul", "bem2d_eigenvectors"]

NOALLOC_MAX_N = 1024  # BEM2D_NOALLOC_MAX_N


class Bem2dError(RuntimeError):
    def __init__(self, code, msg):
        self.code = code
        super().__init__("bem2d_gpu error %d (%s): %s" % (code, ERR.get(code, "INFO"), msg))


class LapackError(Bem2dError):
    """A zero pivot (the reference throws LapackError)."""


class Geometry_c(ctypes.Structure):
    _fields_ = [("n_elem", ctypes.c_int32),
                ("kind", ctypes.c_void_p), ("param", ctypes.c_void_p),
                ("index", ctypes.c_void_p), ("next", ctypes.c_void_p),
                ("prev", ctypes.c_void_p),
                ("n_unk", ctypes.c_int32),
                ("unk_elem", ctypes.c_void_p), ("unk_kind", ctypes.c_void_p),
                ("unk_param", ctypes.c_void_p)]


class Quad_c(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32), ("N", ctypes.c_int32), ("sigma", ctypes.c_double)]


class SolveInfo_c(ctypes.Structure):
    _fields_ = [("info", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("residual", ctypes.c_double)]


_LIB = None


def load():
    """Load the CUDA library (raises if it is not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libbem2d_gpu.so is not built; run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(LIB_PATH)
        vp, i32, i64, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        lib.bem2d_ctx_create.argtypes = [i32, ctypes.POINTER(vp)]
        lib.bem2d_ctx_destroy.argtypes = [vp]
        lib.bem2d_ctx_destroy.restype = None
        lib.bem2d_ctx_last_error.argtypes = [vp]
        lib.bem2d_ctx_last_error.restype = ctypes.c_char_p
        lib.bem2d_ctx_stream.argtypes = [vp]
        lib.bem2d_ctx_stream.restype = vp
        lib.bem2d_ctx_set_stream.argtypes = [vp, vp]
        lib.bem2d_ctx_launch_count.argtypes = [vp]
        lib.bem2d_ctx_launch_count.restype = i64
        lib.bem2d_gauss.argtypes = [i32, vp, vp]
        lib.bem2d_discrete_kernel.argtypes = [vp, vp, vp, i32, d, d, d, d, d, vp, i64]
        lib.bem2d_discrete_kernel_mixed.argtypes = [vp, vp, vp, i32, d, d, d, d, d, vp, i64,
                                                    vp, i64]
        lib.bem2d_eval_ident.argtypes = [vp, vp, vp, vp, i64]
        lib.bem2d_dot_prod_basfuns.argtypes = [vp, vp, vp, i32, d, d, d, d, d, d, vp]
        lib.bem2d_solve_system.argtypes = [vp, i32, vp, i64, vp, vp, i32, d, vp]
        lib.bem2d_solve_system_noalloc.argtypes = [vp, i32, vp, i64, vp, vp, vp]
        lib.bem2d_sweep_solve.argtypes = [vp, i32, vp, vp, vp, vp, d, d, i32, d, i32, vp, vp]
        lib.bem2d_scattering_solve.argtypes = [vp, vp, vp, d, d, d, d, d, i32, d, vp, vp]
        lib.bem2d_fma_peak.argtypes = [i32, ctypes.POINTER(d)]
        lib.bem2d_change_basis.argtypes = [vp, i32, vp, i64, vp, i64, vp, i32, vp, i64]
        lib.bem2d_l2_norm_cond.argtypes = [vp, i32, vp, i64, d, ctypes.POINTER(d),
                                           ctypes.POINTER(d)]
        lib.bem2d_num_range.argtypes = [vp, i32, vp, i64, i32, vp, d, i32, vp]
        lib.bem2d_eval_kernel.argtypes = [vp, vp, vp, i32, d, d, d, vp, i32, vp, vp]
        lib.bem2d_hermitian_eigenvalues.argtypes = [vp, i32, vp, i64, vp]
        lib.bem2d_singular_values.argtypes = [vp, i32, vp, i64, vp]
        lib.bem2d_eigenvalues.argtypes = [vp, i32, vp, i64, vp]
        lib.bem2d_l2_norm_cond_prec.argtypes = [vp, i32, vp, i64, d, i32, ctypes.POINTER(d),
                                                ctypes.POINTER(d)]
        lib.bem2d_debug_panel_timeout.argtypes = [vp, i32, i32]
        lib.bem2d_noalloc_scratch_fits.argtypes = [ctypes.POINTER(i64), ctypes.POINTER(i64)]
        lib.bem2d_debug_tc_update.argtypes = [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64]
        lib.bem2d_matmul.argtypes = [vp, i32, i32, i32, vp, i64, vp, i64, vp, i64]
        lib.bem2d_eigenvectors.argtypes = [vp, i32, vp, i64, vp, vp, i64]
        lib.bem2d_ctx_enable_timers.argtypes = [vp, i32]
        lib.bem2d_ctx_timer.argtypes = [vp, i32, ctypes.POINTER(d), ctypes.POINTER(i64)]
        _LIB = lib
    return _LIB


def _ld(a, n):
    """Leading dimension of a column-major matrix: numpy (Fortran order) or a
    torch tensor (column-major view, or row-major storage of the transpose)."""
    if hasattr(a, "stride"):
        return a.stride(1) if a.stride(0) == 1 else a.stride(0)
    return n


def _sync_producers(*objs):
    """The library orders its work on the context's stream.  torch CUDA
    tensors handed to it (inputs, or outputs torch has just allocated and
    filled) are written on torch's stream: wait for that stream first."""
    for o in objs:
        if isinstance(o, (list, tuple)):
            o = o[0] if o else None
        if getattr(o, "is_cuda", False):
            import torch
            torch.cuda.current_stream().synchronize()
            return


def _ptr(a):
    """Raw address of a numpy array or a torch tensor."""
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)


class _GeomHold:
    """A C geometry struct that keeps its arrays alive."""

    def __init__(self, g):
        a = g.arrays() if isinstance(g, G.Geometry) else g
        self.arrays = a
        self.c = Geometry_c(len(a["kind"]), a["kind"].ctypes.data, a["param"].ctypes.data,
                            a["index"].ctypes.data, a["next"].ctypes.data,
                            a["prev"].ctypes.data, len(a["unk_elem"]),
                            a["unk_elem"].ctypes.data, a["unk_kind"].ctypes.data,
                            a["unk_param"].ctypes.data)
        self.n = len(a["unk_elem"])


def _k(k, eta):
    """Wavenumber (real or complex) as (re, im) and the coupling eta, whose
    default is Re k (CombinedSingleConjDouble(k), lib/bem2d_kernel.cpp:89)."""
    kc = complex(k)
    return kc.real, kc.imag, (kc.real if eta is None else float(eta))


def quad(q=(3, 5, 0.15)):
    return Quad_c(int(q[0]), int(q[1]), float(q[2]))


class Context:
    """One bem2d_ctx (device workspace + stream)."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.bem2d_ctx_create(device, ctypes.byref(h))
        if rc != 0:
            raise Bem2dError(rc, "bem2d_ctx_create failed (no GPU?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.bem2d_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc == 0:
            return
        msg = self.lib.bem2d_ctx_last_error(self.h).decode()
        if rc > 0:
            raise LapackError(rc, msg)
        raise Bem2dError(rc, msg)

    @property
    def launches(self):
        return int(self.lib.bem2d_ctx_launch_count(self.h))

    @property
    def stream(self):
        return self.lib.bem2d_ctx_stream(self.h)

    PHASES = ("far", "near", "lu", "solve")

    def enable_timers(self, on=True):
        self._check(self.lib.bem2d_ctx_enable_timers(self.h, 1 if on else 0))

    def timers(self):
        """{phase: (total ms, count)} since enable_timers()."""
        out = {}
        for i, name in enumerate(self.PHASES):
            ms, n = ctypes.c_double(), ctypes.c_int64()
            self._check(self.lib.bem2d_ctx_timer(self.h, i, ctypes.byref(ms), ctypes.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    # -- assembly ----------------------------------------------------------
    def discrete_kernel(self, g, kernel="combined", k=10.0, eta=None, q=(3, 5, 0.15),
                        alpha=1.0, beta=0.0, out=None):
        _sync_producers(out)
        gh = _GeomHold(g)
        n = gh.n
        if out is None:
            out = np.zeros((n, n), dtype=np.complex128, order="F")
        ld = n
        if hasattr(out, "stride"):  # torch: column-major view, or row-major storage of A^T
            ld = out.stride(1) if out.stride(0) == 1 else out.stride(0)
        kr, ki, eta = _k(k, eta)
        qq = quad(q)
        self._check(self.lib.bem2d_discrete_kernel(
            self.h, ctypes.byref(gh.c), ctypes.byref(qq), KERNEL[kernel], kr, ki,
            eta, float(alpha), float(beta), _ptr(out), ld))
        return out

    def discrete_kernel_mixed(self, g, kernel="combined", k=10.0, eta=None, q=(3, 5, 0.15),
                              alpha=1.0, beta=0.0, out=None, out32=None):
        """Mixed-precision assembly: (complex128, complex64) matrices (host
        numpy by default, or the given torch CUDA tensors)."""
        _sync_producers(out, out32)
        gh = _GeomHold(g)
        n = gh.n
        if out is None:
            out = np.zeros((n, n), dtype=np.complex128, order="F")
        if out32 is None:
            out32 = np.zeros((n, n), dtype=np.complex64, order="F")
        kr, ki, eta = _k(k, eta)
        qq = quad(q)
        self._check(self.lib.bem2d_discrete_kernel_mixed(
            self.h, ctypes.byref(gh.c), ctypes.byref(qq), KERNEL[kernel], kr, ki,
            eta, float(alpha), float(beta), _ptr(out), _ld(out, n), _ptr(out32),
            _ld(out32, n)))
        return out, out32

    def eval_ident(self, g, q=(3, 5, 0.15), out=None):
        _sync_producers(out)
        gh = _GeomHold(g)
        n = gh.n
        if out is None:
            out = np.zeros((n, n), dtype=np.complex128, order="F")
        qq = quad(q)
        self._check(self.lib.bem2d_eval_ident(self.h, ctypes.byref(gh.c), ctypes.byref(qq),
                                              _ptr(out), _ld(out, n)))
        return out

    def rhs(self, g, k, direction, eta=None, q=(3, 5, 0.15), fun="combinedplanewave",
            scale=2.0, out=None):
        _sync_producers(out)
        gh = _GeomHold(g)
        if out is None:
            out = np.zeros(gh.n, dtype=np.complex128)
        kr, ki, eta = _k(k, eta)
        qq = quad(q)
        self._check(self.lib.bem2d_dot_prod_basfuns(
            self.h, ctypes.byref(gh.c), ctypes.byref(qq), FUN[fun], kr, ki,
            float(direction[0]), float(direction[1]), eta, float(scale), _ptr(out)))
        return out

    # -- solve -------------------------------------------------------------
    def solve(self, A, b, precision="fp64", tol=0.0, out=None):
        _sync_producers(A, b, out)
        n = A.shape[0]
        if out is None:
            out = np.zeros(n, dtype=np.complex128)
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
            b = np.ascontiguousarray(b, dtype=np.complex128)
            lda = n
        else:
            lda = _ld(A, n)
        info = SolveInfo_c()
        self._check(self.lib.bem2d_solve_system(self.h, n, _ptr(A), lda, _ptr(b), _ptr(out),
                                                PREC[precision], float(tol), ctypes.byref(info)))
        self.last_info = (info.info, info.iterations, info.residual)
        return out

    def solve_noalloc(self, A, b, out=None):
        """FP64 solve through bem2d_solve_system_noalloc (no device allocation,
        n <= NOALLOC_MAX_N)."""
        _sync_producers(A, b, out)
        n = A.shape[0]
        if out is None:
            out = np.zeros(n, dtype=np.complex128)
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
            b = np.ascontiguousarray(b, dtype=np.complex128)
            lda = n
        else:
            lda = _ld(A, n)
        info = SolveInfo_c()
        self._check(self.lib.bem2d_solve_system_noalloc(self.h, n, _ptr(A), lda, _ptr(b),
                                                        _ptr(out), ctypes.byref(info)))
        self.last_info = (info.info, info.iterations, info.residual)
        return out

    def debug_panel_timeout(self, n=512, polls=64):
        """Return code of bem2d_debug_panel_timeout (BEM2D_ERR_TIMEOUT = -6
        expected) and the context's message."""
        rc = self.lib.bem2d_debug_panel_timeout(self.h, int(n), int(polls))
        return rc, self.lib.bem2d_ctx_last_error(self.h).decode()

    def matmul(self, A, B, out=None):
        """A @ B (complex128) through bem2d_matmul; numpy in, numpy out, or
        column-major torch CUDA views."""
        _sync_producers(A, B, out)
        m, k = A.shape
        n = B.shape[1]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        if isinstance(B, np.ndarray):
            B = np.asfortranarray(B, dtype=np.complex128)
        if out is None:
            out = np.zeros((m, n), dtype=np.complex128, order="F")
        self._check(self.lib.bem2d_matmul(self.h, m, n, k, _ptr(A), _ld(A, m), _ptr(B), _ld(B, k),
                                          _ptr(out), _ld(out, m)))
        return out

    def tc_update(self, C, A, B):
        """C -= A B in place on complex64 torch CUDA tensors holding
        column-major matrices (column-major views, as x.t() of a row-major
        tensor) through bem2d_debug_tc_update."""
        _sync_producers(C, A, B)
        M, N = C.shape
        K = A.shape[1]
        self._check(self.lib.bem2d_debug_tc_update(self.h, M, N, K, _ptr(C), _ld(C, M), _ptr(A),
                                                   _ld(A, M), _ptr(B), _ld(B, K)))
        return C

    # -- dense operators ---------------------------------------------------
    def change_basis(self, K, M, bstart, out=None):
        """U^{-H} K U^{-1} with M = U^H U block diagonal (blocks at bstart)."""
        _sync_producers(K, M, out)
        n = K.shape[0]
        if isinstance(K, np.ndarray):
            K = np.asfortranarray(K, dtype=np.complex128)
        if isinstance(M, np.ndarray):
            M = np.asfortranarray(M, dtype=np.complex128)
        bs = np.ascontiguousarray(bstart, dtype=np.int32)
        if out is None:
            out = np.zeros((n, n), dtype=np.complex128, order="F")
        self._check(self.lib.bem2d_change_basis(self.h, n, _ptr(K), _ld(K, n), _ptr(M),
                                                _ld(M, n), _ptr(bs), len(bs) - 1, _ptr(out),
                                                _ld(out, n)))
        return out

    def norm_cond(self, A, tol=0.0, precision=None):
        """(sigma_max, sigma_max / sigma_min) of A; precision None:
        bem2d_l2_norm_cond, else bem2d_l2_norm_cond_prec with "fp64" or
        "mixed" (complex64 LU + FP64 refinement for sigma_min)."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        nrm, cond = ctypes.c_double(), ctypes.c_double()
        if precision is None:
            self._check(self.lib.bem2d_l2_norm_cond(self.h, n, _ptr(A), _ld(A, n), float(tol),
                                                    ctypes.byref(nrm), ctypes.byref(cond)))
        else:
            self._check(self.lib.bem2d_l2_norm_cond_prec(
                self.h, n, _ptr(A), _ld(A, n), float(tol), PREC[precision],
                ctypes.byref(nrm), ctypes.byref(cond)))
        return nrm.value, cond.value

    def num_range_lmax(self, A, thetas, tol=0.0, precision="fp64"):
        """lambda_max of (e^{i th} A + e^{-i th} A^H)/2 for each angle."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        th = np.ascontiguousarray(thetas, dtype=np.float64)
        out = np.zeros(len(th))
        self._check(self.lib.bem2d_num_range(self.h, n, _ptr(A), _ld(A, n), len(th), _ptr(th),
                                             float(tol), PREC[precision], _ptr(out)))
        return out

    def hermitian_eigenvalues(self, A):
        """Eigenvalues (ascending) of the Hermitian matrix A's upper triangle
        defines (HermitianEigenvalues)."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        out = np.zeros(n)
        self._check(self.lib.bem2d_hermitian_eigenvalues(self.h, n, _ptr(A), _ld(A, n),
                                                         _ptr(out)))
        return out

    def singular_values(self, A):
        """Singular values of A, descending (SingularValues)."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        out = np.zeros(n)
        self._check(self.lib.bem2d_singular_values(self.h, n, _ptr(A), _ld(A, n), _ptr(out)))
        return out

    def eigenvalues(self, A):
        """Eigenvalues of the general complex A (Eigenvalues, zgeev)."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        out = np.zeros(n, dtype=np.complex128)
        self._check(self.lib.bem2d_eigenvalues(self.h, n, _ptr(A), _ld(A, n), _ptr(out)))
        return out

    def eigenvectors(self, A):
        """(eigenvalues, right eigenvectors as columns) of the general complex
        A (Eigenvalues with eigenvectors, zgeev 'V')."""
        _sync_producers(A)
        n = A.shape[0]
        if isinstance(A, np.ndarray):
            A = np.asfortranarray(A, dtype=np.complex128)
        w = np.zeros(n, dtype=np.complex128)
        V = np.zeros((n, n), dtype=np.complex128, order="F")
        self._check(self.lib.bem2d_eigenvectors(self.h, n, _ptr(A), _ld(A, n), _ptr(w), _ptr(V),
                                                n))
        return w, V

    def potential(self, g, coeffs, points, kernel="single", k=10.0, eta=0.0, q=(3, 5, 0.15)):
        """sum_u c_u int K(p, y) phi_u(y) ds(y) at the points (EvalKernel)."""
        gh = _GeomHold(g)
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2)
        out = np.zeros(len(pts), dtype=np.complex128)
        kr, ki, eta = _k(k, eta)
        qq = quad(q)
        self._check(self.lib.bem2d_eval_kernel(self.h, ctypes.byref(gh.c), ctypes.byref(qq),
                                               KERNEL[kernel], kr, ki, eta,
                                               _ptr(c), len(pts), _ptr(pts), _ptr(out)))
        return out

    def scattering_solve(self, g, k, direction, eta=None, q=(3, 5, 0.15), precision="fp64",
                         tol=0.0, out=None):
        _sync_producers(out)
        gh = _GeomHold(g)
        if out is None:
            out = np.zeros(gh.n, dtype=np.complex128)
        kr, ki, eta = _k(k, eta)
        qq = quad(q)
        info = SolveInfo_c()
        self._check(self.lib.bem2d_scattering_solve(
            self.h, ctypes.byref(gh.c), ctypes.byref(qq), kr, ki, eta,
            float(direction[0]), float(direction[1]), PREC[precision], float(tol), _ptr(out),
            ctypes.byref(info)))
        self.last_info = (info.info, info.iterations, info.residual)
        return out

    def sweep_solve(self, geoms, ks, direction, etas=None, q=(3, 5, 0.15), precision="mixed",
                    tol=0.0, nworkers=0, outs=None):
        """Batched bem2d_sweep_solve over (geoms[i], ks[i]); returns the list of
        solutions (numpy, or the given `outs`, which may be CUDA tensors)."""
        _sync_producers(outs)
        nk = len(geoms)
        holds = [g if isinstance(g, _GeomHold) else _GeomHold(g) for g in geoms]
        garr = (Geometry_c * max(nk, 1))(*[h.c for h in holds])
        kk = np.ascontiguousarray(ks, dtype=np.float64)
        ee = None if etas is None else np.ascontiguousarray(etas, dtype=np.float64)
        if outs is None:
            outs = [np.zeros(h.n, dtype=np.complex128) for h in holds]
        xptr = (ctypes.c_void_p * max(nk, 1))(*[_ptr(o).value for o in outs])
        infos = (SolveInfo_c * max(nk, 1))()
        qq = quad(q)
        self._check(self.lib.bem2d_sweep_solve(
            self.h, nk, garr, ctypes.byref(qq), kk.ctypes.data,
            None if ee is None else ee.ctypes.data, float(direction[0]), float(direction[1]),
            PREC[precision], float(tol), int(nworkers), xptr, infos))
        self.sweep_infos = [(infos[i].info, infos[i].iterations, infos[i].residual)
                            for i in range(nk)]
        return outs


def gauss(n):
    lib = load()
    x = np.zeros(n)
    w = np.zeros(n)
    rc = lib.bem2d_gauss(n, x.ctypes.data, w.ctypes.data)
    if rc:
        raise Bem2dError(rc, "bem2d_gauss")
    return x, w


def noalloc_scratch_fits():
    """(fits, bytes needed at BEM2D_NOALLOC_MAX_N, bytes of the static array)."""
    lib = load()
    t, cap = ctypes.c_int64(), ctypes.c_int64()
    ok = lib.bem2d_noalloc_scratch_fits(ctypes.byref(t), ctypes.byref(cap))
    return bool(ok), t.value, cap.value


def fma_peak(precision="fp64"):
    """Measured FMA throughput (TFLOP/s) of the FP64 or FP32 pipe."""
    lib = load()
    v = ctypes.c_double()
    rc = lib.bem2d_fma_peak(PREC[precision], ctypes.byref(v))
    if rc:
        raise Bem2dError(rc, "bem2d_fma_peak")
    return v.value
