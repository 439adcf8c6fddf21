"""Complex wavenumbers on the GPU: the reference's AMOS branch
(lib/bem2d_kernel.cpp:15-112 with k.im != 0, BesselH0/H1(complex) at
lib/bem2d_mathroutines.cpp:44-75) against the reference's own outputs.

The fixtures (tests/golden/*_ck.npz) come from the reference library built
in place, its zbesh served by a binary128 evaluator that agrees with
scipy's AMOS to 4e-15 (make_golden.py checks it).  Cases: the trapping
domain of resonances/trapresonance.cpp at k = 6 - i, a disk in an absorbing
medium (k = 8 + 0.5i), a kite at k = 12 - 3i and PolBasis(2) on a square.

Bars as for real k: FP64 matrices, right-hand sides and potentials within
1e-12 relative (Frobenius); FP64 solutions within 1e-11 or, for the
ill-conditioned cases, 10 cond(A) times the matrix and right-hand-side
differences; the mixed solver (complex64 LU + FP64 refinement) within
1e-10 or that bound.
"""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, QUAD

pytestmark = pytest.mark.gpu

CK_CASES = sorted(n for n in CASES if CASES[n].get("kim"))


def _load(name):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    return z, json.loads(str(z["meta"]))


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def blocks_of(g):
    """Unknown ranges per element (the mass matrix's diagonal blocks)."""
    ue = g.arrays()["unk_elem"]
    starts = [0] + [i for i in range(1, len(ue)) if ue[i] != ue[i - 1]] + [len(ue)]
    return np.array(starts, dtype=np.int32)


def kc(spec):
    return complex(spec["k"], spec["kim"])


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", CK_CASES)
def test_matrix_matches_reference(ctx, name):
    z, meta = _load(name)
    spec = CASES[name]
    assert meta["kim"] == spec["kim"]
    g = spec["geom"]()
    k, eta = kc(spec), spec["eta"]
    A = ctx.discrete_kernel(g, "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
    assert rel(A, z["A"]) < 1e-12
    for kn in spec.get("kernels", ()):
        K = ctx.discrete_kernel(g, kn, k, eta, QUAD)
        assert rel(K, z["K_" + kn]) < 1e-12, kn


@pytest.mark.parametrize("name", CK_CASES)
def test_rhs_and_solution(ctx, name):
    z, meta = _load(name)
    spec = CASES[name]
    g = spec["geom"]()
    k, eta, d = kc(spec), spec["eta"], spec["direction"]
    b = ctx.rhs(g, k, d, eta, QUAD)
    assert rel(b, z["rhs"]) < 1e-12
    A = ctx.discrete_kernel(g, "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
    # two FP64 solvers given systems that differ by dA, db agree to about
    # cond(A) (|dA|/|A| + |db|/|b|); with Im k < 0 the kernel grows like
    # e^{-Im k |x-y|} and cond(A) reaches 7e4 (kite at k = 12 - 3i)
    tol_x = max(1e-11, 10 * np.linalg.cond(z["A"]) * (rel(A, z["A"]) + rel(b, z["rhs"])))
    x = ctx.scattering_solve(g, k, d, eta, QUAD, precision="fp64")
    assert rel(x, z["x"]) < tol_x
    xm = ctx.scattering_solve(g, k, d, eta, QUAD, precision="mixed")
    assert rel(xm, z["x"]) < max(1e-10, tol_x), ctx.last_info


def test_mixed_assembly_entry(ctx):
    """bem2d_discrete_kernel_mixed with a complex k: the FP64 matrix and its
    complex64 rounding."""
    spec = CASES["kite_ck"]
    z, _ = _load("kite_ck")
    A, A32 = ctx.discrete_kernel_mixed(spec["geom"](), "combined", kc(spec), spec["eta"], QUAD,
                                       alpha=2.0, beta=1.0)
    assert rel(A, z["A"]) < 1e-12
    assert np.array_equal(A32, A.astype(np.complex64))


def test_norm_cond_trap(ctx):
    """The resonance scan's quantity: ||A^{-1}|| = cond / norm of
    ChangeBasis(A, Id) at k = 6 - i on the trapping domain."""
    z, _ = _load("trap_ck")
    spec = CASES["trap_ck"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", kc(spec), spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    nrm, cond = ctx.norm_cond(B)
    ref_n, ref_c = z["normcond"]
    assert abs(nrm - ref_n) < 1e-11 * ref_n
    assert abs(cond - ref_c) < 1e-9 * ref_c


def test_evalsol(ctx):
    """u = u_inc - S phi (SoundSoftScattering::EvalSol) in an absorbing medium."""
    z, _ = _load("disk_absorbing_ck")
    spec = CASES["disk_absorbing_ck"]
    g = spec["geom"]()
    k, d = kc(spec), spec["direction"]
    x = ctx.scattering_solve(g, k, d, spec["eta"], QUAD, precision="fp64")
    pts = z["evalsol_points"]
    pot = ctx.potential(g, x, pts, "single", k)
    uinc = np.exp(1j * k * (d[0] * pts[:, 0] + d[1] * pts[:, 1]))
    assert rel(uinc - pot, z["evalsol"]) < 1e-11


@pytest.mark.parametrize("kernel", ["single", "double", "conjdouble", "combined"])
def test_vanishing_imaginary_part_meets_real_path(ctx, kernel):
    """k = 40 + 1e-14 i through the complex-argument evaluator against k = 40
    through the real one (fitted polynomials, an independent method): kite
    N = 512, arguments k|x - y| up to ~110.  The 1e-14 shift moves the matrix
    by about |x - y| 1e-14 relative."""
    from bem2d_gb300 import geometry as G
    g = G.kite(512).add_poly_basis(0)
    Ar = ctx.discrete_kernel(g, kernel, 40.0, 40.0, QUAD, alpha=2.0, beta=1.0)
    Ac = ctx.discrete_kernel(g, kernel, complex(40.0, 1e-14), 40.0, QUAD, alpha=2.0, beta=1.0)
    assert rel(Ac, Ar) < 1e-12


def test_outside_domain_is_rejected(ctx):
    """arg k < -pi/3 is outside the complex evaluator's domain."""
    from bem2d_gb300 import capi
    from bem2d_gb300 import geometry as G
    g = G.kite(16).add_poly_basis(0)
    with pytest.raises(capi.Bem2dError) as e:
        ctx.discrete_kernel(g, "single", complex(1.0, -2.0), 1.0, QUAD)
    assert e.value.code == -7  # BEM2D_ERR_UNSUPPORTED
