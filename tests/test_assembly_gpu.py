"""GPU assembly parity: the CUDA path through the C ABI against the
reference's own outputs (tests/golden) and the CPU oracle.

Bar: FP64 assembly within 1e-12 relative Frobenius norm of the reference
matrix; right-hand sides within 1e-12; solutions (FP64 and mixed) with a
normwise backward error <= 1e-14 for the system the GPU assembled, and
within the perturbation bound 2 cond(A) (eA + eb + be + be_ref) of the
reference's own solution (test_rhs_and_solution states the bound)."""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, QUAD

pytestmark = pytest.mark.gpu

TOL_MAT = 1e-12


def _load(name):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    return z, json.loads(str(z["meta"]))


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


# real wavenumbers here; the complex-k cases: test_wavenumber_complex_gpu.py
REAL_CASES = sorted(n for n in CASES if not CASES[n].get("kim"))


@pytest.mark.parametrize("name", REAL_CASES)
def test_matrix_matches_reference(ctx, name):
    z, meta = _load(name)
    spec = CASES[name]
    g = spec["geom"]()
    k, eta = spec["k"], spec["eta"]
    if "rhs" in z:
        A = ctx.discrete_kernel(g, "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
        if "A" in z:
            assert rel(A, z["A"]) < TOL_MAT
        else:
            assert rel(A @ z["probe_v"], z["Av"]) < TOL_MAT
            assert rel(A.conj().T @ z["probe_w"], z["AHw"]) < TOL_MAT
            assert rel(A[z["sample_i"], z["sample_j"]], z["sample"]) < TOL_MAT
            assert rel(np.diag(A), z["diag"]) < TOL_MAT
    for kn in spec.get("kernels", ()):
        K = ctx.discrete_kernel(g, kn, k, eta, QUAD)
        R = z["K_" + kn]
        if np.linalg.norm(R) == 0:
            assert np.abs(K).max() < 1e-15
        else:
            assert rel(K, R) < TOL_MAT, kn
    M = ctx.eval_ident(g, QUAD)
    assert rel(np.diag(M), z["ident_diag"]) < 1e-14


@pytest.mark.parametrize("name", [n for n in REAL_CASES if CASES[n].get("scattering", True)])
def test_rhs_and_solution(ctx, name):
    """Solutions against the reference's x, with a bound derived per case.

    The GPU assembles (A, b) and solves A x = b; the library's own measure of
    the backward error, |b - A x| / (|A|_F |x| + |b|) (the mixed solver's
    stopping rule), is asserted <= 1e-14, and the 2-norm one
    be = |b - A x| / (|A|_2 |x| + |b|) enters the bound.  The reference
    solved its own (A_ref, b_ref) with LAPACK, backward error be_ref (computed
    from its fixtures).  First-order perturbation theory then bounds
        |x - x_ref| / |x_ref| <= 2 cond(A) (eA + eb + be + be_ref),
    eA = |A - A_ref|_F / |A|_2 (an upper bound of the 2-norm relative
    perturbation), eb = |b - b_ref| / |b|, cond(A) = sigma_max / sigma_min
    from the library's own L2NormCond.  A_ref is the reference's matrix where
    the fixture holds it, else the CPU oracle's (pinned to the reference's
    probes of the same matrix by test_oracle.py)."""
    from oracle import oracle as O
    z, meta = _load(name)
    spec = CASES[name]
    g = spec["geom"]()
    k, eta, d = spec["k"], spec["eta"], spec["direction"]
    b = ctx.rhs(g, k, d, eta, QUAD)
    b_ref = z["rhs"]
    assert rel(b, b_ref) < TOL_MAT
    A = ctx.discrete_kernel(g, "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
    A_ref = z["A"] if "A" in z else O.discrete_kernel(g, "combined", k, eta, QUAD,
                                                      alpha=2.0, beta=1.0)
    x_ref = z["x"]
    smax, cond = ctx.norm_cond(A)
    nb = np.linalg.norm(b)
    eA = np.linalg.norm(A - A_ref) / smax
    eb = np.linalg.norm(b - b_ref) / nb
    be_ref = np.linalg.norm(b_ref - A_ref @ x_ref) / (smax * np.linalg.norm(x_ref) +
                                                      np.linalg.norm(b_ref))
    for prec in ("fp64", "mixed"):
        x = ctx.scattering_solve(g, k, d, eta, QUAD, precision=prec)
        r = np.linalg.norm(b - A @ x)
        be = r / (smax * np.linalg.norm(x) + nb)
        be_f = r / (np.linalg.norm(A) * np.linalg.norm(x) + nb)  # the library's own measure
        bound = 2.0 * cond * (eA + eb + be + be_ref)
        err = rel(x, x_ref)
        report = ("%s: cond %.3g eA %.2g eb %.2g be %.2g be_ref %.2g -> bound %.3g, error %.3g"
                  % (prec, cond, eA, eb, be, be_ref, bound, err))
        print(name, report)
        assert be_f <= 1e-14, report
        assert err <= bound, report


def test_device_pointers_and_leading_dimension(ctx):
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import geometry as G
    g = G.kite(96).add_poly_basis(0)
    A_host = ctx.discrete_kernel(g, "combined", 12.0, 12.0, QUAD, alpha=2.0, beta=1.0)
    n = g.n_unknowns
    # device output with a padded leading dimension (ld = n + 7)
    buf = torch.zeros((n, n + 7), dtype=torch.complex128, device="cuda")
    view = buf.t()  # column-major view: (n + 7) x n, entry (i,j) at i + j*(n+7)
    from bem2d_gb300 import capi
    import ctypes
    gh = capi._GeomHold(g)
    qq = capi.quad(QUAD)
    rc = ctx.lib.bem2d_discrete_kernel(ctx.h, ctypes.byref(gh.c), ctypes.byref(qq), 3, 12.0, 0.0,
                                       12.0, 2.0, 1.0, ctypes.c_void_p(buf.data_ptr()), n + 7)
    assert rc == 0
    A_dev = view[:n, :].cpu().numpy()
    assert np.array_equal(A_dev, A_host)


def test_oracle_at_kite_config_size(ctx):
    """Kite, N = 2048, k = 100 (the benchmark workload): GPU vs the CPU
    oracle on 64 full rows and the right-hand side."""
    from bem2d_gb300 import geometry as G
    from oracle import oracle as O
    from golden.cases import seeded_angle
    import math
    g = G.kite(2048).add_poly_basis(0)
    th = seeded_angle(0)
    d = (math.cos(th), math.sin(th))
    A = ctx.discrete_kernel(g, "combined", 100.0, 100.0, QUAD, alpha=2.0, beta=1.0)
    rows = np.random.default_rng(3).choice(2048, 64, replace=False)
    R = O.discrete_kernel_rows(g, rows, "combined", 100.0, 100.0, QUAD, alpha=2.0, beta=1.0)
    # Rounding floor of the FP64 formulation itself: moving every element's
    # parameter t1 by one ulp changes the reference matrix by `floor` (the
    # double-layer term n.(x - y) cancels for near pairs on a curve).  The GPU
    # result must agree with the oracle to 1e-12 or to within 3x that floor.
    g2 = G.kite(2048).add_poly_basis(0)
    rng = np.random.default_rng(1)
    for p in g2.param:
        p[0] = float(np.nextafter(p[0], 2.0 if rng.random() < 0.5 else -2.0))
    R2 = O.discrete_kernel_rows(g2, rows[:16], "combined", 100.0, 100.0, QUAD, alpha=2.0,
                                beta=1.0)
    floor = rel(R2, R[:16])
    assert rel(A[rows, :], R) < max(TOL_MAT, 3 * floor), floor
    b = ctx.rhs(g, 100.0, d, 100.0, QUAD)
    assert rel(b, O.rhs(g, 100.0, d, 100.0)) < TOL_MAT


@pytest.mark.parametrize("n", [400, 1500])
def test_fine_ellipse_arc_matches_oracle(ctx, n):
    """Fine elliptic-arc meshes (the sweep's): FP64 and mixed assembly of the
    ellipse (2, 1), k = 40, against the CPU oracle on 48 full rows, to
    1e-12 relative or the rounding floor of the FP64 formulation (the
    oracle's own change when each element's first end point moves by one
    ulp), whichever is larger.  The self pairs' points need sincos-accurate
    positions: an addition-theorem evaluation (about one ulp more rounding
    per point) measured 2.4 floors here (2.2e-12 at n = 1500)."""
    from bem2d_gb300 import geometry as G
    from oracle import oracle as O
    g = G.ellipse_arc_closed(n).add_poly_basis(0)
    k = 40.0
    rows = np.random.default_rng(n).choice(n, 48, replace=False)
    R = O.discrete_kernel_rows(g, rows, "combined", k, k, QUAD, alpha=2.0, beta=1.0)
    g2 = G.ellipse_arc_closed(n).add_poly_basis(0)
    rng = np.random.default_rng(2)
    for p in g2.param:
        p[0] = float(np.nextafter(p[0], 10.0 if rng.random() < 0.5 else -10.0))
    floor = rel(O.discrete_kernel_rows(g2, rows[:12], "combined", k, k, QUAD, alpha=2.0,
                                       beta=1.0), R[:12])
    A = ctx.discrete_kernel(g, "combined", k, k, QUAD, alpha=2.0, beta=1.0)
    Am, _ = ctx.discrete_kernel_mixed(g, "combined", k, k, QUAD, alpha=2.0, beta=1.0)
    e64, emx = rel(A[rows, :], R), rel(Am[rows, :], R)
    print("ellipse arc n=%d: FP64 %.3g, mixed %.3g vs oracle (one-ulp floor %.3g)"
          % (n, e64, emx, floor))
    assert e64 < max(TOL_MAT, floor), floor
    assert emx < max(TOL_MAT, floor), floor


MIXED_CASES = ["disk160", "kite128", "ellipsearc100", "trefoil48", "invellipse48",
               "square_graded", "lshape_graded", "square_poly2", "triangle_lin", "two_squares"]


@pytest.mark.parametrize("name", MIXED_CASES)
def test_mixed_assembly_matches_fp64(ctx, name):
    """Far field in float-float on the FP32 pipe: within 1e-12 of the FP64
    assembly (relative Frobenius); the complex64 copy is its rounding."""
    spec = CASES[name]
    g = spec["geom"]()
    k, eta = spec["k"], spec["eta"]
    for kn in ("combined",) + tuple(spec.get("kernels", ())):
        a, b = (2.0, 1.0) if kn == "combined" else (1.0, 0.0)
        A64 = ctx.discrete_kernel(g, kn, k, eta, QUAD, alpha=a, beta=b)
        Am, A32 = ctx.discrete_kernel_mixed(g, kn, k, eta, QUAD, alpha=a, beta=b)
        if np.linalg.norm(A64) == 0:
            assert np.abs(Am).max() < 1e-15
            continue
        assert rel(Am, A64) < 1e-12, kn
        assert rel(A32.astype(np.complex128), Am) < 1e-7


def test_mixed_assembly_kite_config(ctx):
    """Kite N = 2048, k = 100: the mixed assembly against the FP64 one."""
    from bem2d_gb300 import geometry as G
    g = G.kite(2048).add_poly_basis(0)
    A64 = ctx.discrete_kernel(g, "combined", 100.0, 100.0, QUAD, alpha=2.0, beta=1.0)
    Am, A32 = ctx.discrete_kernel_mixed(g, "combined", 100.0, 100.0, QUAD, alpha=2.0, beta=1.0)
    assert rel(Am, A64) < 1e-12
    # entry-wise: no entry off by more than 1e-12 of the largest
    assert np.abs(Am - A64).max() < 1e-12 * np.abs(A64).max()


@pytest.mark.parametrize("n", [3, 47, 309])
def test_mixed_assembly_odd_sizes(ctx, n):
    """Odd unknown counts (the float-float node table then ends off a 16-byte
    boundary): mixed assembly and solve against the FP64 path."""
    from bem2d_gb300 import geometry as G
    g = G.ellipse_arc_closed(n).add_poly_basis(0)
    k = 20.0
    A64 = ctx.discrete_kernel(g, "combined", k, k, QUAD, alpha=2.0, beta=1.0)
    Am, _ = ctx.discrete_kernel_mixed(g, "combined", k, k, QUAD, alpha=2.0, beta=1.0)
    assert rel(Am, A64) < 1e-12
    x64 = ctx.scattering_solve(g, k, (1.0, 0.0), k, QUAD, precision="fp64")
    xm = ctx.scattering_solve(g, k, (1.0, 0.0), k, QUAD, precision="mixed")
    assert rel(xm, x64) < 1e-10
