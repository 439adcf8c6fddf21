"""Parity at the full sizes of the large target workloads.

* Graded L-shape, N = 16384, k = 500 (the large single solve): 64 seeded full
  rows of the FP64 GPU matrix and the right-hand side against the CPU oracle
  (a C restatement of the reference's DiscreteKernel / DotProdBasFuns, pinned
  to the reference's fixtures); the mixed solution's backward error against
  the FP64-assembled A; mixed against the plain FP64 solution.
* Graded square, N = 8192, k = 200 (norm and condition number of
  ChangeBasis(A, Id), as SoundSoftScattering::NormCond): both arithmetic modes
  of L2NormCond against a second method, the extreme eigenvalues of B^H B
  (cuSOLVER through torch.linalg.eigvalsh).
At these sizes the reference itself would take hours on the CPU; the
smaller graded cases of tests/golden pin the same code paths against the
reference's own outputs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QUAD = (3, 5, 0.15)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def test_lshape16384_rows_rhs_and_solutions(ctx):
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import capi
    from bem2d_gb300 import geometry as G
    from oracle import oracle as O
    g = G.lshape(4072, 8, 0.15).add_poly_basis(0)
    n = g.n_unknowns
    assert n == 16384
    k = eta = 500.0
    d = (1.0, 0.0)
    hold = capi._GeomHold(g.arrays())
    A = torch.empty((n, n), dtype=torch.complex128, device="cuda")  # holds A^T
    ctx.discrete_kernel(hold.arrays, "combined", k, eta, QUAD, 2.0, 1.0, out=A)
    rows = np.sort(np.random.default_rng(3).choice(n, 64, replace=False))
    R = O.discrete_kernel_rows(g, rows, "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
    Ar = A[:, torch.from_numpy(rows).cuda()].T.cpu().numpy()
    # rounding floor of the FP64 formulation: the reference matrix moves by
    # `floor` when each element's first end point moves by one ulp
    g2 = G.lshape(4072, 8, 0.15).add_poly_basis(0)
    rng = np.random.default_rng(1)
    for p in g2.param:
        p[0] = float(np.nextafter(p[0], 2.0 if rng.random() < 0.5 else -2.0))
    R2 = O.discrete_kernel_rows(g2, rows[:16], "combined", k, eta, QUAD, alpha=2.0, beta=1.0)
    floor = rel(R2, R[:16])
    err_rows = rel(Ar, R)
    print("L-shape rows vs oracle %.3g (one-ulp floor %.3g)" % (err_rows, floor))
    assert err_rows < max(1e-12, 3 * floor)
    b = ctx.rhs(hold.arrays, k, d, eta, QUAD)
    assert rel(b, O.rhs(g, k, d, eta)) < 1e-12
    bt = torch.from_numpy(b).cuda()
    nA = float(torch.linalg.matrix_norm(A))
    nb = float(np.linalg.norm(b))
    xs = {}
    # mixed: 3xTF32 trailing updates; mixed_tf32: 1xTF32 (more refinement)
    for prec in ("mixed", "mixed_tf32", "fp64"):
        x = torch.zeros(n, dtype=torch.complex128, device="cuda")
        ctx.scattering_solve(hold.arrays, k, d, eta, QUAD, precision=prec, out=x)
        r = bt - A.T @ x
        be = float(torch.linalg.vector_norm(r)) / (nA * float(torch.linalg.vector_norm(x)) + nb)
        print("L-shape %s backward error %.3g, steps %d" % (prec, be, ctx.last_info[1]))
        assert be <= 1e-14, (prec, be)
        xs[prec] = x
    for prec in ("mixed", "mixed_tf32"):
        dx = float(torch.linalg.vector_norm(xs[prec] - xs["fp64"]) /
                   torch.linalg.vector_norm(xs["fp64"]))
        print("L-shape %s vs FP64 %.3g" % (prec, dx))
        assert dx <= 1e-10, prec


def test_square8192_norm_cond(ctx):
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import capi
    from bem2d_gb300 import geometry as G
    g = G.graded_square(2032, 8, 0.15).add_poly_basis(0)
    n = g.n_unknowns
    assert n == 8192
    hold = capi._GeomHold(g.arrays())
    A = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    M = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    B = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    ctx.discrete_kernel(hold.arrays, "combined", 200.0, 200.0, QUAD, 2.0, 1.0, out=A)
    ctx.eval_ident(hold.arrays, QUAD, out=M)
    ctx.change_basis(A, M, np.arange(n + 1, dtype=np.int32), out=B)
    # second method: eigenvalues of B^H B (cuSOLVER heevd through torch);
    # squaring costs cond(B)^2 eps in relative accuracy, ~1e-13 at cond ~ 23
    Bt = B.T  # the column-major matrix as a torch view
    ev = torch.linalg.eigvalsh(Bt.conj().T @ Bt)
    smax, smin = float(ev[-1]) ** 0.5, float(ev[0]) ** 0.5
    for prec in ("fp64", "mixed"):
        nrm, cond = ctx.norm_cond(B, precision=prec)
        e = (abs(nrm - smax) / smax, abs(cond / nrm - 1 / smin) * smin,
             abs(cond - smax / smin) / (smax / smin))
        print("square8192 %s: norm %.15g cond %.15g, rel. errors %s" % (prec, nrm, cond, e))
        assert max(e) < 1e-10, (prec, e)
