"""GPU dense solve (SolveSystem replacement) through the C ABI.

FP64 LU: within 1e-12 of LAPACK's solution (relative 2-norm) on
well-conditioned matrices; mixed (complex64 LU + FP64 refinement): within
1e-10.  Zero pivots raise LapackError like the reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def rand_system(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += 2 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return np.asfortranarray(A), b


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [1, 2, 7, 63, 64, 65, 200, 513, 1100])
def test_fp64_and_mixed_match_lapack(ctx, n):
    A, b = rand_system(n, n)
    x_ref = np.linalg.solve(A, b)
    x = ctx.solve(A, b, "fp64")
    assert rel(x, x_ref) < 1e-12
    xm = ctx.solve(A, b, "mixed")
    assert rel(xm, x_ref) < 1e-10, ctx.last_info
    assert ctx.last_info[2] <= 1e-12


def test_pivoting_needed(ctx):
    # leading zero forces a row exchange; LAPACK-style partial pivoting
    A = np.asfortranarray([[0, 1, 2], [3, 4, 5], [6, 7, 9]], dtype=np.complex128)
    b = np.array([1, 2, 3], dtype=np.complex128)
    assert rel(ctx.solve(A, b, "fp64"), np.linalg.solve(A, b)) < 1e-14


def test_zero_pivot_raises_lapack_error(ctx):
    from bem2d_gb300 import capi
    A, b = rand_system(100, 5)
    A[:, 37] = 0
    with pytest.raises(capi.LapackError) as e:
        ctx.solve(A, b, "fp64")
    assert e.value.code == 38
    with pytest.raises(capi.LapackError):
        ctx.solve(A, b, "mixed")


def test_device_resident_inputs(ctx):
    torch = pytest.importorskip("torch")
    A, b = rand_system(300, 11)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # row-major A^T == column-major A
    bt = torch.from_numpy(b).cuda()
    xt = torch.zeros(300, dtype=torch.complex128, device="cuda")
    ctx.solve(At.t(), bt, "mixed", out=xt)
    assert rel(xt.cpu().numpy(), np.linalg.solve(A, b)) < 1e-10


def test_repeat_calls_reuse_workspace(ctx):
    for n in (400, 100, 400):
        A, b = rand_system(n, 100 + n)
        assert rel(ctx.solve(A, b, "fp64"), np.linalg.solve(A, b)) < 1e-12


def test_large_order_grid_solve():
    """n = 8200 uses the grid-wide triangular solves (n >= 8192): residual
    ||b - A x|| / (||A||_F ||x|| + ||b||) at FP64 roundoff for both
    precisions, inputs and outputs on the device."""
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import capi
    n = 8200
    g = torch.Generator(device="cuda").manual_seed(8200)
    A = torch.randn((n, n), dtype=torch.complex128, device="cuda", generator=g)
    A += 2 * n ** 0.5 * torch.eye(n, dtype=torch.complex128, device="cuda")
    b = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    At = A.T.contiguous().T  # column-major view of A
    ctx = capi.Context(0)
    try:
        for prec, bound in (("fp64", 1e-13), ("mixed", 1e-13)):
            x = torch.zeros(n, dtype=torch.complex128, device="cuda")
            ctx.solve(At, b, prec, out=x)
            r = torch.linalg.vector_norm(b - A @ x)
            berr = float(r / (torch.linalg.matrix_norm(A) * torch.linalg.vector_norm(x) +
                              torch.linalg.vector_norm(b)))
            assert berr < bound, (prec, berr)
    finally:
        ctx.close()


def _device_system(n, seed, row_scale=False):
    """A seeded complex Gaussian matrix on the device (no diagonal shift:
    pivoting matters on every column), optionally with rows scaled by
    10^U(-3, 3); column-major view and right-hand side."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn((n, n), dtype=torch.complex128, device="cuda", generator=g)
    if row_scale:
        s = 10.0 ** (6.0 * torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 3.0)
        A = A * s[:, None]
    b = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    return A, A.T.contiguous().T, b


@pytest.mark.parametrize("n,row_scale", [(4200, False), (7000, True), (9000, False)])
def test_tall_panels_tournament_pivoting(ctx, n, row_scale):
    """Orders above 4096 factor their tall complex64 panels (more rows than
    a 16-CTA cluster holds in registers) with the shared-memory rows panel
    up to 16 x 416 rows and with tournament pivoting beyond.  The mixed
    solve must still reach FP64 backward error, |b - A x| / (|A|_F |x| +
    |b|) < 1e-14, and agree with the FP64 path (partial pivoting) to the
    conditioning: |x_mixed - x_fp64| / |x_fp64| <= cond_est * 1e-14, with
    cond_est = |A|_F |x| / |b| (a lower bound of cond) times 10."""
    torch = pytest.importorskip("torch")
    A, Acm, b = _device_system(n, n, row_scale)
    xs = {}
    for prec in ("fp64", "mixed"):
        x = torch.zeros(n, dtype=torch.complex128, device="cuda")
        ctx.solve(Acm, b, prec, out=x)
        r = torch.linalg.vector_norm(b - A @ x)
        nA = torch.linalg.matrix_norm(A)
        berr = float(r / (nA * torch.linalg.vector_norm(x) + torch.linalg.vector_norm(b)))
        assert berr < 1e-14, (prec, berr, ctx.last_info)
        xs[prec] = x
    cond_est = 10.0 * float(torch.linalg.matrix_norm(A) * torch.linalg.vector_norm(xs["fp64"]) /
                            torch.linalg.vector_norm(b))
    err = float(torch.linalg.vector_norm(xs["mixed"] - xs["fp64"]) /
                torch.linalg.vector_norm(xs["fp64"]))
    assert err <= cond_est * 1e-14, (err, cond_est)


def test_tall_panel_zero_column_reports_its_pivot(ctx):
    """A zero column inside a tall panel (n = 8000, column 101 of the panel
    starting at row 64, 7936 rows: tournament pivoting): the tournament's
    candidates are all zero there, and both paths report LAPACK's info = 101
    as LapackError."""
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import capi
    A, Acm, b = _device_system(8000, 77)
    Acm[:, 100] = 0
    for prec in ("fp64", "mixed"):
        x = torch.zeros(8000, dtype=torch.complex128, device="cuda")
        with pytest.raises(capi.LapackError) as e:
            ctx.solve(Acm, b, prec, out=x)
        assert e.value.code == 101, prec


@pytest.mark.parametrize("n,cond", [(400, 1e9), (1500, 1e10)])
def test_mixed_gmres_ir_fallback_on_ill_conditioned(ctx, n, cond):
    """A = Q1 diag(s) Q2^H with n - 8 singular values in [0.5, 1] and eight
    geometric from 1e-3 down to 1/cond (a few near-singular directions, as
    near a resonance): cond(A) times the complex64 factor's error is far
    above one, so plain refinement cannot converge; the mixed solve must
    fall back to GMRES-IR and still reach the FP64 backward error
    |b - A x| / (|A|_F |x| + |b|) <= 1e-14, with a solution within
    cond * 1e-14 of the FP64 path's."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(n)

    def unitary():
        Z = torch.randn((n, n), dtype=torch.complex128, device="cuda", generator=g)
        Q, R = torch.linalg.qr(Z)
        return Q * (torch.diagonal(R) / torch.diagonal(R).abs())[None, :]

    s = torch.cat([0.5 + 0.5 * torch.rand(n - 8, dtype=torch.float64, device="cuda", generator=g),
                   torch.logspace(-3, -np.log10(cond), 8, dtype=torch.float64, device="cuda")])
    A = (unitary() * s[None, :]) @ unitary().conj().T
    b = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    Acm = A.T.contiguous().T
    xs = {}
    for prec in ("fp64", "mixed"):
        x = torch.zeros(n, dtype=torch.complex128, device="cuda")
        ctx.solve(Acm, b, prec, out=x)
        r = torch.linalg.vector_norm(b - A @ x)
        berr = float(r / (torch.linalg.matrix_norm(A) * torch.linalg.vector_norm(x) +
                          torch.linalg.vector_norm(b)))
        assert berr <= 1e-14, (prec, berr, ctx.last_info)
        xs[prec] = x
    assert ctx.last_info[1] > 2  # more than plain refinement's two steps
    err = float(torch.linalg.vector_norm(xs["mixed"] - xs["fp64"]) /
                torch.linalg.vector_norm(xs["fp64"]))
    assert err <= cond * 1e-14, err


def _berr(A, x, b):
    torch = pytest.importorskip("torch")
    r = torch.linalg.vector_norm(b - A @ x)
    return float(r / (torch.linalg.matrix_norm(A) * torch.linalg.vector_norm(x) +
                      torch.linalg.vector_norm(b)))


@pytest.mark.parametrize("n", [3000, 9000])
def test_update_precision_options(ctx, n):
    """The LU's tensor-core trailing update with 3xTF32 ("mixed") and 1xTF32
    ("mixed_tf32") products on a well-conditioned system (complex Gaussian
    plus 2 sqrt(n) I, cond(A) ~ 3): both reach the FP64 backward error
    |b - A x| / (|A|_F |x| + |b|) <= 1e-14 and agree with the FP64 path to
    cond_est * 1e-14 (cond_est = 10 |A|_F |x| / |b|, as above).  The 1xTF32
    factor is accurate to ~1e-3 instead of ~1e-6, so its refinement takes
    more steps; the line printed gives steps and errors per option."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(n + 1)
    A = torch.randn((n, n), dtype=torch.complex128, device="cuda", generator=g)
    A += 2.0 * np.sqrt(n) * torch.eye(n, dtype=torch.complex128, device="cuda")
    b = torch.randn(n, dtype=torch.complex128, device="cuda", generator=g)
    Acm = A.T.contiguous().T
    xs, its = {}, {}
    for prec in ("fp64", "mixed", "mixed_tf32"):
        x = torch.zeros(n, dtype=torch.complex128, device="cuda")
        ctx.solve(Acm, b, prec, out=x)
        assert _berr(A, x, b) <= 1e-14, (prec, ctx.last_info)
        xs[prec], its[prec] = x, ctx.last_info[1]
    cond_est = 10.0 * float(torch.linalg.matrix_norm(A) * torch.linalg.vector_norm(xs["fp64"]) /
                            torch.linalg.vector_norm(b))
    errs = {p: float(torch.linalg.vector_norm(xs[p] - xs["fp64"]) /
                     torch.linalg.vector_norm(xs["fp64"])) for p in ("mixed", "mixed_tf32")}
    print("n=%d cond_est=%.1f iterations %s rel_err_vs_fp64 %s" % (n, cond_est, its, errs))
    for p, e in errs.items():
        assert e <= cond_est * 1e-14, (p, e)
    assert its["mixed_tf32"] >= its["mixed"]


def test_update_1xtf32_falls_back_to_gmres_ir(ctx):
    """1xTF32 factor on a complex Gaussian matrix without a diagonal shift
    (n = 4200, cond(A) ~ 1e4): cond(A) times the factor's ~1e-3 error is
    above one, so plain refinement stalls; GMRES-IR with that factor must
    still reach |b - A x| / (|A|_F |x| + |b|) <= 1e-14."""
    torch = pytest.importorskip("torch")
    A, Acm, b = _device_system(4200, 4201)
    x = torch.zeros(4200, dtype=torch.complex128, device="cuda")
    ctx.solve(Acm, b, "mixed_tf32", out=x)
    assert _berr(A, x, b) <= 1e-14, ctx.last_info
    print("n=4200 mixed_tf32 steps (refinement + GMRES-IR factor applications):",
          ctx.last_info[1])
