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
