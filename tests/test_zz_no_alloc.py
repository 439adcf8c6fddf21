"""The allocation-free dense solve (bem2d_solve_system_noalloc) through the C ABI.

Two calls in a row, each checked against bem2d_solve_system (FP64) on the same
system within the FP64 solve tolerance of the other tests (1e-12, relative
2-norm): first a seeded n = 1000 system from host memory, then the n = 160
scattering matrix of the unit disk (reference golden fixture) from device
memory, so the second call runs on the scratch array the first one left
behind.  The device's free memory must not change across the second call.
Collected last so that it also runs after every other GPU test."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12


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


def test_two_calls_match_solve_system(ctx):
    torch = pytest.importorskip("torch")
    # call 1: host buffers, n = 1000
    A1, b1 = rand_system(1000, 2024)
    x1_ref = ctx.solve(A1, b1, "fp64")
    # call 2 inputs: the disk scattering system, on the device
    g = np.load(os.path.join(GOLDEN, "disk160.npz"))
    A2, b2 = np.asfortranarray(g["A"]), g["rhs"]
    x2_ref = ctx.solve(A2, b2, "fp64")

    x1 = ctx.solve_noalloc(A1, b1)
    assert ctx.last_info[0] == 0
    assert rel(x1, x1_ref) < TOL
    assert rel(x1, np.linalg.solve(A1, b1)) < TOL

    A2t = torch.from_numpy(np.ascontiguousarray(A2.T)).cuda()  # row-major A^T
    b2t = torch.from_numpy(b2).cuda()
    x2t = torch.zeros(A2.shape[0], dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    ctx.solve_noalloc(A2t.t(), b2t, out=x2t)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before
    x2 = x2t.cpu().numpy()
    assert rel(x2, x2_ref) < TOL
    assert rel(x2, g["x"]) < TOL  # the reference's own LAPACK solution


def test_largest_order(ctx):
    """n = BEM2D_NOALLOC_MAX_N, the order whose work buffers come closest to
    the size of the static array: the host-side layout check says they fit,
    and the solution matches bem2d_solve_system and LAPACK."""
    from bem2d_gb300 import capi
    fits, need, cap = capi.noalloc_scratch_fits()
    assert fits and need <= cap, (need, cap)
    n = capi.NOALLOC_MAX_N
    A, b = rand_system(n, 7)
    x = ctx.solve_noalloc(A, b)
    assert ctx.last_info[0] == 0
    assert rel(x, ctx.solve(A, b, "fp64")) < TOL
    assert rel(x, np.linalg.solve(A, b)) < TOL


def test_rejects_n_above_limit(ctx):
    from bem2d_gb300 import capi
    n = capi.NOALLOC_MAX_N + 1
    A = np.eye(n, dtype=np.complex128, order="F")
    b = np.ones(n, dtype=np.complex128)
    with pytest.raises(capi.Bem2dError) as e:
        ctx.solve_noalloc(A, b)
    assert e.value.code == -1
    assert "BEM2D_NOALLOC_MAX_N = %d" % capi.NOALLOC_MAX_N in str(e.value)


def test_zero_pivot_reported_like_solve_system(ctx):
    from bem2d_gb300 import capi
    A, b = rand_system(100, 5)
    A[:, 37] = 0
    with pytest.raises(capi.LapackError) as e:
        ctx.solve_noalloc(A, b)
    assert e.value.code == 38
