"""The complex64 LU's tensor-core trailing update C -= A B (tcgen05
kind::tf32, 3xTF32) through bem2d_debug_tc_update, against a complex128
product of the same complex64 operands (torch on the GPU).

Bar, per entry: |C - C_ref| <= (K + 4) 2^-22 (|A| |B| + |C|)_ij, the
classical FP32 dot-product bound that the 3xTF32 split reproduces (each
product keeps about 21 bits, accumulation in FP32).  Shapes cover full and
ragged tiles (64 x 128 complex), K below, at and above a 16-deep chunk, the
rank-64 and rank-256 updates of the LU, padded leading dimensions, and more
tiles than SMs (the persistent schedule wraps)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def colmajor(torch, rows, cols, gen, pad=0):
    """A complex64 column-major rows x cols view with leading dimension rows + pad."""
    T = torch.randn((cols, rows + pad), dtype=torch.complex64, device="cuda", generator=gen)
    return T[:, :rows].t()


@pytest.mark.parametrize("M,N,K,pad", [
    (1, 1, 1, 0), (64, 128, 16, 0), (65, 129, 17, 3), (128, 256, 64, 0), (300, 200, 64, 5),
    (3000, 2000, 64, 0), (2048, 64, 64, 0), (1000, 1000, 256, 1), (4096, 4096, 256, 0),
    (700, 3000, 40, 2)])
def test_tc_update_matches_complex128(ctx, M, N, K, pad):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(M * 7919 + N * 104729 + K)
    C = colmajor(torch, M, N, g, pad)
    A = colmajor(torch, M, K, g, pad)
    B = colmajor(torch, K, N, g, pad)
    c128 = torch.complex128
    ref = C.to(c128) - A.to(c128) @ B.to(c128)
    scale = A.abs().double() @ B.abs().double() + C.abs().double()
    ctx.tc_update(C, A, B)
    err = ((C.to(c128) - ref).abs() / scale).max().item()
    bound = (K + 4) * 2.0 ** -22
    print("tc update M=%d N=%d K=%d: max relative error %.3g (bound %.3g)" % (M, N, K, err, bound))
    assert err <= bound
