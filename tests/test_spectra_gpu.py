"""Dense spectra on the GPU: SingularValues (lib/bem2d_mathroutines.cpp:268-320,
zgesvd), HermitianEigenvalues (:353-433, zheev 'N', 'U') and Eigenvalues
(:437-466, zgeev 'N', 'N') through the C ABI.

Bars: singular values within 1e-12 sigma_max of LAPACK's (numpy) and of the
reference's own output (tests/golden/square_numrange.npz: SingularValues of
ChangeBasis(A, Id)); Hermitian eigenvalues within 1e-12 ||H||_2 of LAPACK's
eigvalsh on the matrix the upper triangle defines; general eigenvalues
within 1e-12 max|lambda| of known eigenvalues of normal matrices and within
1e-11 ||A||_2 of LAPACK's zgeev (numpy) for random and boundary-element
matrices, matched as sets.  Householder reduction, bisection and shifted QR
are backward stable: absolute errors ~ n eps ||A|| times the eigenvalues'
condition numbers.
"""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, QUAD

pytestmark = pytest.mark.gpu


def _load(name):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    return z, json.loads(str(z["meta"]))


def blocks_of(g):
    ue = g.arrays()["unk_elem"]
    starts = [0] + [i for i in range(1, len(ue)) if ue[i] != ue[i - 1]] + [len(ue)]
    return np.array(starts, dtype=np.int32)


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 130, 301])
def test_singular_values_random(ctx, n):
    rng = np.random.default_rng(n)
    A = crandn(rng, n, n)
    s = ctx.singular_values(A)
    ref = np.linalg.svd(A, compute_uv=False)
    assert np.all(np.diff(s) <= 0)
    assert np.abs(s - ref).max() <= 1e-12 * ref[0]


def test_singular_values_graded_spectrum(ctx):
    """Singular values spread over 10 decades: small ones to absolute accuracy."""
    rng = np.random.default_rng(3)
    n = 96
    U, _ = np.linalg.qr(crandn(rng, n, n))
    V, _ = np.linalg.qr(crandn(rng, n, n))
    sig = np.logspace(0, -10, n)
    A = (U * sig) @ V.conj().T
    s = ctx.singular_values(A)
    assert np.abs(s - sig).max() <= 1e-13


@pytest.mark.parametrize("n", [1, 2, 5, 64, 257])
def test_hermitian_eigenvalues_random(ctx, n):
    rng = np.random.default_rng(100 + n)
    A = crandn(rng, n, n)  # lower triangle and the diagonal's imaginary part are ignored
    H = np.triu(A, 1) + np.triu(A, 1).conj().T + np.diag(A.diagonal().real)
    w = ctx.hermitian_eigenvalues(A)
    ref = np.linalg.eigvalsh(H)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref).max() <= 1e-12 * np.abs(ref).max()


def test_singular_values_match_reference(ctx):
    """SingularValues(ChangeBasis(A, Id)) as the reference computed it."""
    z, _ = _load("square_numrange")
    spec = CASES["square_numrange"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    s = ctx.singular_values(B)
    ref = z["singvals"]
    assert np.abs(s - ref).max() <= 1e-12 * ref[0]


def test_resonance_scan_quantity(ctx):
    """The resonance scan (resonances/trapresonance.cpp) reads 1 / sigma_min of
    ChangeBasis(A, Id) at complex k: here k = 6 - i on the trapping domain,
    against the reference's norm and condition number of the same matrix."""
    z, _ = _load("trap_ck")
    spec = CASES["trap_ck"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", complex(spec["k"], spec["kim"]), spec["eta"], QUAD,
                            alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    s = ctx.singular_values(B)
    ref_n, ref_c = z["normcond"]
    assert abs(s[0] - ref_n) <= 1e-11 * ref_n
    assert abs(s[-1] - ref_n / ref_c) <= 1e-11 * ref_n


def test_device_buffers(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    n = 50
    A = crandn(rng, n, n)
    # column-major view of a row-major torch tensor: store A^T row-major
    dAt = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    from bem2d_gb300 import capi
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    ctx._check(ctx.lib.bem2d_singular_values(ctx.h, n, capi._ptr(dAt), n, capi._ptr(out)))
    ref = np.linalg.svd(A, compute_uv=False)
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-12 * ref[0]


def test_rejects_bad_arguments(ctx):
    from bem2d_gb300 import capi
    with pytest.raises(capi.Bem2dError):
        ctx._check(ctx.lib.bem2d_singular_values(ctx.h, 0, None, 1, None))
    A = np.zeros((4, 4), dtype=np.complex128, order="F")
    out = np.zeros(4)
    with pytest.raises(capi.Bem2dError):  # lda < n
        ctx._check(ctx.lib.bem2d_hermitian_eigenvalues(ctx.h, 4, capi._ptr(A), 3, capi._ptr(out)))


def match_err(a, b):
    """Largest distance between the eigenvalue sets a and b under the best
    one-to-one pairing."""
    from scipy.optimize import linear_sum_assignment
    C = np.abs(a[:, None] - b[None, :])
    r, c = linear_sum_assignment(C)
    return C[r, c].max()


@pytest.mark.parametrize("n", [1, 2, 3, 10, 64, 200])
def test_eigenvalues_random(ctx, n):
    rng = np.random.default_rng(200 + n)
    A = crandn(rng, n, n)
    w = ctx.eigenvalues(A)
    assert match_err(w, np.linalg.eigvals(A)) <= 1e-11 * np.linalg.norm(A, 2)


def test_eigenvalues_normal_known(ctx):
    rng = np.random.default_rng(17)
    n = 120
    Q, _ = np.linalg.qr(crandn(rng, n, n))
    lam = crandn(rng, n)
    A = (Q * lam) @ Q.conj().T
    w = ctx.eigenvalues(A)
    assert match_err(w, lam) <= 1e-12 * np.abs(lam).max() * 10


def test_eigenvalues_structured(ctx):
    rng = np.random.default_rng(4)
    T = np.triu(crandn(rng, 40, 40))
    assert match_err(ctx.eigenvalues(T), np.diag(T)) <= 1e-13 * np.abs(T).max()
    assert np.abs(ctx.eigenvalues(np.eye(7, dtype=np.complex128)) - 1).max() <= 1e-15
    assert np.abs(ctx.eigenvalues(np.zeros((5, 5), dtype=np.complex128))).max() == 0


def test_eigenvalues_boundary_element_matrix(ctx):
    """The numrangecomps drivers' call: Eigenvalues(ChangeBasis(A, Id))."""
    spec = CASES["square_numrange"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    w = ctx.eigenvalues(B)
    assert match_err(w, np.linalg.eigvals(B)) <= 1e-11 * np.linalg.norm(B, 2)


def _zgeev_normalised(V):
    """zgeev's normalisation of eigenvector columns: unit 2-norm, the first
    entry of largest modulus real and positive."""
    V = V / np.linalg.norm(V, axis=0)
    k = np.argmax(np.abs(V) ** 2, axis=0)
    ph = V[k, np.arange(V.shape[1])]
    return V * (np.conj(ph) / np.abs(ph))


def _check_eigenvectors(A, w, V, tol_res, tol_vec=None):
    """Residuals |A v - lambda v| <= tol_res |A|_2 for every pair, unit
    columns with a real positive largest entry, the eigenvalues as a set
    against LAPACK's zgeev, and (tol_vec) each vector against LAPACK's for
    eigenvalues separated from the rest by at least 1e-3 |A|_2, up to a unit
    phase (ties in the largest modulus, as in the symmetric vectors of a
    square's matrix, make zgeev's choice of phase a matter of rounding)."""
    n = A.shape[0]
    nrm = np.linalg.norm(A, 2) if n else 1.0
    R = A @ V - V * w[None, :]
    assert np.abs(np.linalg.norm(V, axis=0) - 1).max() < 1e-13
    k = np.argmax(np.abs(V) ** 2, axis=0)
    top = V[k, np.arange(n)]
    assert np.abs(top.imag).max() == 0 and (top.real > 0).all()
    assert (np.linalg.norm(R, axis=0) / max(nrm, 1e-300)).max() <= tol_res
    wl, Vl = np.linalg.eig(A)
    assert match_err(w, wl) <= 1e-11 * max(nrm, 1e-300)
    if tol_vec is not None:
        Vl = _zgeev_normalised(Vl)
        for i in range(n):
            j = int(np.argmin(np.abs(wl - w[i])))
            gap = np.partition(np.abs(w - w[i]), 1)[1] if n > 1 else np.inf
            if gap < 1e-3 * nrm:
                continue
            p = np.vdot(Vl[:, j], V[:, i])  # Vl_j rotated onto V_i's phase
            dist = np.linalg.norm(V[:, i] - (p / abs(p)) * Vl[:, j])
            assert dist <= tol_vec * nrm / gap, (i, gap, dist)


@pytest.mark.parametrize("n", [1, 2, 3, 10, 64, 200])
def test_eigenvectors_random(ctx, n):
    rng = np.random.default_rng(300 + n)
    A = crandn(rng, n, n)
    w, V = ctx.eigenvectors(A)
    _check_eigenvectors(A, w, V, 1e-13 * max(1, n) ** 0.5, 1e-12)


def test_eigenvectors_triangular_and_diagonal(ctx):
    rng = np.random.default_rng(9)
    T = np.triu(crandn(rng, 30, 30))
    w, V = ctx.eigenvectors(T)
    _check_eigenvectors(T, w, V, 1e-13)
    D = np.diag(np.arange(1, 9) + 0.5j)
    w, V = ctx.eigenvectors(D)
    P = np.abs(V)  # a permutation: one unit entry per column, matching w
    assert np.abs(P.max(axis=0) - 1).max() < 1e-15 and np.abs(P.sum(axis=0) - 1).max() < 1e-14
    assert np.abs(w - np.diag(D)[np.argmax(P, axis=0)]).max() < 1e-15


def test_eigenvectors_boundary_element_matrix(ctx):
    """squaredensity.cpp's call: Eigenvalues(ChangeBasis(A, Id), w, V) on the
    boundary-element matrix (eigenvalues cluster near 1, a compact
    perturbation of the identity)."""
    spec = CASES["square_numrange"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    w, V = ctx.eigenvectors(B)
    _check_eigenvectors(B, w, V, 1e-13, 1e-11)
