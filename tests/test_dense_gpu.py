"""GPU dense operators through the C ABI: ChangeBasis, L2NormCond (Lanczos
extreme singular values), NumRange eigenvalues and EvalKernel potentials,
against the reference's outputs (tests/golden) and the CPU oracle."""
import json
import os

import numpy as np
import pytest

from golden.cases import CASES, QUAD

pytestmark = pytest.mark.gpu


def _load(name):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    return z, json.loads(str(z["meta"]))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def blocks_of(g):
    """Unknown ranges per element (the mass matrix's diagonal blocks)."""
    ue = g.arrays()["unk_elem"]
    starts = [0] + [i for i in range(1, len(ue)) if ue[i] != ue[i - 1]] + [len(ue)]
    return np.array(starts, dtype=np.int32)


@pytest.mark.parametrize("name", ["disk160", "kite128", "square_poly2", "triangle_lin"])
def test_change_basis_matches_oracle(ctx, name):
    from oracle import oracle as O
    spec = CASES[name]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    M = ctx.eval_ident(g, QUAD)
    B = ctx.change_basis(A, M, blocks_of(g))
    R = O.change_basis(A, M)
    assert rel(B, R) < 1e-13


@pytest.mark.parametrize("name", ["disk160", "diskchords64", "kite128", "ellipsearc100",
                                  "square_graded", "square_poly2", "two_squares",
                                  "square_numrange"])
def test_norm_cond_matches_reference(ctx, name):
    """SoundSoftScattering::NormCond = L2NormCond(ChangeBasis(A, Id))."""
    z, meta = _load(name)
    spec = CASES[name]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    nrm, cond = ctx.norm_cond(B)
    ref_n, ref_c = z["normcond"]
    assert abs(nrm - ref_n) < 1e-11 * ref_n
    assert abs(cond - ref_c) < 1e-9 * ref_c


def test_norm_cond_random(ctx):
    rng = np.random.default_rng(5)
    n = 300
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 3 * np.sqrt(n) * np.eye(n)
    s = np.linalg.svd(A, compute_uv=False)
    nrm, cond = ctx.norm_cond(A)
    assert abs(nrm - s[0]) < 1e-12 * s[0]
    assert abs(cond - s[0] / s[-1]) < 1e-10 * cond


def test_num_range_matches_reference(ctx):
    """lambda_max per angle vs zheev (oracle), and the reference's NumRange
    boundary points (written with 6 digits)."""
    from oracle import oracle as O
    z, meta = _load("square_numrange")
    spec = CASES["square_numrange"]
    g = spec["geom"]()
    A = ctx.discrete_kernel(g, "combined", spec["k"], spec["eta"], QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    n = spec["numrange"]
    th = np.concatenate([np.arange(n) * np.pi / n, np.arange(n) * np.pi / n + np.pi])
    lm = ctx.num_range_lmax(B, th)
    ref = O.numrange_lmax(B, th)
    assert np.abs(lm - ref).max() < 1e-12 * np.abs(ref).max()
    # complex64 Lanczos + complex128 Lanczos from its Ritz vectors: same bar
    lm_mixed = ctx.num_range_lmax(B, th, precision="mixed")
    assert np.abs(lm_mixed - ref).max() < 1e-12 * np.abs(ref).max()
    steps = np.arange(n) * np.pi / n
    eigs = np.concatenate([-lm[n:], lm[:n], [-lm[n]]])
    st = np.concatenate([steps, steps, [0.0]])
    pts = []
    for i in range(2 * n):
        c1, c2, s1, s2 = np.cos(st[i]), np.cos(st[i + 1]), np.sin(st[i]), np.sin(st[i + 1])
        t1 = (eigs[i + 1] - eigs[i] * (c1 * c2 + s1 * s2)) / (s1 * c2 - s2 * c1)
        pts.append(np.exp(-1j * st[i]) * (eigs[i] + 1j * t1))
    pts.append(pts[0])
    assert np.abs(np.array(pts) - z["numrange"]).max() < 1e-5 * np.abs(z["numrange"]).max()


@pytest.mark.parametrize("name", ["disk160", "kite128"])
def test_evalsol_matches_reference(ctx, name):
    """u = u_inc - S phi at field points (SoundSoftScattering::EvalSol)."""
    z, meta = _load(name)
    spec = CASES[name]
    g = spec["geom"]()
    k, d = spec["k"], spec["direction"]
    x = ctx.scattering_solve(g, k, d, spec["eta"], QUAD, precision="fp64")
    pts = z["evalsol_points"]
    pot = ctx.potential(g, x, pts, "single", k)
    uinc = np.exp(1j * k * (d[0] * pts[:, 0] + d[1] * pts[:, 1]))
    assert rel(uinc - pot, z["evalsol"]) < 1e-11


@pytest.mark.parametrize("kernel", ["single", "double", "conjdouble", "combined"])
def test_potential_matches_oracle(ctx, kernel):
    from oracle import oracle as O
    g = CASES["square_poly2"]["geom"]()
    rng = np.random.default_rng(9)
    c = rng.standard_normal(g.n_unknowns) + 1j * rng.standard_normal(g.n_unknowns)
    pts = rng.uniform(-1.0, 2.0, (257, 2))
    out = ctx.potential(g, c, pts, kernel, 7.0, 3.0)
    ref = O.potential(g, c, pts, kernel, 7.0, 3.0)
    assert rel(out, ref) < 1e-12


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (64, 64, 64), (300, 17, 129), (1000, 700, 1500),
                                   (2048, 2048, 2048)])
def test_matmul_matches_numpy(ctx, m, n, k):
    """Matrix * Matrix (cblas_zgemm in the reference): complex128 product on
    the GPU within 1e-14 sqrt(k) of numpy's, relative to |A| |B|."""
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    C = ctx.matmul(A, B)
    R = A @ B
    scale = np.abs(A) @ np.abs(B)
    assert (np.abs(C - R) / scale).max() < 1e-14 * max(1, k ** 0.5)


@pytest.mark.parametrize("n", [1100, 2500])
def test_norm_cond_mixed_inverse_path(ctx, n):
    """From 1024 unknowns the mixed norm / condition number iterates with the
    explicit complex64 inverse W = U^{-1} L^{-1} (products with W and W^H
    instead of triangular solves; FP64 refinement of every product in the
    second phase).  A = Q1 diag(s) Q2^H with seeded unitary Q1, Q2 and known
    singular values (sigma_max = 300 and sigma_min = 0.5 separated from the
    rest, which lie in [1, 150], as the boundary-element operators' extreme
    values are): sigma_max to 1e-12, sigma_min and cond to 1e-10 for both
    precisions."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(n)

    def unitary():
        Z = torch.randn((n, n), dtype=torch.complex128, device="cuda", generator=g)
        Q, R = torch.linalg.qr(Z)
        return Q * (torch.diagonal(R) / torch.diagonal(R).abs())[None, :]

    rng = np.random.default_rng(n)
    s = np.concatenate([[300.0], rng.uniform(1.0, 150.0, n - 2), [0.5]])
    A = (unitary() * torch.from_numpy(s).cuda()[None, :]) @ unitary().conj().T
    Acm = A.T.contiguous().T  # column-major view of A
    for prec in ("mixed", "fp64"):
        nrm, cond = ctx.norm_cond(Acm, precision=prec)
        assert abs(nrm - 300.0) < 1e-12 * 300.0, (prec, nrm)
        smin = nrm / cond
        assert abs(smin - 0.5) < 1e-10 * 0.5, (prec, smin)
        assert abs(cond - 600.0) < 1e-10 * 600.0, (prec, cond)


def test_num_range_mixed_matches_fp64_at_size(ctx):
    """Unit square with 256 elements per side (N = 1024), k = 20, 36
    angles, tol = 1e-11: the mixed scan (complex64 Lanczos, then the
    complex128 Lanczos whose products with A run in float-float on the FP32
    pipe) against the plain FP64 scan: |lambda_mixed - lambda_fp64| <=
    2e-11 max |lambda| (both stop at 1e-11 of |H|), and both against dense
    eigvalsh (torch, complex128) at six angles to the same bar."""
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import geometry as G
    g = G.polygon_uniform([(0, 0), (1, 0), (1, 1), (0, 1)], 256).add_poly_basis(0)
    A = ctx.discrete_kernel(g, "combined", 20.0, 20.0, QUAD, alpha=2.0, beta=1.0)
    B = ctx.change_basis(A, ctx.eval_ident(g, QUAD), blocks_of(g))
    th = 2 * np.pi * np.arange(36) / 36
    lm = ctx.num_range_lmax(B, th, tol=1e-11, precision="mixed")
    l64 = ctx.num_range_lmax(B, th, tol=1e-11, precision="fp64")
    scale = np.abs(l64).max()
    assert np.abs(lm - l64).max() <= 2e-11 * scale
    Bt = torch.from_numpy(np.asarray(B)).cuda()
    for j in range(0, 36, 6):
        z = complex(np.cos(th[j]), np.sin(th[j]))
        H = 0.5 * (z * Bt + np.conj(z) * Bt.conj().T)
        ev = float(torch.linalg.eigvalsh(H)[-1])
        assert abs(lm[j] - ev) <= 2e-11 * scale, (j, lm[j], ev)
        assert abs(l64[j] - ev) <= 2e-11 * scale, (j, l64[j], ev)
