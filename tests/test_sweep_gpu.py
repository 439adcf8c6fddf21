"""Batched wavenumber sweep (bem2d_sweep_solve) through the C ABI.

Every problem of a sweep must give the solution of the single-problem entry
(bem2d_scattering_solve) on the same inputs: the sweep only changes where and
when the work runs, so the tolerance is 1e-14 (relative 2-norm), for both
precisions.  The mixed sweep's solutions must also be within 1e-10 of the FP64
ones, the bar of the mixed path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def small_sweep(nk=10):
    """Ellipse (2,1) sweep with the N_k = ceil(10 k P / 2pi) rule, k in [3, 30]."""
    from bem2d_gb300 import geometry as G
    ks, ns = G.sweep_sizes(nk, 3.0, 30.0)
    return [G.ellipse_arc_closed(n).add_poly_basis(0) for n in ns], ks


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_matches_single_solves(ctx, precision):
    geoms, ks = small_sweep()
    d = (np.cos(0.7), np.sin(0.7))
    xs = ctx.sweep_solve(geoms, ks, d, precision=precision, nworkers=4)
    for g, k, x in zip(geoms, ks, xs):
        xr = ctx.scattering_solve(g, k, d, precision=precision)
        assert rel(x, xr) < 1e-14, (k, g.n_unknowns)
    if precision == "mixed":
        for g, k, x in zip(geoms, ks, xs):
            assert rel(x, ctx.scattering_solve(g, k, d, precision="fp64")) < 1e-10
        assert all(info[0] == 0 and info[2] <= 1e-12 for info in ctx.sweep_infos)


def test_sweep_repeat_and_more_workers_than_problems(ctx):
    geoms, ks = small_sweep(3)
    d = (1.0, 0.0)
    x1 = ctx.sweep_solve(geoms, ks, d, nworkers=16)
    x2 = ctx.sweep_solve(geoms, ks, d, nworkers=2)
    for a, b in zip(x1, x2):
        assert rel(a, b) < 1e-14


def test_sweep_device_outputs_and_eta(ctx):
    torch = pytest.importorskip("torch")
    geoms, ks = small_sweep(4)
    etas = np.cbrt(ks ** 2)  # the reference's second coupling, eta = k^(2/3)
    d = (0.0, 1.0)
    outs = [torch.zeros(g.n_unknowns, dtype=torch.complex128, device="cuda") for g in geoms]
    ctx.sweep_solve(geoms, ks, d, etas=etas, outs=outs)
    for g, k, e, x in zip(geoms, ks, etas, outs):
        xr = ctx.scattering_solve(g, k, d, eta=e, precision="mixed")
        assert rel(x.cpu().numpy(), xr) < 1e-14


def test_sweep_reports_failing_problem(ctx):
    from bem2d_gb300 import capi
    geoms, ks = small_sweep(3)
    ks = np.array(ks)
    ks[1] = np.nan  # invalid wavenumber in problem 1 (rejected on the host)
    with pytest.raises(capi.Bem2dError) as e:
        ctx.sweep_solve(geoms, ks, (1.0, 0.0))
    assert "problem 1" in str(e.value)
