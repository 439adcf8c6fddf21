"""Failure detection on the GPU, in forms that fault and hang nothing.

Where the reference raises LapackError from its LAPACK calls
(lib/bem2d_mathroutines.cpp:262, 346, 348), this library also reports two
failures LAPACK cannot have:

* a bounded device-side wait that gives up (BEM2D_ERR_TIMEOUT): one LU panel
  on the cooperative-grid panel kernel waits for a candidate slot that no
  block posts, with a limit of a few dozen polls; the kernel returns, the
  call reports the timeout, and the same context then solves normally;
* a NaN or infinity in an assembled matrix or right-hand side
  (BEM2D_ERR_NONFINITE): a NaN injected on the host into one element's
  parameters must be reported, not returned as a NaN matrix or solution.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QUAD = (3, 5, 0.15)
TIMEOUT = -6
NONFINITE = -4


@pytest.fixture(scope="module")
def ctx():
    from bem2d_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()


def _system(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A += 2 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return np.asfortranarray(A), b


@pytest.mark.parametrize("polls", [8, 64])
def test_panel_wait_times_out_and_context_survives(ctx, polls):
    rc, msg = ctx.debug_panel_timeout(512, polls)
    assert rc == TIMEOUT, (rc, msg)
    assert "gave up" in msg
    # the context (and the panel kernels) work afterwards: a complex64 LU of
    # order 9000 uses the same cooperative-grid panel kernel
    for n in (300, 9000):
        A, b = _system(n, n)
        x = ctx.solve(A, b, "mixed")
        r = np.linalg.norm(b - A @ x) / (np.linalg.norm(A) * np.linalg.norm(x) +
                                         np.linalg.norm(b))
        assert r < 1e-13, (n, r)


def test_nan_element_is_reported(ctx):
    from bem2d_gb300 import capi
    from bem2d_gb300 import geometry as G
    g = G.kite(128).add_poly_basis(0)
    g.param[17][0] = float("nan")  # t1 of element 17
    for call in (lambda: ctx.discrete_kernel(g, "combined", 15.0, 15.0, QUAD, 2.0, 1.0),
                 lambda: ctx.discrete_kernel_mixed(g, "combined", 15.0, 15.0, QUAD, 2.0, 1.0),
                 lambda: ctx.scattering_solve(g, 15.0, (1.0, 0.0), 15.0, QUAD,
                                              precision="fp64"),
                 lambda: ctx.scattering_solve(g, 15.0, (1.0, 0.0), 15.0, QUAD,
                                              precision="mixed")):
        with pytest.raises(capi.Bem2dError) as e:
            call()
        assert e.value.code == NONFINITE, str(e.value)
        assert "non-finite" in str(e.value)
    # the same context assembles and solves the clean geometry afterwards
    g2 = G.kite(128).add_poly_basis(0)
    x = ctx.scattering_solve(g2, 15.0, (1.0, 0.0), 15.0, QUAD, precision="mixed")
    assert np.all(np.isfinite(x))


def test_nan_element_in_sweep_names_the_problem(ctx):
    """A sweep stops at the first failed problem and reports the failure."""
    from bem2d_gb300 import capi
    from bem2d_gb300 import geometry as G
    gs = [G.ellipse_arc_closed(n).add_poly_basis(0) for n in (200, 240, 280)]
    gs[1].param[3][0] = float("nan")
    with pytest.raises(capi.Bem2dError) as e:
        ctx.sweep_solve(gs, [20.0, 24.0, 28.0], (1.0, 0.0), None, QUAD, "mixed", nworkers=2)
    assert e.value.code == NONFINITE, str(e.value)
