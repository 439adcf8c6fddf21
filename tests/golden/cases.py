"""Parity cases shared by the golden-vector generator and the tests.

Each case builds an element table with bem2d_gb300.geometry and names the
operations to pin.  The reference library itself (compiled by oracle/Makefile
into oracle/_ref) produced the committed fixtures; see make_golden.py.
"""
from __future__ import annotations

import math

import numpy as np

from bem2d_gb300 import geometry as G

SQUARE = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
LSHAPE = [(0.0, 0.0), (1.0, 0.0), (1.0, 0.5), (0.5, 0.5), (0.5, 1.0), (0.0, 1.0)]
TRIANGLE = [(0.0, 0.0), (1.0, 0.0), (0.3, 0.8)]


def seeded_angle(seed=0):
    """Plane-wave angle drawn U[0, 2pi) from a seeded generator."""
    return float(np.random.default_rng(seed).uniform(0, 2 * math.pi))


def _dir(theta):
    return (math.cos(theta), math.sin(theta))


# trapping domain of the reference's resonance scan (resonances/trapresonance.cpp)
_TA, _TC = 0.31, 1.0
_TL = _TC - _TA
TRAP = [(0.0, 0.0), (-_TC, 0.0), (-_TC, -_TL), (_TL, -_TL), (_TL, 2 * _TC - _TL),
        (-_TC, 2 * _TC - _TL), (-_TC, 2 * _TA), (0.0, 2 * _TA)]


def _two_squares():
    a = G.polygon_uniform([(0, 0), (1, 0), (1, 1), (0, 1)], 6)
    b = G.polygon_uniform([(2, 0), (3, 0), (3, 1), (2, 1)], 6)
    return G.merge([a, b])


# name -> dict(geom=callable, k, direction, eta, quad, full, kernels, extra)
CASES = {
    # unit disk, 160 equal-arc elements, k = 10, d = (1,0)
    "disk160": dict(geom=lambda: G.curve_equispaced(G.CIRCLE, 160).add_poly_basis(0),
                    k=10.0, direction=(1.0, 0.0), eta=10.0, full=True,
                    kernels=("single", "double", "conjdouble"),
                    evalsol=[(-1.5, 0.0), (2.0, 1.0), (0.0, -3.0), (1.2, 0.4)]),
    "diskchords64": dict(geom=lambda: G.disk_chords(64, 1.0).add_poly_basis(0),
                         k=5.0, direction=(1.0, 0.0), eta=5.0, full=True),
    "kite128": dict(geom=lambda: G.kite(128).add_poly_basis(0), k=15.0,
                    direction=_dir(seeded_angle(0)), eta=15.0, full=True,
                    evalsol=[(2.0, 0.0), (-2.5, 1.0), (0.3, 2.2)]),
    "ellipsearc100": dict(geom=lambda: G.ellipse_arc_closed(100).add_poly_basis(0),
                          k=10.0, direction=(0.0, 1.0), eta=10.0, full=True),
    "trefoil48": dict(geom=lambda: G.curve_equispaced(G.TREFOIL, 48).add_poly_basis(0),
                      k=6.0, direction=(0.6, 0.8), eta=3.0, full=True),
    "ellipse48": dict(geom=lambda: G.curve_equispaced(G.ELLIPSE, 48, (2.0,)).add_poly_basis(0),
                      k=4.0, direction=(1.0, 0.0), eta=4.0, full=True),
    "invellipse48": dict(geom=lambda: G.curve_equispaced(G.INVELLIPSE, 48, (0.3,)).add_poly_basis(0),
                         k=7.0, direction=(1.0, 0.0), eta=7.0, full=True),
    # graded polygons (reference Polygon(points, ppw, k, L, sigma) rule)
    "square_graded": dict(geom=lambda: G.polygon_graded(SQUARE, 10, 5.0, 3, 0.15).add_poly_basis(0),
                          k=5.0, direction=_dir(0.3), eta=5.0, full=False),
    "lshape_graded": dict(geom=lambda: G.lshape(40, 8, 0.15).add_poly_basis(0),
                          k=30.0, direction=_dir(seeded_angle(1)), eta=30.0, full=False),
    # other bases
    "square_poly2": dict(geom=lambda: G.polygon_uniform(SQUARE, 8).add_poly_basis(2),
                         k=3.0, direction=(1.0, 0.0), eta=3.0, full=True,
                         kernels=("single", "conjdouble")),
    "triangle_lin": dict(geom=lambda: G.polygon_uniform(TRIANGLE, 10).add_lin_basis(),
                         k=4.0, direction=(0.0, -1.0), eta=4.0, full=True),
    # open chain: first prev / last next unset
    "line_open": dict(geom=lambda: G.line_uniform((0.0, 0.0), (1.0, 0.5), 40).add_poly_basis(0),
                      k=8.0, direction=(1.0, 0.0), eta=8.0, full=True, scattering=False,
                      kernels=("single", "double")),
    # multi-piece geometry relinked by Geometry(vector<pGeometry>)
    "two_squares": dict(geom=lambda: _two_squares().add_poly_basis(0), k=4.0,
                        direction=(1.0, 0.0), eta=4.0, full=True),
    # numerical range / singular values of ChangeBasis(A, Id)
    "square_numrange": dict(geom=lambda: G.polygon_uniform(SQUARE, 16).add_poly_basis(0),
                            k=5.0, direction=(1.0, 0.0), eta=5.0, full=True,
                            numrange=18, singvals=True),
    # complex wavenumbers k + i kim (the reference's AMOS branch); eta real
    "trap_ck": dict(geom=lambda: G.polygon_graded_n(TRAP, [8] * 8, 3, 0.15).add_poly_basis(0),
                    k=6.0, kim=-1.0, direction=(1.0, 0.0), eta=abs(complex(6.0, -1.0)),
                    full=True, kernels=("single", "conjdouble")),
    "disk_absorbing_ck": dict(geom=lambda: G.curve_equispaced(G.CIRCLE, 64).add_poly_basis(0),
                              k=8.0, kim=0.5, direction=(1.0, 0.0), eta=8.0, full=True,
                              kernels=("double",),
                              evalsol=[(-1.5, 0.0), (2.0, 1.0), (0.0, -3.0)]),
    "kite_ck": dict(geom=lambda: G.kite(96).add_poly_basis(0), k=12.0, kim=-3.0,
                    direction=_dir(seeded_angle(2)), eta=12.0, full=True),
    "square_poly2_ck": dict(geom=lambda: G.polygon_uniform(SQUARE, 8).add_poly_basis(2),
                            k=3.0, kim=-0.5, direction=(1.0, 0.0), eta=3.0, full=True,
                            kernels=("single", "conjdouble")),
}

QUAD = (3, 5, 0.15)
