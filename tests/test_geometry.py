"""Element tables for the benchmark configurations (sizes and links)."""
import math

import numpy as np

from bem2d_gb300 import geometry as G


def test_config_sizes():
    assert G.lshape(4072, 8, 0.15).n_elem == 16384
    assert G.graded_square(2032, 8, 0.15).n_elem == 8192
    ks, ns = G.sweep_sizes()
    assert len(ks) == 256 and min(ns) == 309 and max(ns) == 3084
    assert G.kite(2048).n_elem == 2048


def test_graded_polygon_rule():
    # Polygon(points, ppw, k, L, sigma): n = max(150, ceil(ppw k len / 2 pi)) + 2L per side
    g = G.polygon_graded([(0, 0), (1, 0), (1, 1), (0, 1)], 10, 5.0, 3, 0.15)
    assert g.n_elem == 4 * (150 + 6)
    p = np.array(g.param)
    lens = np.hypot(p[:, 2] - p[:, 0], p[:, 3] - p[:, 1])
    assert abs(lens.sum() - 4.0) < 1e-12
    assert abs(lens.min() - 0.15 ** 3 / 150) < 1e-15
    # the chain is closed: each element ends where the next begins
    assert np.allclose(p[:, 2:4], np.roll(p[:, 0:2], -1, axis=0), atol=1e-15)


def test_links_and_flatmap():
    g = G.polygon_uniform([(0, 0), (1, 0), (0, 1)], 4).add_poly_basis(2)
    a = g.arrays()
    assert list(a["next"][:3]) == [1, 2, 3] and a["prev"][0] == 11
    # element-major: (e0,P0),(e0,P1),(e0,P2),(e1,P0),...
    assert list(a["unk_elem"][:6]) == [0, 0, 0, 1, 1, 1]
    assert list(a["unk_param"][:6]) == [0, 1, 2, 0, 1, 2]
    m = G.merge([G.polygon_uniform([(0, 0), (1, 0), (0, 1)], 2),
                 G.polygon_uniform([(2, 0), (3, 0), (2, 1)], 2)])
    assert m.index == list(range(12)) and m.next[11] == 0 and m.prev[0] == 11


def test_open_line_links_unset():
    g = G.line_uniform((0, 0), (1, 0), 5)
    assert g.prev[0] == G.NO_LINK and g.next[4] == G.NO_LINK


def test_ellipse_perimeter():
    from scipy.special import ellipe
    assert abs(4 * 2 * ellipe(1 - 0.25) - G.ELLIPSE21_PERIMETER) < 1e-12
