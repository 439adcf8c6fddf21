"""Element tables: the geometry layout the C-ABI (include/bem2d_gpu.h) takes.

A `Geometry` here is the flat form of bem2d's `Geometry` object
(lib/bem2d_geometry.h:17-75): one row per element (kind + 8 parameters +
index/next/prev, as `Element` stores them, lib/bem2d_element.h:14-70) and a
flat (element, basis) list in `Geometry::FlatMap()` order (element-major,
bases of one element in insertion order, lib/bem2d_geometry.h:48-57).

The builders restate the reference's shape constructors operation by
operation, so that element end points come out bit-identical:
  DiskShapePiecewiseConst   lib/bem2d_shape.cpp:11-34
  Polygon(points, ppw, k, L, sigma)   lib/bem2d_shape.cpp:36-112
  Polygon(points, n)        lib/bem2d_shape.cpp:114-138
  Line(p0, p1, n)           lib/bem2d_shape.cpp:217-233
plus explicit AnalyticCurveElement lists (lib/bem2d_element.h:96-116) with
equispaced parameters.  Arc-length partitions (AnalyticCurve, which needs
GSL's ODE solver) are not reproduced here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# element kinds (match BEM2D_ELEM_* in include/bem2d_gpu.h)
SEGMENT, CIRCLE, TREFOIL, KITE, ELLIPSE, ELLIPSEARC, INVELLIPSE = range(7)
CURVE_NAMES = {CIRCLE: "circle", TREFOIL: "trefoil", KITE: "kite",
               ELLIPSE: "ellipse", ELLIPSEARC: "ellipsearc",
               INVELLIPSE: "invellipse"}
# basis kinds (match BEM2D_BASIS_*)
POLY, LIN = 0, 1
# sentinel for an unset next/prev link
NO_LINK = -1

PI = 3.14159265358979323846


@dataclass
class Geometry:
    kind: list = field(default_factory=list)
    param: list = field(default_factory=list)
    index: list = field(default_factory=list)
    next: list = field(default_factory=list)
    prev: list = field(default_factory=list)
    bases: list = field(default_factory=list)   # (kind, param) added to all elements
    extra: list = field(default_factory=list)   # (element, kind, param) single-element bases

    # -- element construction ------------------------------------------------
    def add_segment(self, p1, p2, idx):
        self.kind.append(SEGMENT)
        self.param.append([p1[0], p1[1], p2[0], p2[1], 0.0, 0.0, 0.0, 0.0])
        self.index.append(idx)
        self.next.append(NO_LINK)
        self.prev.append(NO_LINK)

    def add_curve(self, kind, t1, t2, cparams, idx):
        c = list(cparams) + [0.0] * (4 - len(cparams))
        self.kind.append(kind)
        self.param.append([t1, t2, c[0], c[1], c[2], c[3], 0.0, 0.0])
        self.index.append(idx)
        self.next.append(NO_LINK)
        self.prev.append(NO_LINK)

    def link_closed(self):
        """next/prev as the shape builders set them for a closed chain."""
        n = len(self.kind)
        for i in range(n):
            self.next[i] = (i + 1) % n
            self.prev[i] = (i - 1) % n
        return self

    # -- bases ---------------------------------------------------------------
    def add_basis(self, kind, param):
        """Geometry::AddBasis(pBasis): one basis on every element."""
        self.bases.append((kind, float(param)))
        return self

    def add_poly_basis(self, degree):
        """PolBasis::AddBasis(degree, geom): degrees 0..degree."""
        for d in range(degree + 1):
            self.add_basis(POLY, d)
        return self

    def add_lin_basis(self):
        """LinBasis::AddBasis(geom): LinBasis(1) then LinBasis(-1)."""
        self.add_basis(LIN, 1)
        self.add_basis(LIN, -1)
        return self

    # -- flat tables ---------------------------------------------------------
    @property
    def n_elem(self):
        return len(self.kind)

    def flat(self):
        """Flat (element, basis) map in Geometry::FlatMap() order."""
        ne = self.n_elem
        per = [[] for _ in range(ne)]
        key = 0
        # global insertion keys decide the order inside one element's map
        for (bk, bp) in self.bases:
            for e in range(ne):
                per[e].append((key, bk, bp))
                key += 1
        for (e, bk, bp) in self.extra:
            per[e].append((key, bk, bp))
            key += 1
        ue, uk, up = [], [], []
        for e in range(ne):
            for (_, bk, bp) in sorted(per[e]):
                ue.append(e)
                uk.append(bk)
                up.append(bp)
        return (np.asarray(ue, np.int32), np.asarray(uk, np.int32),
                np.asarray(up, np.float64))

    def arrays(self):
        """Contiguous arrays in the C-ABI layout."""
        ue, uk, up = self.flat()
        return dict(
            kind=np.ascontiguousarray(self.kind, np.int32),
            param=np.ascontiguousarray(self.param, np.float64).reshape(-1, 8),
            index=np.ascontiguousarray(self.index, np.int64),
            next=np.ascontiguousarray(self.next, np.int64),
            prev=np.ascontiguousarray(self.prev, np.int64),
            unk_elem=ue, unk_kind=uk, unk_param=up)

    @property
    def n_unknowns(self):
        return len(self.flat()[0])

    def to_refspec(self, quad=(3, 5, 0.15)):
        """Case lines for oracle/ref_dump (the reference run on this table)."""
        lines = ["quad %d %d %.17g" % quad]
        for i in range(self.n_elem):
            p = self.param[i]
            lk = (self.index[i], self.next[i], self.prev[i])
            if self.kind[i] == SEGMENT:
                lines.append("seg %.17g %.17g %.17g %.17g %d %d %d"
                             % (p[0], p[1], p[2], p[3], *lk))
            else:
                lines.append("curve %s %.17g %.17g %.17g %.17g %.17g %.17g %d %d %d"
                             % (CURVE_NAMES[self.kind[i]], p[0], p[1], p[2],
                                p[3], p[4], p[5], *lk))
        if self.extra:
            raise ValueError("single-element bases are not expressible in a refspec")
        for (bk, bp) in self.bases:
            lines.append("basis %s %.17g" % ("poly" if bk == POLY else "lin", bp))
        return lines


# ---- point arithmetic with the reference's rounding order ------------------
def _add(p, q):
    return (p[0] + q[0], p[1] + q[1])


def _sub(p, q):
    return (p[0] - q[0], p[1] - q[1])


def _scale(t, p):
    return (t * p[0], t * p[1])


def _length(p):
    return math.sqrt(p[0] * p[0] + p[1] * p[1])


# ---- shape builders ---------------------------------------------------------
def disk_chords(n, radius=1.0):
    """DiskShapePiecewiseConst(n, radius): n chords of the circle."""
    g = Geometry()
    angle = 2 * PI / n
    pts = [(radius * math.cos(i * angle), radius * math.sin(i * angle)) for i in range(n)]
    for i in range(n):
        g.add_segment(pts[i], pts[(i + 1) % n], i)
    return g.link_closed()


def polygon_uniform(points, n):
    """Polygon(points, n): n equal elements per side."""
    g = Geometry()
    p = list(points) + [points[0]]
    for i in range(len(points)):
        direction = _sub(p[i + 1], p[i])
        for j in range(n):
            p1 = _add(p[i], _scale((1.0 * j) / n, direction))
            p2 = _add(p[i], _scale((1.0 * (j + 1)) / n, direction))
            g.add_segment(p1, p2, n * i + j)
    return g.link_closed()


def _graded_side(g, p0, p1, n, L, sigma, count):
    """One side of Polygon(points, ppw, k, L, sigma) with n coarse cells."""
    direction = _sub(p1, p0)
    if L == 0:
        g.add_segment(p0, _add(p0, _scale(1.0 / n, direction)), count)
        count += 1
    else:
        tsigma = 1.0
        for _ in range(L):
            tsigma = tsigma * sigma
        g.add_segment(p0, _add(p0, _scale(tsigma / n, direction)), count)
        count += 1
        for _ in range(L):
            q1 = _add(p0, _scale(tsigma / n, direction))
            tsigma = tsigma / sigma
            q2 = _add(p0, _scale(tsigma / n, direction))
            g.add_segment(q1, q2, count)
            count += 1
    for j in range(1, n - 1):
        q1 = _add(p0, _scale((1.0 * j) / n, direction))
        q2 = _add(p0, _scale((1.0 * (j + 1)) / n, direction))
        g.add_segment(q1, q2, count)
        count += 1
    if L == 0:
        g.add_segment(_add(p0, _scale((1.0 * (n - 1)) / n, direction)), p1, count)
        count += 1
    else:
        tsigma = 1.0
        base = _scale((1.0 * (n - 1)) / n, direction)
        for _ in range(L):
            q1 = _add(_add(p0, base), _scale((1 - tsigma) / n, direction))
            tsigma *= sigma
            q2 = _add(_add(p0, base), _scale((1 - tsigma) / n, direction))
            g.add_segment(q1, q2, count)
            count += 1
        q1 = _add(_add(p0, base), _scale((1 - tsigma) / n, direction))
        g.add_segment(q1, p1, count)
        count += 1
    return count


def polygon_graded(points, ppw, k, L=0, sigma=0.15):
    """Polygon(points, ppw, k, L, sigma): n = max(150, ceil(ppw k |side| / 2pi))."""
    ns = []
    p = list(points) + [points[0]]
    for i in range(len(points)):
        direction = _sub(p[i + 1], p[i])
        n = int(math.ceil(ppw * float(k) * _length(direction) / 2.0 / PI))
        ns.append(max(150, n))
    return polygon_graded_n(points, ns, L, sigma)


def polygon_graded_n(points, ns, L=0, sigma=0.15):
    """The graded Polygon rule with an explicit coarse-cell count per side."""
    g = Geometry()
    p = list(points) + [points[0]]
    count = 0
    for i in range(len(points)):
        count = _graded_side(g, p[i], p[i + 1], ns[i], L, sigma, count)
    return g.link_closed()


def line_uniform(p0, p1, n):
    """Line(p0, p1, n): open chain; first prev / last next stay unset."""
    g = Geometry()
    direction = _sub(p1, p0)
    for j in range(n):
        q1 = _add(p0, _scale((1.0 * j) / n, direction))
        q2 = _add(p0, _scale((1.0 * (j + 1)) / n, direction))
        g.add_segment(q1, q2, j)
    for i in range(n):
        g.next[i] = i + 1 if i + 1 < n else NO_LINK
        g.prev[i] = i - 1 if i >= 1 else NO_LINK
    return g


def curve_equispaced(kind, n, cparams=(), closed=True):
    """n AnalyticCurveElement(i/n, (i+1)/n) on one curve."""
    g = Geometry()
    for i in range(n):
        g.add_curve(kind, i / n, (i + 1) / n, cparams, i)
    if closed:
        g.link_closed()
    else:
        for i in range(n):
            g.next[i] = i + 1 if i + 1 < n else NO_LINK
            g.prev[i] = i - 1 if i >= 1 else NO_LINK
    return g


def merge(geoms):
    """Geometry(vector<pGeometry>): concatenate and relink cyclically
    (lib/bem2d_geometry.cpp:22-64)."""
    g = Geometry()
    for h in geoms:
        for i in range(h.n_elem):
            g.kind.append(h.kind[i])
            g.param.append(list(h.param[i]))
            g.index.append(0)
            g.next.append(0)
            g.prev.append(0)
    n = g.n_elem
    for i in range(n):
        g.index[i] = i
        g.next[i] = (i + 1) % n
        g.prev[i] = (i - 1) % n
    return g


# ---- the benchmark geometries ----------------------------------------------
def kite(n):
    """Kite curve x(t) = (cos t + 0.65 cos 2t - 0.65, 1.5 sin t), n elements
    equispaced in t."""
    return curve_equispaced(KITE, n)


def ellipse_arc_closed(n, a=2.0, b=1.0):
    """EllipseArc(a, b, 0, 2pi) as a closed curve with n equispaced elements."""
    return curve_equispaced(ELLIPSEARC, n, (a, b, 0.0, 2 * PI))


ELLIPSE21_PERIMETER = 9.688448220547675  # perimeter of the (2,1) ellipse


def sweep_sizes(n_k=256, k_lo=20.0, k_hi=200.0):
    """Wavenumbers and unknown counts of the ellipse sweep:
    N_k = ceil(10 k P / 2pi) with P the (2,1) ellipse perimeter."""
    ks = np.linspace(k_lo, k_hi, n_k)
    ns = [int(math.ceil(10 * k * ELLIPSE21_PERIMETER / (2 * PI))) for k in ks]
    return ks, ns


def lshape(n_unit=4072, L=8, sigma=0.15):
    """L-shaped domain (unit square minus [0.5,1]^2), graded corners:
    n_unit coarse cells per unit length."""
    pts = [(0, 0), (1, 0), (1, .5), (.5, .5), (.5, 1), (0, 1)]
    lens = [1, .5, .5, .5, .5, 1]
    return polygon_graded_n(pts, [int(round(n_unit * s)) for s in lens], L, sigma)


def graded_square(n_side=2032, L=8, sigma=0.15):
    """Unit square with geometric corner grading: n_side coarse cells per side."""
    pts = [(0, 0), (1, 0), (1, 1), (0, 1)]
    return polygon_graded_n(pts, [n_side] * 4, L, sigma)
