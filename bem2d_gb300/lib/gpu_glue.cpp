// bem2d C++ API (GB300 build): assembly entry points, lowered to the C ABI.
#include "gpu_glue.h"

#include <cstdlib>
#include <string>
#include <typeinfo>
#include <unordered_map>

#include "bem2d_basistypes.h"
#include "bem2d_curvetypes.h"
#include "bem2d_exceptions.h"
#include "bem2d_quadrature.h"
#include "bem2d_soundsoftscattering.h"

namespace bem2d {
namespace detail {

bem2d_ctx* ctx() {
  static bem2d_ctx* c = nullptr;
  if (!c) {
    const char* dev = std::getenv("BEM2D_DEVICE");
    const int rc = bem2d_ctx_create(dev ? std::atoi(dev) : 0, &c);
    if (rc != BEM2D_OK) throw GpuError(rc, "bem2d: no usable CUDA device");
  }
  return c;
}

void check(int rc, const char* what) {
  if (rc == BEM2D_OK) return;
  const std::string msg = std::string(what) + ": " + bem2d_ctx_last_error(ctx());
  if (rc > 0) throw LapackError();
  switch (rc) {
    case BEM2D_ERR_ARG:
      throw ParameterException();
    case BEM2D_ERR_UNSUPPORTED:
      throw UnsupportedError(msg);
    default:
      throw GpuError(rc, msg);
  }
}

bem2d_geometry PackedGeometry::view() const {
  bem2d_geometry g;
  g.n_elem = (int32_t)kind.size();
  g.kind = kind.data();
  g.param = param.data();
  g.index = index.data();
  g.next = next.data();
  g.prev = prev.data();
  g.n_unk = (int32_t)unk_elem.size();
  g.unk_elem = unk_elem.data();
  g.unk_kind = unk_kind.data();
  g.unk_param = unk_param.data();
  return g;
}

static void pack_element(PackedGeometry& p, const Element* e) {
  double prm[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int kind;
  if (const ConstElement* c = dynamic_cast<const ConstElement*>(e)) {
    kind = BEM2D_ELEM_SEGMENT;
    prm[0] = c->p1().x;
    prm[1] = c->p1().y;
    prm[2] = c->p2().x;
    prm[3] = c->p2().y;
  } else if (const AnalyticCurveElement* a = dynamic_cast<const AnalyticCurveElement*>(e)) {
    prm[0] = a->tstart();
    prm[1] = a->tend();
    const Curve* cv = a->curve().get();
    if (dynamic_cast<const Circle*>(cv)) {
      kind = BEM2D_ELEM_CIRCLE;
    } else if (dynamic_cast<const Trefoil*>(cv)) {
      kind = BEM2D_ELEM_TREFOIL;
    } else if (dynamic_cast<const Kite*>(cv)) {
      kind = BEM2D_ELEM_KITE;
    } else if (const Ellipse* el = dynamic_cast<const Ellipse*>(cv)) {
      kind = BEM2D_ELEM_ELLIPSE;
      prm[2] = el->rho();
    } else if (const EllipseArc* ea = dynamic_cast<const EllipseArc*>(cv)) {
      kind = BEM2D_ELEM_ELLIPSEARC;
      prm[2] = ea->a();
      prm[3] = ea->b();
      prm[4] = ea->theta1();
      prm[5] = ea->theta2();
    } else if (const InvEllipse* ie = dynamic_cast<const InvEllipse*>(cv)) {
      kind = BEM2D_ELEM_INVELLIPSE;
      prm[2] = ie->alpha();
    } else {
      throw UnsupportedError(std::string("curve type not evaluated on the GPU: ") + typeid(*cv).name());
    }
  } else {
    throw UnsupportedError(std::string("element type not evaluated on the GPU: ") + typeid(*e).name());
  }
  p.kind.push_back(kind);
  p.param.insert(p.param.end(), prm, prm + 8);
  p.index.push_back((int64_t)e->index());
  p.next.push_back((int64_t)e->next());
  p.prev.push_back((int64_t)e->prev());
}

PackedGeometry Pack(const Geometry::flat_basis_map& fm) {
  PackedGeometry p;
  std::unordered_map<const Element*, int> pos;
  for (const auto& eb : fm) {
    const Element* e = eb.first.get();
    auto it = pos.find(e);
    int ei;
    if (it == pos.end()) {
      ei = (int)p.kind.size();
      pos[e] = ei;
      pack_element(p, e);
    } else {
      ei = it->second;
    }
    p.unk_elem.push_back(ei);
    const Basis* b = eb.second.get();
    if (const PolBasis* pb = dynamic_cast<const PolBasis*>(b)) {
      p.unk_kind.push_back(BEM2D_BASIS_POLY);
      p.unk_param.push_back(pb->degree());
    } else if (const LinBasis* lb = dynamic_cast<const LinBasis*>(b)) {
      p.unk_kind.push_back(BEM2D_BASIS_LIN);
      p.unk_param.push_back(lb->sign());
    } else {
      throw UnsupportedError(std::string("basis type not evaluated on the GPU: ") + typeid(*b).name());
    }
  }
  return p;
}

PackedGeometry Pack(const Geometry& g) { return Pack(*g.FlatMap()); }

static bem2d_quad quad_of(const QuadOption& q) {
  bem2d_quad r;
  r.L = q.L;
  r.N = q.N;
  r.sigma = q.sigma;
  return r;
}

static pMatrix assemble(const Geometry& geom, QuadOption opts, int kernel, freqtype k,
                        double eta, double alpha, double beta) {
  PackedGeometry p = Pack(geom);
  const bem2d_geometry g = p.view();
  const bem2d_quad q = quad_of(opts);
  const int n = g.n_unk;
  pMatrix m(new Matrix(n));
  check(bem2d_discrete_kernel(ctx(), &g, &q, kernel, k.re, k.im, eta, alpha, beta, &(*m->data)[0], n),
        "DiscreteKernel");
  return m;
}

pMatrix CombinedSystemMatrix(const Geometry& g, QuadOption q, freqtype k, double eta) {
  return assemble(g, q, BEM2D_KERNEL_COMBINED, k, eta, 2.0, 1.0);
}

static pMatrix rhs(const Geometry& geom, QuadOption opts, int fun, freqtype k, Point d, double eta) {
  PackedGeometry p = Pack(geom);
  const bem2d_geometry g = p.view();
  const bem2d_quad q = quad_of(opts);
  pMatrix m(new Matrix(g.n_unk, 1));
  check(bem2d_dot_prod_basfuns(ctx(), &g, &q, fun, k.re, k.im, d.x, d.y, eta, 1.0, &(*m->data)[0]),
        "DotProdBasFuns");
  return m;
}

void EvalKernelGpu(const Geometry::flat_basis_map& basfuns, const std::vector<Point>& points,
                   cvector& vals, const complex* alpha, int kernel, freqtype k, double eta, int N) {
  if (points.size() != vals.size()) throw SizeError();
  if (points.empty()) return;
  PackedGeometry p = Pack(basfuns);
  const bem2d_geometry g = p.view();
  bem2d_quad q;
  q.L = 1;
  q.N = N;
  q.sigma = 0.15;
  std::vector<double> xy(2 * points.size());
  for (std::size_t i = 0; i < points.size(); ++i) {
    xy[2 * i] = points[i].x;
    xy[2 * i + 1] = points[i].y;
  }
  cvector out(points.size());
  check(bem2d_eval_kernel(ctx(), &g, &q, kernel, k.re, k.im, eta, alpha, (int)points.size(),
                          xy.data(), &out[0]),
        "EvalKernel");
  for (std::size_t i = 0; i < points.size(); ++i) vals[i] += out[i];
}

}  // namespace detail

pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, SingleLayer g) {
  return detail::assemble(geom, opts, BEM2D_KERNEL_SINGLE, g.k(), 0.0, 1.0, 0.0);
}
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, DoubleLayer g) {
  return detail::assemble(geom, opts, BEM2D_KERNEL_DOUBLE, g.k(), 0.0, 1.0, 0.0);
}
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, ConjDoubleLayer g) {
  return detail::assemble(geom, opts, BEM2D_KERNEL_CONJDOUBLE, g.k(), 0.0, 1.0, 0.0);
}
pMatrix DiscreteKernel(const Geometry& geom, QuadOption opts, CombinedSingleConjDouble g) {
  return detail::assemble(geom, opts, BEM2D_KERNEL_COMBINED, g.getk(), g.eta(), 1.0, 0.0);
}

pMatrix EvalIdent(const Geometry& geom, QuadOption opts) {
  detail::PackedGeometry p = detail::Pack(geom);
  const bem2d_geometry g = p.view();
  const bem2d_quad q = detail::quad_of(opts);
  const int n = g.n_unk;
  pMatrix m(new Matrix(n));
  detail::check(bem2d_eval_ident(detail::ctx(), &g, &q, &(*m->data)[0], n), "EvalIdent");
  return m;
}

pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, PlaneWave fun) {
  return detail::rhs(geom, ops, BEM2D_FUN_PLANEWAVE, fun.k(), fun.direction(), 0.0);
}
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, NormalPlaneWave fun) {
  return detail::rhs(geom, ops, BEM2D_FUN_NORMALPLANEWAVE, fun.k(), fun.direction(), 0.0);
}
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, CombinedPlaneWave fun) {
  return detail::rhs(geom, ops, BEM2D_FUN_COMBINEDPLANEWAVE, fun.k(), fun.direction(), fun.eta());
}
pMatrix DotProdBasFuns(const Geometry& geom, QuadOption ops, IdFun) {
  // exp(i 0 d.x) = 1
  freqtype k0 = {0, 0};
  return detail::rhs(geom, ops, BEM2D_FUN_PLANEWAVE, k0, Point(1, 0), 0.0);
}

}  // namespace bem2d
