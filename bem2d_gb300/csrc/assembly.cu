// Galerkin assembly kernels for sm_103a (FP64 path).
//
//  node_table_kernel  per (unknown, Gauss node): Map, Normal, |J| w phi
//  far_fp64_kernel    one CTA per 32 x 32 tile of (test, trial) unknowns;
//                     the tile's node data staged in shared memory; tensor
//                     Gauss rule (Integrate<kernel,Gauss2D>,
//                     lib/bem2d_quadrature.h:37-65, selected for non-adjacent
//                     elements at :283-287); coalesced column-major stores
//  near_fp64_kernel   one warp per self/adjacent pair: graded rules
//                     (IntegrateIdent :67-109 with AdaptedGauss1; Integrate
//                     with AdaptedGauss3 / AdaptedGauss2 for next / prev,
//                     :271-282), fused  alpha*K + beta*M  epilogue
//  ident_kernel       EvalIdent (lib/bem2d_quadrature.cpp:79-127)
//  rhs_kernel         DotProdBasFuns (lib/bem2d_quadrature.h:111-156)
#include "common.cuh"
#include "ff.cuh"

namespace bem2d_gpu {

// ---------------------------------------------------------------------------
// One thread per unknown: Map, Normal and |J| w phi at each Gauss node (FP64
// table); optionally the float-float table relative to the element centre
// Map(1/2).
__global__ void node_table_kernel(DevGeom g, DevRules r, NodeTable t, NodeTableFF tf,
                                  int want_ff) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= g.n_unk) return;
  const int e = g.unk_elem[u];
  const double* prm = g.param + 8 * (size_t)e;
  const ElemPt mid = elem_eval(g.kind[e], prm, 0.5);
  float rad = 0.0f;
  for (int q = 0; q < r.ng; ++q) {
    const size_t idx = (size_t)u * r.ng + q;
    const double tq = r.gx[q];
    const ElemPt p = elem_eval(g.kind[e], prm, tq);
    double nx, ny;
    elem_normal(p, &nx, &ny);
    const double w = elem_jac(p) * r.gw[q] * basis_eval(g.unk_kind[u], g.unk_param[u], tq);
    t.x[idx] = p.mx;
    t.y[idx] = p.my;
    t.nx[idx] = nx;
    t.ny[idx] = ny;
    t.w[idx] = w;
    if (want_ff) {
      const double ox = p.mx - mid.mx, oy = p.my - mid.my;
      const ff fox = ff_from_double(ox), foy = ff_from_double(oy);
      const ff fnx = ff_from_double(nx), fny = ff_from_double(ny), fw = ff_from_double(w);
      tf.ox[idx] = make_float2(fox.hi, fox.lo);
      tf.oy[idx] = make_float2(foy.hi, foy.lo);
      tf.nx[idx] = make_float2(fnx.hi, fnx.lo);
      tf.ny[idx] = make_float2(fny.hi, fny.lo);
      tf.w[idx] = make_float2(fw.hi, fw.lo);
      rad = fmaxf(rad, (float)sqrt(ox * ox + oy * oy));
    }
  }
  if (want_ff) {
    tf.c[u] = make_double2(mid.mx, mid.my);
    tf.rad[u] = rad * (1.0f + 1e-6f);
  }
}

void launch_node_table(const DevGeom& g, const DevRules& r, NodeTable t,
                       const NodeTableFF* tf, cudaStream_t s) {
  NodeTableFF z{};
  node_table_kernel<<<(g.n_unk + 127) / 128, 128, 0, s>>>(g, r, t, tf ? *tf : z, tf ? 1 : 0);
}

// ---------------------------------------------------------------------------
// Far field.  Tile: 32 test unknowns (rows, one per lane) x 32 trial unknowns
// (columns, 4 per warp).  Shared memory holds, per node q and tile row /
// column: x, y, nx, ny, w  ([field][q][32]) plus the element links.
constexpr int kTile = 32;
constexpr int kFarThreads = 256;

template <int KERNEL, int NG>
__global__ void __launch_bounds__(kFarThreads)
far_fp64_kernel(DevGeom g, NodeTable t, int ng_rt, double k, double eta,
                double alpha, double2* __restrict__ out, long long ld) {
  const int ng = NG > 0 ? NG : ng_rt;
  extern __shared__ double smem[];
  double* rs = smem;                     // rows: 5 * ng * 32
  double* cs = smem + 5 * ng * kTile;    // cols: 5 * ng * 32
  long long* links = reinterpret_cast<long long*>(cs + 5 * ng * kTile);
  long long* r_idx = links;              // [32]
  long long* r_next = links + kTile;
  long long* r_prev = links + 2 * kTile;
  long long* c_idx = links + 3 * kTile;

  const int row0 = blockIdx.x * kTile, col0 = blockIdx.y * kTile;
  const int n = g.n_unk;
  // stage node data
  for (int v = threadIdx.x; v < ng * kTile; v += blockDim.x) {
    const int q = v / kTile, l = v - q * kTile;
    const int ur = min(row0 + l, n - 1), uc = min(col0 + l, n - 1);
    const size_t ir = (size_t)ur * ng + q, ic = (size_t)uc * ng + q;
    const int o = q * kTile + l;
    rs[0 * ng * kTile + o] = t.x[ir];
    rs[1 * ng * kTile + o] = t.y[ir];
    rs[2 * ng * kTile + o] = t.nx[ir];
    rs[3 * ng * kTile + o] = t.ny[ir];
    rs[4 * ng * kTile + o] = t.w[ir];
    cs[0 * ng * kTile + o] = t.x[ic];
    cs[1 * ng * kTile + o] = t.y[ic];
    cs[2 * ng * kTile + o] = t.nx[ic];
    cs[3 * ng * kTile + o] = t.ny[ic];
    cs[4 * ng * kTile + o] = t.w[ic];
  }
  if (threadIdx.x < kTile) {
    const int l = threadIdx.x;
    const int er = g.unk_elem[min(row0 + l, n - 1)];
    const int ec = g.unk_elem[min(col0 + l, n - 1)];
    r_idx[l] = g.index[er];
    r_next[l] = g.next[er];
    r_prev[l] = g.prev[er];
    c_idx[l] = g.index[ec];
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = row0 + lane;
  const double kq = 0.25 * k, eq = 0.25 * eta;
  const long long ri = r_idx[lane], rn = r_next[lane], rp = r_prev[lane];
  const int SZ = ng * kTile;

#pragma unroll 1
  for (int cc = warp; cc < kTile; cc += kFarThreads / 32) {
    const int col = col0 + cc;
    const long long ci = c_idx[cc];
    const bool near = (ri == ci) || (rn == ci) || (rp == ci);
    if (row >= n || col >= n || near) continue;
    double acc_re = 0.0, acc_im = 0.0;
#pragma unroll 1
    for (int q1 = 0; q1 < ng; ++q1) {
      const int o1 = q1 * kTile + lane;
      const double x1 = rs[o1], y1 = rs[SZ + o1], n1x = rs[2 * SZ + o1],
                   n1y = rs[3 * SZ + o1], w1 = rs[4 * SZ + o1];
#pragma unroll
      for (int q2 = 0; q2 < ng; ++q2) {  // fully unrolled when NG > 0
        const int o2 = q2 * kTile + cc;
        double re, im;
        kernel_d<KERNEL>(k, kq, eq, x1, y1, cs[o2], cs[SZ + o2], n1x, n1y,
                         cs[2 * SZ + o2], cs[3 * SZ + o2], &re, &im);
        const double ww = w1 * cs[4 * SZ + o2];
        acc_re = fma(re, ww, acc_re);
        acc_im = fma(im, ww, acc_im);
      }
    }
    out[(size_t)col * ld + row] = make_double2(alpha * acc_re, alpha * acc_im);
  }
}

template <int KERNEL>
static void launch_far_k(const DevGeom& g, const NodeTable& t, int ng, double k,
                         double eta, double alpha, double2* out, long long ld,
                         cudaStream_t s) {
  const size_t smem = sizeof(double) * 10 * ng * kTile + sizeof(long long) * 4 * kTile;
  dim3 grid((g.n_unk + kTile - 1) / kTile, (g.n_unk + kTile - 1) / kTile);
  if (ng == 5) {
    far_fp64_kernel<KERNEL, 5><<<grid, kFarThreads, smem, s>>>(g, t, ng, k, eta, alpha, out, ld);
  } else {
    auto fn = far_fp64_kernel<KERNEL, 0>;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    fn<<<grid, kFarThreads, smem, s>>>(g, t, ng, k, eta, alpha, out, ld);
  }
}

void launch_far_fp64(const DevGeom& g, const NodeTable& t, int ng, int kernel,
                     double k, double eta, double alpha, double2* out,
                     long long ld, cudaStream_t s) {
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      launch_far_k<BEM2D_KERNEL_SINGLE>(g, t, ng, k, eta, alpha, out, ld, s);
      break;
    case BEM2D_KERNEL_DOUBLE:
      launch_far_k<BEM2D_KERNEL_DOUBLE>(g, t, ng, k, eta, alpha, out, ld, s);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      launch_far_k<BEM2D_KERNEL_CONJDOUBLE>(g, t, ng, k, eta, alpha, out, ld, s);
      break;
    default:
      launch_far_k<BEM2D_KERNEL_COMBINED>(g, t, ng, k, eta, alpha, out, ld, s);
  }
}

// ---------------------------------------------------------------------------
// Near field: one warp per (test, trial) pair of adjacent or identical
// elements.  Lanes stride over the rule's points; a shuffle tree reduces.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int KERNEL>
__device__ __forceinline__ void pair_point(const DevGeom& g, int ui, int uj,
                                           int e1, int e2, double s, double t,
                                           double k, double kq, double eq,
                                           double* re, double* im) {
  const double* p1 = g.param + 8 * (size_t)e1;
  const double* p2 = g.param + 8 * (size_t)e2;
  const ElemPt a = elem_eval(g.kind[e1], p1, s);
  const ElemPt b = elem_eval(g.kind[e2], p2, t);
  double n1x, n1y, n2x, n2y;
  elem_normal(a, &n1x, &n1y);
  elem_normal(b, &n2x, &n2y);
  double kr, ki;
  kernel_d<KERNEL>(k, kq, eq, a.mx, a.my, b.mx, b.my, n1x, n1y, n2x, n2y, &kr, &ki);
  const double f = basis_eval(g.unk_kind[ui], g.unk_param[ui], s) *
                   basis_eval(g.unk_kind[uj], g.unk_param[uj], t) *
                   elem_jac(a) * elem_jac(b);
  *re = kr * f;
  *im = ki * f;
}

// mass-matrix entry of a same-index pair (EvalIdent's inner loop)
__device__ __forceinline__ double mass_entry(const DevGeom& g, const DevRules& r,
                                             int ui, int uj) {
  const int ej = g.unk_elem[uj];
  double m = 0.0;
  for (int q = 0; q < r.ng; ++q) {
    const double tq = r.gx[q];
    const ElemPt p = elem_eval(g.kind[ej], g.param + 8 * (size_t)ej, tq);
    m += elem_jac(p) * basis_eval(g.unk_kind[ui], g.unk_param[ui], tq) *
         basis_eval(g.unk_kind[uj], g.unk_param[uj], tq) * r.gw[q];
  }
  return m;
}

template <int KERNEL>
__global__ void __launch_bounds__(256)
near_fp64_kernel(DevGeom g, DevRules r, const NearPair* __restrict__ pairs,
                 int npairs, double k, double eta, double alpha, double beta,
                 double2* __restrict__ out, long long ld, float2* __restrict__ out32,
                 long long ld32) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= npairs) return;
  const NearPair pr = pairs[wid];
  const int e1 = g.unk_elem[pr.i], e2 = g.unk_elem[pr.j];
  const double kq = 0.25 * k, eq = 0.25 * eta;
  double acc_re = 0.0, acc_im = 0.0;
  if (pr.rule == RULE_SELF) {
    // IntegrateIdent: Duffy split, points (x, (1-y)x) and (1-x, 1-x+yx),
    // both weighted by x * w.
    for (int p = lane; p < r.n1; p += 32) {
      const double x = r.r1[3 * p], y = r.r1[3 * p + 1], w = r.r1[3 * p + 2];
      double re, im;
      pair_point<KERNEL>(g, pr.i, pr.j, e1, e2, x, (1 - y) * x, k, kq, eq, &re, &im);
      acc_re = fma(re, x * w, acc_re);
      acc_im = fma(im, x * w, acc_im);
      pair_point<KERNEL>(g, pr.i, pr.j, e1, e2, 1 - x, 1 - x + y * x, k, kq, eq, &re, &im);
      acc_re = fma(re, x * w, acc_re);
      acc_im = fma(im, x * w, acc_im);
    }
  } else if (pr.rule == RULE_G3_PAIR) {
    // (i, j) with AdaptedGauss3 at (x, y), (j, i) with its mirror
    // AdaptedGauss2 at (y, x): the same point pairs, one evaluation each
    double acc2_re = 0.0, acc2_im = 0.0;
    for (int p = lane; p < r.n3; p += 32) {
      const double x = r.r3[3 * p], y = r.r3[3 * p + 1], w = r.r3[3 * p + 2];
      const ElemPt a = elem_eval(g.kind[e1], g.param + 8 * (size_t)e1, x);
      const ElemPt b = elem_eval(g.kind[e2], g.param + 8 * (size_t)e2, y);
      double n1x, n1y, n2x, n2y;
      elem_normal(a, &n1x, &n1y);
      elem_normal(b, &n2x, &n2y);
      double r1, i1, r2, i2;
      kernel_d_pair<KERNEL>(k, kq, eq, a.mx, a.my, b.mx, b.my, n1x, n1y, n2x, n2y, &r1, &i1,
                            &r2, &i2);
      const double f = basis_eval(g.unk_kind[pr.i], g.unk_param[pr.i], x) *
                       basis_eval(g.unk_kind[pr.j], g.unk_param[pr.j], y) * elem_jac(a) *
                       elem_jac(b) * w;
      acc_re = fma(r1, f, acc_re);
      acc_im = fma(i1, f, acc_im);
      acc2_re = fma(r2, f, acc2_re);
      acc2_im = fma(i2, f, acc2_im);
    }
    acc2_re = warp_sum(acc2_re);
    acc2_im = warp_sum(acc2_im);
    if (lane == 0) {
      const double re = alpha * acc2_re, im = alpha * acc2_im;
      out[(size_t)pr.i * ld + pr.j] = make_double2(re, im);
      if (out32) out32[(size_t)pr.i * ld32 + pr.j] = make_float2((float)re, (float)im);
    }
  } else {
    const double* rule = pr.rule == RULE_G2 ? r.r2 : r.r3;
    const int np = pr.rule == RULE_G2 ? r.n2 : r.n3;
    for (int p = lane; p < np; p += 32) {
      const double x = rule[3 * p], y = rule[3 * p + 1], w = rule[3 * p + 2];
      double re, im;
      pair_point<KERNEL>(g, pr.i, pr.j, e1, e2, x, y, k, kq, eq, &re, &im);
      acc_re = fma(re, w, acc_re);
      acc_im = fma(im, w, acc_im);
    }
  }
  acc_re = warp_sum(acc_re);
  acc_im = warp_sum(acc_im);
  if (lane == 0) {
    double re = alpha * acc_re, im = alpha * acc_im;
    if (pr.same && beta != 0.0) re = fma(beta, mass_entry(g, r, pr.i, pr.j), re);
    out[(size_t)pr.j * ld + pr.i] = make_double2(re, im);
    if (out32) out32[(size_t)pr.j * ld32 + pr.i] = make_float2((float)re, (float)im);
  }
}

void launch_near_fp64(const DevGeom& g, const DevRules& r, const NearPair* pairs,
                      int npairs, int kernel, double k, double eta, double alpha,
                      double beta, double2* out, long long ld, cudaStream_t s,
                      float2* out32, long long ld32) {
  if (npairs == 0) return;
  const int blocks = (npairs * 32 + 255) / 256;
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      near_fp64_kernel<BEM2D_KERNEL_SINGLE><<<blocks, 256, 0, s>>>(g, r, pairs, npairs, k, eta, alpha, beta, out, ld, out32, ld32);
      break;
    case BEM2D_KERNEL_DOUBLE:
      near_fp64_kernel<BEM2D_KERNEL_DOUBLE><<<blocks, 256, 0, s>>>(g, r, pairs, npairs, k, eta, alpha, beta, out, ld, out32, ld32);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      near_fp64_kernel<BEM2D_KERNEL_CONJDOUBLE><<<blocks, 256, 0, s>>>(g, r, pairs, npairs, k, eta, alpha, beta, out, ld, out32, ld32);
      break;
    default:
      near_fp64_kernel<BEM2D_KERNEL_COMBINED><<<blocks, 256, 0, s>>>(g, r, pairs, npairs, k, eta, alpha, beta, out, ld, out32, ld32);
  }
}

// ---------------------------------------------------------------------------
__global__ void ident_kernel(DevGeom g, DevRules r, const NearPair* __restrict__ pairs,
                             int npairs, double2* __restrict__ out, long long ld) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const NearPair pr = pairs[p];
  if (!pr.same) return;
  out[(size_t)pr.j * ld + pr.i] = make_double2(mass_entry(g, r, pr.i, pr.j), 0.0);
}

void launch_ident(const DevGeom& g, const DevRules& r, const NearPair* pairs,
                  int npairs, double2* out, long long ld, cudaStream_t s) {
  if (npairs == 0) return;
  ident_kernel<<<(npairs + 127) / 128, 128, 0, s>>>(g, r, pairs, npairs, out, ld);
}

// ---------------------------------------------------------------------------
// b_u = scale * sum_q f(x_q) |J| phi_u w_q, f one of the plane-wave
// functionals (lib/bem2d_fun.h:14-93).
__global__ void rhs_kernel(int n, NodeTable t, int ng, int fun, double k,
                           double dx, double dy, double eta, double scale,
                           double2* __restrict__ out) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  double acc_re = 0.0, acc_im = 0.0;
  for (int q = 0; q < ng; ++q) {
    const size_t o = (size_t)u * ng + q;
    const double ph = k * (dx * t.x[o] + dy * t.y[o]);
    double fs, fc;
    sincos(ph, &fs, &fc);
    double vr, vi;
    if (fun == BEM2D_FUN_PLANEWAVE) {
      vr = fc;
      vi = fs;
    } else {
      const double nd = t.nx[o] * dx + t.ny[o] * dy;
      vr = -k * fs * nd;  // i k f (n.d)
      vi = k * fc * nd;
      if (fun == BEM2D_FUN_COMBINEDPLANEWAVE) {  // - i eta f
        vr += eta * fs;
        vi -= eta * fc;
      }
    }
    acc_re = fma(vr, t.w[o], acc_re);
    acc_im = fma(vi, t.w[o], acc_im);
  }
  out[u] = make_double2(scale * acc_re, scale * acc_im);
}

void launch_rhs(const DevGeom& g, const NodeTable& t, int ng, int fun, double k,
                double dx, double dy, double eta, double scale, double2* out,
                cudaStream_t s) {
  rhs_kernel<<<(g.n_unk + 127) / 128, 128, 0, s>>>(g.n_unk, t, ng, fun, k, dx, dy,
                                                   eta, scale, out);
}

// ---------------------------------------------------------------------------
// Potential of a density at points (EvalKernel, lib/bem2d_quadrature.h:184-228):
// out[p] = sum_u c_u sum_q K(x_p, y_uq) W_uq, both normals the source node's.
// One thread per point; unknowns staged through shared memory in chunks.
template <int KERNEL>
__global__ void __launch_bounds__(128)
potential_kernel(int nunk, NodeTable t, int ng, double k, double eta,
                 const double2* __restrict__ coef, int npts, const double* __restrict__ pts,
                 double2* __restrict__ out) {
  __shared__ double sx[128], sy[128], snx[128], sny[128], sw[128];
  __shared__ double2 sc[128];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const double px = p < npts ? pts[2 * p] : 0.0, py = p < npts ? pts[2 * p + 1] : 0.0;
  const double kq = 0.25 * k, eq = 0.25 * eta;
  double ar = 0.0, ai = 0.0;
  const int total = nunk * ng;
  for (int base = 0; base < total; base += 128) {
    const int v = base + threadIdx.x;
    __syncthreads();
    if (v < total) {
      sx[threadIdx.x] = t.x[v];
      sy[threadIdx.x] = t.y[v];
      snx[threadIdx.x] = t.nx[v];
      sny[threadIdx.x] = t.ny[v];
      sw[threadIdx.x] = t.w[v];
      sc[threadIdx.x] = coef[v / ng];
    }
    __syncthreads();
    const int cnt = min(128, total - base);
    if (p < npts) {
      for (int i = 0; i < cnt; ++i) {
        double kr, ki;
        kernel_d<KERNEL>(k, kq, eq, px, py, sx[i], sy[i], snx[i], sny[i], snx[i], sny[i], &kr,
                         &ki);
        // coefficient * kernel * weight
        const double2 c = sc[i];
        const double vr = (c.x * kr - c.y * ki) * sw[i], vi = (c.x * ki + c.y * kr) * sw[i];
        ar += vr;
        ai += vi;
      }
    }
  }
  if (p < npts) out[p] = make_double2(ar, ai);
}

void launch_potential(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                      double eta, const double2* coef, int npts, const double* pts,
                      double2* out, cudaStream_t s) {
  const int blocks = (npts + 127) / 128;
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      potential_kernel<BEM2D_KERNEL_SINGLE><<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, eta, coef, npts, pts, out);
      break;
    case BEM2D_KERNEL_DOUBLE:
      potential_kernel<BEM2D_KERNEL_DOUBLE><<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, eta, coef, npts, pts, out);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      potential_kernel<BEM2D_KERNEL_CONJDOUBLE><<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, eta, coef, npts, pts, out);
      break;
    default:
      potential_kernel<BEM2D_KERNEL_COMBINED><<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, eta, coef, npts, pts, out);
  }
}

}  // namespace bem2d_gpu
