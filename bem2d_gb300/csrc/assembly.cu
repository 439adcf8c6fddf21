// Galerkin assembly kernels for sm_103a (FP64 path).
//
//  node_table_kernel  per (unknown, Gauss node): Map, Normal, |J| w phi
//  far_fp64_kernel    one CTA per 32 x 32 tile of (test, trial) unknowns;
//                     the tile's node data staged in shared memory; tensor
//                     Gauss rule (Integrate<kernel,Gauss2D>,
//                     lib/bem2d_quadrature.h:37-65, selected for non-adjacent
//                     elements at :283-287); coalesced column-major stores
//  near_kernel        one warp per self/adjacent pair: graded rules
//                     (IntegrateIdent :67-109 with AdaptedGauss1; Integrate
//                     with AdaptedGauss3 / AdaptedGauss2 for next / prev,
//                     :271-282), fused  alpha*K + beta*M  epilogue; element
//                     geometry tabulated per warp at the rules' distinct
//                     coordinates; the mixed-precision variant evaluates
//                     the Bessel functions in float-float
//  ident_kernel       EvalIdent (lib/bem2d_quadrature.cpp:79-127)
//  rhs_kernel         DotProdBasFuns (lib/bem2d_quadrature.h:111-156)
#include <algorithm>

#include "common.cuh"
#include "ff.cuh"
#include "kernel_ff.cuh"

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

// CK: complex wavenumber k + i ki (complex-argument Hankel functions).
template <int KERNEL, int NG, bool CK>
__global__ void __launch_bounds__(kFarThreads)
far_fp64_kernel(DevGeom g, NodeTable t, int ng_rt, double k, double ki, double eta,
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
        if (CK)
          kernel_c<KERNEL>(k, ki, eq, x1, y1, cs[o2], cs[SZ + o2], n1x, n1y,
                           cs[2 * SZ + o2], cs[3 * SZ + o2], &re, &im);
        else
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

template <int KERNEL, bool CK>
static void launch_far_k(const DevGeom& g, const NodeTable& t, int ng, double k, double ki,
                         double eta, double alpha, double2* out, long long ld,
                         cudaStream_t s) {
  const size_t smem = sizeof(double) * 10 * ng * kTile + sizeof(long long) * 4 * kTile;
  dim3 grid((g.n_unk + kTile - 1) / kTile, (g.n_unk + kTile - 1) / kTile);
  if constexpr (!CK) {  // the complex-k kernel keeps its node loop rolled
    if (ng == 5) {
      far_fp64_kernel<KERNEL, 5, false><<<grid, kFarThreads, smem, s>>>(g, t, ng, k, ki, eta,
                                                                        alpha, out, ld);
      return;
    }
  }
  auto fn = far_fp64_kernel<KERNEL, 0, CK>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  fn<<<grid, kFarThreads, smem, s>>>(g, t, ng, k, ki, eta, alpha, out, ld);
}

template <bool CK>
static void launch_far_any(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                           double ki, double eta, double alpha, double2* out, long long ld,
                           cudaStream_t s) {
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      launch_far_k<BEM2D_KERNEL_SINGLE, CK>(g, t, ng, k, ki, eta, alpha, out, ld, s);
      break;
    case BEM2D_KERNEL_DOUBLE:
      launch_far_k<BEM2D_KERNEL_DOUBLE, CK>(g, t, ng, k, ki, eta, alpha, out, ld, s);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      launch_far_k<BEM2D_KERNEL_CONJDOUBLE, CK>(g, t, ng, k, ki, eta, alpha, out, ld, s);
      break;
    default:
      launch_far_k<BEM2D_KERNEL_COMBINED, CK>(g, t, ng, k, ki, eta, alpha, out, ld, s);
  }
}

void launch_far_fp64(const DevGeom& g, const NodeTable& t, int ng, int kernel,
                     double k, double eta, double alpha, double2* out,
                     long long ld, cudaStream_t s) {
  launch_far_any<false>(g, t, ng, kernel, k, 0.0, eta, alpha, out, ld, s);
}

void launch_far_fp64_ck(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                        double ki, double eta, double alpha, double2* out, long long ld,
                        cudaStream_t s) {
  launch_far_any<true>(g, t, ng, kernel, k, ki, eta, alpha, out, ld, s);
}

// ---------------------------------------------------------------------------
// Near field: one warp per (test, trial) pair of adjacent or identical
// elements.  Lanes stride over the rule's points; a shuffle tree reduces.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
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

// Element geometry at the distinct coordinates of a rule, per warp in shared
// memory (structure of arrays): Map, Normal and |J| phi, phi the basis
// function of the pair's unknown on that element.
struct GeoTab {
  double* x;
  double* y;
  double* nx;
  double* ny;
  double* f;
};

__device__ __forceinline__ void geo_fill(const DevGeom& g, int e, int u, const double* vals, int n,
                                         bool mirror, const GeoTab& tb, int off, int lane) {
  const double* prm = g.param + 8 * (size_t)e;
  for (int v = lane; v < n; v += 32) {
    const double s = mirror ? 1 - vals[v] : vals[v];
    const ElemPt p = elem_eval(g.kind[e], prm, s);
    double nx, ny;
    elem_normal(p, &nx, &ny);
    tb.x[off + v] = p.mx;
    tb.y[off + v] = p.my;
    tb.nx[off + v] = nx;
    tb.ny[off + v] = ny;
    tb.f[off + v] = elem_jac(p) * basis_eval(g.unk_kind[u], g.unk_param[u], s);
  }
}

// K(x, y) (re1, im1) and, if PAIR, K(y, x) (re2, im2) at a test point x
// (normal n1) and a trial point y (normal n2).  FP64: kernel_d; MIXED: the
// distance and the normal factors from the FP64 difference w = x - y, the
// Bessel functions and the kernel in float-float.  CK (FP64 only): complex
// wavenumber k + i ki.
template <int KERNEL, bool MIXED, bool PAIR, bool CK>
__device__ __forceinline__ void near_point(double k, double ki, double kq, double eq,
                                           const KConstFF& kc,
                                           const float* tab, double ax, double ay, double n1x,
                                           double n1y, double bx, double by, double n2x,
                                           double n2y, double* re1, double* im1, double* re2,
                                           double* im2) {
  if (CK) {
    if (PAIR)
      kernel_c_pair<KERNEL>(k, ki, eq, ax, ay, bx, by, n1x, n1y, n2x, n2y, re1, im1, re2, im2);
    else
      kernel_c<KERNEL>(k, ki, eq, ax, ay, bx, by, n1x, n1y, n2x, n2y, re1, im1);
    return;
  }
  if (!MIXED) {
    if (PAIR)
      kernel_d_pair<KERNEL>(k, kq, eq, ax, ay, bx, by, n1x, n1y, n2x, n2y, re1, im1, re2, im2);
    else
      kernel_d<KERNEL>(k, kq, eq, ax, ay, bx, by, n1x, n1y, n2x, n2y, re1, im1);
    return;
  }
  const double wx = ax - bx, wy = ay - by;
  const ff dx = ff_from_double(wx), dy = ff_from_double(wy);
  const ff d2 = ff_add_fast(ff_sqr(dx), ff_sqr(dy));
  const ff id = ff_rsqrt(d2);  // 1/d
  const BesselFF b = bessel01_ff(ff_mul(ff_mul(d2, id), kc.k), ff_mul(id, kc.invk), tab);
  ff cd1 = ff_make(0.0f, 0.0f), cd2 = ff_make(0.0f, 0.0f);
  if (KERNEL != BEM2D_KERNEL_SINGLE) {
    const double n1w = fma(n1x, wx, n1y * wy);  // n_x . (x - y)
    const double n2w = fma(n2x, wx, n2y * wy);  // n_y . (x - y)
    cd1 = ff_mul(ff_from_double(KERNEL == BEM2D_KERNEL_DOUBLE ? -n2w : n1w), id);
    if (PAIR) cd2 = ff_mul(ff_from_double(KERNEL == BEM2D_KERNEL_DOUBLE ? n1w : -n2w), id);
  }
  const ffc K1 = kernel_from_bessel<KERNEL>(b, cd1, kc);
  *re1 = ff_to_double(K1.re);
  *im1 = ff_to_double(K1.im);
  if (PAIR) {
    if (KERNEL == BEM2D_KERNEL_SINGLE) {
      *re2 = *re1;
      *im2 = *im1;
    } else {
      const ffc K2 = kernel_from_bessel<KERNEL>(b, cd2, kc);
      *re2 = ff_to_double(K2.re);
      *im2 = ff_to_double(K2.im);
    }
  }
}

template <int KERNEL, bool MIXED, bool CK>
__global__ void __launch_bounds__(256)
near_kernel(DevGeom g, DevRules r, const NearPair* __restrict__ pairs, int npairs, double k,
            double ki, double eta, double alpha, double beta, KConstFF kc, const float* gtab, int cap_s,
            int cap_t, double2* __restrict__ out, long long ld, float2* __restrict__ out32,
            long long ld32) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* tab = reinterpret_cast<float*>(smem_raw);  // e^{ix} table (MIXED)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cap = cap_s + cap_t;
  double* base = reinterpret_cast<double*>(smem_raw + 1024) + (size_t)warp * 5 * cap;
  const GeoTab S{base, base + cap, base + 2 * cap, base + 3 * cap, base + 4 * cap};
  if (MIXED) {
    for (int v = threadIdx.x; v < 256; v += blockDim.x) tab[v] = gtab[v];
    __syncthreads();
  }
  const int wid = blockIdx.x * (blockDim.x >> 5) + warp;
  if (wid >= npairs) return;
  const NearPair pr = pairs[wid];
  const int e1 = g.unk_elem[pr.i], e2 = g.unk_elem[pr.j];
  const double kq = 0.25 * k, eq = 0.25 * eta;
  double acc_re = 0.0, acc_im = 0.0;
  double u1, u2;  // unused second orientation
  if (pr.rule == RULE_SELF) {
    // IntegrateIdent: Duffy split, points (x, (1-y)x) and (1-x, 1-x+yx),
    // both weighted by x * w.  Test-side geometry from the table (x values,
    // then 1 - x); trial-side evaluated per point.
    geo_fill(g, e1, pr.i, r.u1, r.nu1, false, S, 0, lane);
    geo_fill(g, e1, pr.i, r.u1, r.nu1, true, S, r.nu1, lane);
    __syncwarp();
    const double* p2 = g.param + 8 * (size_t)e2;
    for (int p = lane; p < r.n1; p += 32) {
      const double x = r.r1[3 * p], y = r.r1[3 * p + 1], w = r.r1[3 * p + 2];
      const int si = r.k1[p] & 0xffff;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int a = si + h * r.nu1;
        const double t = h == 0 ? (1 - y) * x : 1 - x + y * x;
        const ElemPt b = elem_eval(g.kind[e2], p2, t);
        double n2x, n2y, re, im;
        elem_normal(b, &n2x, &n2y);
        near_point<KERNEL, MIXED, false, CK>(k, ki, kq, eq, kc, tab, S.x[a], S.y[a], S.nx[a],
                                             S.ny[a], b.mx, b.my, n2x, n2y, &re, &im, &u1,
                                             &u2);
        const double f =
            S.f[a] * (elem_jac(b) * basis_eval(g.unk_kind[pr.j], g.unk_param[pr.j], t));
        acc_re = fma(re * f, x * w, acc_re);
        acc_im = fma(im * f, x * w, acc_im);
      }
    }
  } else {
    // AdaptedGauss2 / AdaptedGauss3: test geometry at the rule's x values,
    // trial geometry at its y values.  RULE_G3_PAIR: (i, j) with
    // AdaptedGauss3 at (x, y) and (j, i) with its mirror AdaptedGauss2 at
    // (y, x), the same point pairs, one evaluation each.
    const bool g2 = pr.rule == RULE_G2;
    const double* rule = g2 ? r.r2 : r.r3;
    const int* key = g2 ? r.k2 : r.k3;
    const int np = g2 ? r.n2 : r.n3;
    geo_fill(g, e1, pr.i, g2 ? r.u2 : r.u3, g2 ? r.nu2 : r.nu3, false, S, 0, lane);
    geo_fill(g, e2, pr.j, g2 ? r.v2 : r.v3, g2 ? r.nv2 : r.nv3, false, S, cap_s, lane);
    __syncwarp();
    if (pr.rule == RULE_G3_PAIR) {
      double acc2_re = 0.0, acc2_im = 0.0;
      for (int p = lane; p < np; p += 32) {
        const int kk = key[p];
        const int a = kk & 0xffff, b = cap_s + (kk >> 16);
        double r1, i1, r2, i2;
        near_point<KERNEL, MIXED, true, CK>(k, ki, kq, eq, kc, tab, S.x[a], S.y[a], S.nx[a],
                                            S.ny[a], S.x[b], S.y[b], S.nx[b], S.ny[b], &r1,
                                            &i1, &r2, &i2);
        const double f = S.f[a] * S.f[b] * rule[3 * p + 2];
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
        if (MIXED) out32[(size_t)pr.i * ld32 + pr.j] = make_float2((float)re, (float)im);
      }
    } else {
      for (int p = lane; p < np; p += 32) {
        const int kk = key[p];
        const int a = kk & 0xffff, b = cap_s + (kk >> 16);
        double re, im;
        near_point<KERNEL, MIXED, false, CK>(k, ki, kq, eq, kc, tab, S.x[a], S.y[a], S.nx[a],
                                             S.ny[a], S.x[b], S.y[b], S.nx[b], S.ny[b], &re,
                                             &im, &u1, &u2);
        const double f = S.f[a] * S.f[b] * rule[3 * p + 2];
        acc_re = fma(re, f, acc_re);
        acc_im = fma(im, f, acc_im);
      }
    }
  }
  acc_re = warp_sum(acc_re);
  acc_im = warp_sum(acc_im);
  if (lane == 0) {
    double re = alpha * acc_re, im = alpha * acc_im;
    if (pr.same && beta != 0.0) re = fma(beta, mass_entry(g, r, pr.i, pr.j), re);
    out[(size_t)pr.j * ld + pr.i] = make_double2(re, im);
    if (MIXED) out32[(size_t)pr.j * ld32 + pr.i] = make_float2((float)re, (float)im);
  }
}

// Table capacities (entries per warp) of the near-field kernel for rules r.
static void near_caps(const DevRules& r, int* cap_s, int* cap_t) {
  *cap_s = std::max(2 * r.nu1, std::max(r.nu2, r.nu3));
  *cap_t = std::max(r.nv2, r.nv3);
}

size_t near_table_bytes(const DevRules& r) {
  int cs, ct;
  near_caps(r, &cs, &ct);
  return sizeof(double) * 5 * (size_t)(cs + ct);
}

template <int KERNEL, bool MIXED, bool CK>
static void launch_near_k(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                          double k, double ki, double eta, double alpha, double beta,
                          const float* tab,
                          double2* out, long long ld, float2* out32, long long ld32,
                          cudaStream_t s) {
  int cs, ct;
  near_caps(r, &cs, &ct);
  const size_t per_warp = std::max<size_t>(near_table_bytes(r), 8);  // L = 0: empty rules
  // warps per block: up to 8, within 96 KB of shared memory
  const int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024 - 1024) / per_warp));
  const size_t smem = 1024 + per_warp * wpb;
  const int blocks = (npairs + wpb - 1) / wpb;
  auto fn = near_kernel<KERNEL, MIXED, CK>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  fn<<<blocks, 32 * wpb, smem, s>>>(g, r, pairs, npairs, k, ki, eta, alpha, beta,
                                     make_kconst(k, eta), tab, cs, ct, out, ld, out32, ld32);
}

template <bool MIXED, bool CK>
static void launch_near_m(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                          int kernel, double k, double ki, double eta, double alpha, double beta,
                          const float* tab, double2* out, long long ld, float2* out32,
                          long long ld32, cudaStream_t s) {
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      launch_near_k<BEM2D_KERNEL_SINGLE, MIXED, CK>(g, r, pairs, npairs, k, ki, eta, alpha,
                                                    beta, tab, out, ld, out32, ld32, s);
      break;
    case BEM2D_KERNEL_DOUBLE:
      launch_near_k<BEM2D_KERNEL_DOUBLE, MIXED, CK>(g, r, pairs, npairs, k, ki, eta, alpha,
                                                    beta, tab, out, ld, out32, ld32, s);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      launch_near_k<BEM2D_KERNEL_CONJDOUBLE, MIXED, CK>(g, r, pairs, npairs, k, ki, eta, alpha,
                                                        beta, tab, out, ld, out32, ld32, s);
      break;
    default:
      launch_near_k<BEM2D_KERNEL_COMBINED, MIXED, CK>(g, r, pairs, npairs, k, ki, eta, alpha,
                                                      beta, tab, out, ld, out32, ld32, s);
  }
}

int launch_near(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                int kernel, double k, double eta, double alpha, double beta, double2* out,
                long long ld, cudaStream_t s, float2* out32, long long ld32) {
  if (npairs == 0) return BEM2D_OK;
  if (out32) {
    const float* tab = expi_table_dev();
    if (!tab) return BEM2D_ERR_NOMEM;
    launch_near_m<true, false>(g, r, pairs, npairs, kernel, k, 0.0, eta, alpha, beta, tab, out,
                               ld, out32, ld32, s);
  } else {
    launch_near_m<false, false>(g, r, pairs, npairs, kernel, k, 0.0, eta, alpha, beta, nullptr,
                                out, ld, nullptr, 0, s);
  }
  return BEM2D_OK;
}

int launch_near_ck(const DevGeom& g, const DevRules& r, const NearPair* pairs, int npairs,
                   int kernel, double k, double ki, double eta, double alpha, double beta,
                   double2* out, long long ld, cudaStream_t s) {
  if (npairs == 0) return BEM2D_OK;
  launch_near_m<false, true>(g, r, pairs, npairs, kernel, k, ki, eta, alpha, beta, nullptr, out,
                             ld, nullptr, 0, s);
  return BEM2D_OK;
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
// functionals (lib/bem2d_fun.h:14-93).  The wavenumber is k + i ki:
// e^{i (k + i ki) d.x} = e^{-ki d.x} e^{i k d.x}.
__global__ void rhs_kernel(int n, NodeTable t, int ng, int fun, double k, double ki,
                           double dx, double dy, double eta, double scale,
                           double2* __restrict__ out) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  double acc_re = 0.0, acc_im = 0.0;
  for (int q = 0; q < ng; ++q) {
    const size_t o = (size_t)u * ng + q;
    const double dd = dx * t.x[o] + dy * t.y[o];
    const double ph = k * dd;
    double fs, fc;
    sincos(ph, &fs, &fc);
    if (ki != 0.0) {
      const double a = exp(-ki * dd);
      fs *= a;
      fc *= a;
    }
    double vr, vi;
    if (fun == BEM2D_FUN_PLANEWAVE) {
      vr = fc;
      vi = fs;
    } else {
      const double nd = t.nx[o] * dx + t.ny[o] * dy;
      vr = -k * fs * nd;  // i k f (n.d)
      vi = k * fc * nd;
      if (ki != 0.0) {  // the i * (i ki) f (n.d) part
        vr -= ki * fc * nd;
        vi -= ki * fs * nd;
      }
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
                cudaStream_t s, double ki) {
  rhs_kernel<<<(g.n_unk + 127) / 128, 128, 0, s>>>(g.n_unk, t, ng, fun, k, ki, dx, dy,
                                                   eta, scale, out);
}

// ---------------------------------------------------------------------------
// Potential of a density at points (EvalKernel, lib/bem2d_quadrature.h:184-228):
// out[p] = sum_u c_u sum_q K(x_p, y_uq) W_uq, both normals the source node's.
// One thread per point; unknowns staged through shared memory in chunks.
// CK: complex wavenumber k + i ki.
template <int KERNEL, bool CK>
__global__ void __launch_bounds__(128)
potential_kernel(int nunk, NodeTable t, int ng, double k, double ki, double eta,
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
        double kvr, kvi;
        if (CK)
          kernel_c<KERNEL>(k, ki, eq, px, py, sx[i], sy[i], snx[i], sny[i], snx[i], sny[i],
                           &kvr, &kvi);
        else
          kernel_d<KERNEL>(k, kq, eq, px, py, sx[i], sy[i], snx[i], sny[i], snx[i], sny[i],
                           &kvr, &kvi);
        // coefficient * kernel * weight
        const double2 c = sc[i];
        const double vr = (c.x * kvr - c.y * kvi) * sw[i],
                     vi = (c.x * kvi + c.y * kvr) * sw[i];
        ar += vr;
        ai += vi;
      }
    }
  }
  if (p < npts) out[p] = make_double2(ar, ai);
}

template <bool CK>
static void launch_potential_k(const DevGeom& g, const NodeTable& t, int ng, int kernel,
                               double k, double ki, double eta, const double2* coef, int npts,
                               const double* pts, double2* out, cudaStream_t s) {
  const int blocks = (npts + 127) / 128;
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      potential_kernel<BEM2D_KERNEL_SINGLE, CK>
          <<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, ki, eta, coef, npts, pts, out);
      break;
    case BEM2D_KERNEL_DOUBLE:
      potential_kernel<BEM2D_KERNEL_DOUBLE, CK>
          <<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, ki, eta, coef, npts, pts, out);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      potential_kernel<BEM2D_KERNEL_CONJDOUBLE, CK>
          <<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, ki, eta, coef, npts, pts, out);
      break;
    default:
      potential_kernel<BEM2D_KERNEL_COMBINED, CK>
          <<<blocks, 128, 0, s>>>(g.n_unk, t, ng, k, ki, eta, coef, npts, pts, out);
  }
}

void launch_potential(const DevGeom& g, const NodeTable& t, int ng, int kernel, double k,
                      double eta, const double2* coef, int npts, const double* pts,
                      double2* out, cudaStream_t s, double ki) {
  if (ki != 0.0)
    launch_potential_k<true>(g, t, ng, kernel, k, ki, eta, coef, npts, pts, out, s);
  else
    launch_potential_k<false>(g, t, ng, kernel, k, 0.0, eta, coef, npts, pts, out, s);
}

}  // namespace bem2d_gpu
