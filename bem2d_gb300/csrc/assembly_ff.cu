// Mixed-precision far-field assembly (sm_103a): the bulk of the Galerkin
// matrix evaluated in float-float arithmetic on the FP32 pipe.
//
// Same tiling as the FP64 far kernel (32 x 32 tiles, one lane per test
// unknown, node data staged in shared memory).  Pair geometry: the centre
// difference of the two elements in FP64, node offsets from the centres in
// float-float, so |x - y| keeps ~48 bits relative to itself even for
// neighbouring elements.  Entries whose element pair admits k|x - y| <= 4
// anywhere (bounded with the element radii) are deferred to a second
// float-float pass (deferred_ff_kernel, one thread per element pair), which
// carries the small-argument Bessel branch; keeping them out of the tile
// loop keeps its warps on one branch.  Adjacent and identical pairs belong to
// the near-field kernel as in the FP64 path.  Each entry is stored twice:
// complex128 (refinement residual) and complex64 (the LU).
#include <mutex>

#include "common.cuh"
#include "ff.cuh"
#include "hankel_ff.cuh"
#include "kernel_ff.cuh"

namespace bem2d_gpu {

// The distance-dependent part of the kernel at one node pair: 1/d, the
// asymptotic P/Q factors of H0 and H1, 1/sqrt(x) (the amplitude
// sqrt(2/(pi x)) without its constant) and e^{i(x - pi/4)}.  Shared by entry
// (i, j) and entry (j, i).
struct HankelTermsFF {
  ff y, p0, q0, p1, q1, rx;
  ffc e;
};

__device__ __forceinline__ HankelTermsFF hankel_terms_ff(ff dx, ff dy, const KConstFF& kc,
                                                        const float* tab) {
  HankelTermsFF h;
  const ff d2 = ff_dot2(dx, dx, dy, dy);
  h.y = ff_rsqrt(d2);  // 1/d
  const ff d = ff_mul(d2, h.y);
  const ff x = ff_mul(d, kc.k);
  const ff ix = ff_mul(h.y, kc.invk);
  pq_ff(x.hi, ix, &h.p0, &h.q0, &h.p1, &h.q1);
  h.rx = ff_rsqrt(x);
  h.e = expi_ff(x, tab);
  return h;
}

// E (P + i Q) and a complex value times a real one (ff).
__device__ __forceinline__ ffc ffc_mul_pq(const ffc& e, ff p, ff q) {
  ffc r;
  r.re = ff_dot2(e.re, p, ff_neg(e.im), q);
  r.im = ff_dot2(e.re, q, e.im, p);
  return r;
}

// acc += v without renormalising acc: acc.lo gathers the hi sums' rounding
// errors and the lo parts (ff_acc_norm restores |lo| <= ulp(hi)/2 after a
// few steps, so that the FP32 sum in lo stays ~2^-48 |acc| accurate)
__device__ __forceinline__ void ff_acc(ff& acc, ff v) {
  const ff s = two_sum(acc.hi, v.hi);
  acc.hi = s.hi;
  acc.lo += s.lo + v.lo;
}
__device__ __forceinline__ void ff_acc_norm(ff& acc) { acc = fast_two_sum(acc.hi, acc.lo); }

__device__ __forceinline__ ffc ffc_scale(const ffc& z, ff a) {
  ffc r;
  r.re = ff_mul(z.re, a);
  r.im = ff_mul(z.im, a);
  return r;
}

// One entry in FP64 from the FP64 node table (deferred entries).
template <int KERNEL>
__device__ __forceinline__ void entry_fp64(const NodeTable& t, int ng, int row, int col,
                                           double k, double kq, double eq, double* re,
                                           double* im) {
  double ar = 0.0, ai = 0.0;
  for (int q1 = 0; q1 < ng; ++q1) {
    const size_t a = (size_t)row * ng + q1;
    const double x1 = t.x[a], y1 = t.y[a], n1x = t.nx[a], n1y = t.ny[a], w1 = t.w[a];
    for (int q2 = 0; q2 < ng; ++q2) {
      const size_t b = (size_t)col * ng + q2;
      double vr, vi;
      kernel_d<KERNEL>(k, kq, eq, x1, y1, t.x[b], t.y[b], n1x, n1y, t.nx[b], t.ny[b], &vr, &vi);
      const double ww = w1 * t.w[b];
      ar = fma(vr, ww, ar);
      ai = fma(vi, ww, ai);
    }
  }
  *re = ar;
  *im = ai;
}

constexpr int kTileF = 32;
constexpr int kDeferRC = 1 << 30;  // deferred item: entry (row, col) wanted
constexpr int kDeferCR = 1 << 29;  // deferred item: entry (col, row) wanted
constexpr int kDeferIdx = kDeferCR - 1;
constexpr int kFarFFThreads = 256;
constexpr float kDeferX = 4.001f;

// Tiles are processed in symmetric pairs: CTA b owns tile (I, J), I <= J,
// and computes both (I, J) and (J, I).  The distance-dependent work at a node
// pair (the Hankel terms, most of the cost) is the same for entry (r, c) and
// entry (c, r); only the normal factor of the double-layer kernels differs.
// Entry (r, c) is stored directly (a warp writes 32 consecutive rows of a
// column); entry (c, r) goes to a shared-memory copy of tile (J, I) that is
// written out, column by column, at the end.  A pair that is near in either
// direction is left, in that direction, to the near-field kernel; the
// small-argument test depends on the distance only, so a deferred pair is
// deferred in both directions.  On a diagonal tile only r < c is computed.
__device__ __forceinline__ void tile_of(unsigned b, int* I, int* J) {
  int j = (int)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while ((long long)(j + 1) * (j + 2) / 2 <= (long long)b) ++j;
  while ((long long)j * (j + 1) / 2 > (long long)b) --j;
  *J = j;
  *I = (int)((long long)b - (long long)j * (j + 1) / 2);
}

template <int KERNEL, int NG>
__global__ void __launch_bounds__(kFarFFThreads, 2)
far_ff_kernel(DevGeom g, NodeTable t, NodeTableFF tf, int ng_rt, KConstFF kc, double k,
              double eta, double alpha, double2* __restrict__ out, long long ld,
              float2* __restrict__ out32, long long ld32, DeferList dl, const float* gtab) {
  const int ng = NG > 0 ? NG : ng_rt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tT = reinterpret_cast<double2*>(smem_raw);          // [32][33] tile (J, I)
  unsigned* vT = reinterpret_cast<unsigned*>(tT + kTileF * (kTileF + 1));  // [32] masks
  float* tab = reinterpret_cast<float*>(vT + kTileF);          // 256
  double2* cen = reinterpret_cast<double2*>(tab + 256);        // rows 32, cols 32
  float2* rs = reinterpret_cast<float2*>(cen + 2 * kTileF);    // [5][ng][32]
  float2* cs = rs + 5 * ng * kTileF;                           // [5][ng][32]
  float* rad = reinterpret_cast<float*>(cs + 5 * ng * kTileF); // rows 32, cols 32
  long long* links = reinterpret_cast<long long*>(rad + 2 * kTileF);  // 6 x 32

  int I, J;
  tile_of(blockIdx.x, &I, &J);
  const int row0 = I * kTileF, col0 = J * kTileF;
  const bool diag = I == J;
  const int n = g.n_unk;
  for (int v = threadIdx.x; v < 256; v += blockDim.x) tab[v] = gtab[v];
  if (threadIdx.x < kTileF) vT[threadIdx.x] = 0u;
  const int SZ = ng * kTileF;
  for (int v = threadIdx.x; v < SZ; v += blockDim.x) {
    const int q = v / kTileF, l = v - q * kTileF;
    const int ur = min(row0 + l, n - 1), uc = min(col0 + l, n - 1);
    const size_t ir = (size_t)ur * ng + q, ic = (size_t)uc * ng + q;
    const int o = q * kTileF + l;
    rs[o] = tf.ox[ir];
    rs[SZ + o] = tf.oy[ir];
    rs[2 * SZ + o] = tf.nx[ir];
    rs[3 * SZ + o] = tf.ny[ir];
    rs[4 * SZ + o] = tf.w[ir];
    cs[o] = tf.ox[ic];
    cs[SZ + o] = tf.oy[ic];
    cs[2 * SZ + o] = tf.nx[ic];
    cs[3 * SZ + o] = tf.ny[ic];
    cs[4 * SZ + o] = tf.w[ic];
  }
  if (threadIdx.x < kTileF) {
    const int l = threadIdx.x;
    const int ur = min(row0 + l, n - 1), uc = min(col0 + l, n - 1);
    cen[l] = tf.c[ur];
    cen[kTileF + l] = tf.c[uc];
    rad[l] = tf.rad[ur];
    rad[kTileF + l] = tf.rad[uc];
    const int er = g.unk_elem[ur], ec = g.unk_elem[uc];
    links[l] = g.index[er];
    links[kTileF + l] = g.next[er];
    links[2 * kTileF + l] = g.prev[er];
    links[3 * kTileF + l] = g.index[ec];
    links[4 * kTileF + l] = g.next[ec];
    links[5 * kTileF + l] = g.prev[ec];
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = row0 + lane;
  const long long ri = links[lane], rn = links[kTileF + lane], rp = links[2 * kTileF + lane];
  const double2 crow = cen[lane];
  const float rrow = rad[lane];
  const float kf = (float)k;

#pragma unroll 1
  for (int cc = warp; cc < kTileF; cc += kFarFFThreads / 32) {
    const int col = col0 + cc;
    const long long ci = links[3 * kTileF + cc], cn = links[4 * kTileF + cc],
                    cp = links[5 * kTileF + cc];
    // rc: entry (row, col); cr: entry (col, row)
    bool rc = row < n && col < n && !((ri == ci) || (rn == ci) || (rp == ci));
    bool cr = row < n && col < n && !((ci == ri) || (cn == ri) || (cp == ri));
    if (diag && lane >= cc) rc = cr = false;
    if (!rc && !cr) continue;
    const double dxc = crow.x - cen[kTileF + cc].x, dyc = crow.y - cen[kTileF + cc].y;
    const float dist = sqrtf((float)(dxc * dxc + dyc * dyc));
    if (kf * (dist * (1.0f - 1e-6f) - rrow - rad[kTileF + cc]) <= kDeferX) {
      // small arguments somewhere on this pair: second pass (or here, in
      // FP64, if the list is full).  One list item per pair: (row, col) with the flags
      // kDeferRC / kDeferCR in the top bits of .x for the directions needed.
      const unsigned slot = atomicAdd(dl.count, 1u);
      if (slot < dl.capacity) {
        dl.ij[slot] = make_int2(row | (rc ? kDeferRC : 0) | (cr ? kDeferCR : 0), col);
      } else {
        for (int dir = 0; dir < 2; ++dir) {
          if (!(dir == 0 ? rc : cr)) continue;
          const int a = dir == 0 ? row : col, b = dir == 0 ? col : row;
          double re, im;
          entry_fp64<KERNEL>(t, ng, a, b, k, 0.25 * k, 0.25 * eta, &re, &im);
          out[(size_t)b * ld + a] = make_double2(alpha * re, alpha * im);
          out32[(size_t)b * ld32 + a] = make_float2((float)(alpha * re), (float)(alpha * im));
        }
      }
      continue;
    }
    const ff Dx = ff_from_double(dxc), Dy = ff_from_double(dyc);
    // s0: the terms both orientations share (the single-layer part), t_rc /
    // t_cr: the normal-factor terms of entry (row, col) / (col, row)
    ffc s0, trc, tcr;
    s0.re = s0.im = trc.re = trc.im = tcr.re = tcr.im = ff_make(0.0f, 0.0f);
#pragma unroll 1
    for (int q1 = 0; q1 < ng; ++q1) {
      const int o1 = q1 * kTileF + lane;
      const float2 a0 = rs[o1], a1 = rs[SZ + o1], a2 = rs[2 * SZ + o1], a3 = rs[3 * SZ + o1],
                   a4 = rs[4 * SZ + o1];
      // the row node's position relative to the column element's centre,
      // once per row node: (c_row - c_col) + o_row
      const ff Px = ff_add_fast(Dx, ff_make(a0.x, a0.y));
      const ff Py = ff_add_fast(Dy, ff_make(a1.x, a1.y));
      const ff n1x = ff_make(a2.x, a2.y), n1y = ff_make(a3.x, a3.y);
      // the row node's constant factors: amp0 w_x with k/4 (double-layer
      // part) and eta/4 or 1/4 (single-layer part)
      const ff aw1 = ff_mul(kc.amp0, ff_make(a4.x, a4.y));
      const ff c1 = ff_mul(aw1, kc.kq);
      const ff c0 = KERNEL == BEM2D_KERNEL_SINGLE ? ff_scale2(aw1, 0.25f) : ff_mul(aw1, kc.eq);
#pragma unroll 1
      for (int q2 = 0; q2 < ng; ++q2) {
        const int o2 = q2 * kTileF + cc;
        const float2 b0 = cs[o2], b1 = cs[SZ + o2], b2 = cs[2 * SZ + o2], b3 = cs[3 * SZ + o2],
                     b4 = cs[4 * SZ + o2];
        // w = x - y, x a node of the row element, y of the column element
        const ff dx = ff_add_fast(Px, ff_make(-b0.x, -b0.y));
        const ff dy = ff_add_fast(Py, ff_make(-b1.x, -b1.y));
        const HankelTermsFF h = hankel_terms_ff(dx, dy, kc, tab);
        const ff g = ff_mul(h.rx, ff_make(b4.x, b4.y));  // w_y / sqrt(x)
        if (KERNEL == BEM2D_KERNEL_SINGLE) {
          // K w_x w_y = (i/4) amp w_x w_y E (P0 + i Q0), the same in both
          // orientations
          const ffc Z = ffc_scale(ffc_mul_pq(h.e, h.p0, h.q0), ff_mul(g, c0));
          ff_acc(s0.re, ff_neg(Z.im));
          ff_acc(s0.im, Z.re);
        } else {
          // K w_x w_y = Z0 - dot Z1 with Z1 = amp w_x w_y (k/4)/d E (P1 + i Q1)
          // and, for the combined operator, Z0 = amp w_x w_y (eta/4) E (P0 +
          // i Q0); dot is the orientation's normal factor (n_y . (y - x) for
          // the double layer at (x, y), n_x . (x - y) otherwise)
          const ffc Z1 = ffc_scale(ffc_mul_pq(h.e, h.p1, h.q1), ff_mul(ff_mul(g, h.y), c1));
          if (KERNEL == BEM2D_KERNEL_COMBINED) {
            const ffc Z0 = ffc_scale(ffc_mul_pq(h.e, h.p0, h.q0), ff_mul(g, c0));
            ff_acc(s0.re, Z0.re);
            ff_acc(s0.im, Z0.im);
          }
          const ff n1w = ff_dot2(n1x, dx, n1y, dy);                                // n_x . (x - y)
          const ff n2w = ff_dot2(ff_make(b2.x, b2.y), dx, ff_make(b3.x, b3.y), dy);  // n_y . (x - y)
          // (row, col): -dot = n2w (double layer) or -n1w; (col, row): the reverse
          const ff m_rc = KERNEL == BEM2D_KERNEL_DOUBLE ? n2w : ff_neg(n1w);
          const ff m_cr = KERNEL == BEM2D_KERNEL_DOUBLE ? ff_neg(n1w) : n2w;
          if (rc) {
            ff_acc(trc.re, ff_mul(m_rc, Z1.re));
            ff_acc(trc.im, ff_mul(m_rc, Z1.im));
          }
          if (cr) {
            ff_acc(tcr.re, ff_mul(m_cr, Z1.re));
            ff_acc(tcr.im, ff_mul(m_cr, Z1.im));
          }
        }
      }
      ff_acc_norm(s0.re);
      ff_acc_norm(s0.im);
      ff_acc_norm(trc.re);
      ff_acc_norm(trc.im);
      ff_acc_norm(tcr.re);
      ff_acc_norm(tcr.im);
    }
    ffc arc, acr;
    arc.re = ff_add(s0.re, trc.re);
    arc.im = ff_add(s0.im, trc.im);
    acr.re = ff_add(s0.re, tcr.re);
    acr.im = ff_add(s0.im, tcr.im);
    if (rc) {
      const double re = alpha * ff_to_double(arc.re), im = alpha * ff_to_double(arc.im);
      out[(size_t)col * ld + row] = make_double2(re, im);
      out32[(size_t)col * ld32 + row] = make_float2((float)re, (float)im);
    }
    if (cr) {
      tT[cc * (kTileF + 1) + lane] =
          make_double2(alpha * ff_to_double(acr.re), alpha * ff_to_double(acr.im));
      atomicOr(&vT[cc], 1u << lane);
    }
  }
  __syncthreads();
  // tile (J, I): entry (col0 + cc, row0 + l) = tT[cc][l]; a warp writes 32
  // consecutive rows (cc) of one column (row0 + l)
  for (int l = warp; l < kTileF; l += kFarFFThreads / 32) {
    const int cc = lane;
    if (!((vT[cc] >> l) & 1u)) continue;
    const double2 v = tT[cc * (kTileF + 1) + l];
    out[(size_t)(row0 + l) * ld + col0 + cc] = v;
    out32[(size_t)(row0 + l) * ld32 + col0 + cc] = make_float2((float)v.x, (float)v.y);
  }
}

template <int KERNEL>
__global__ void __launch_bounds__(128)
deferred_ff_kernel(NodeTableFF tf, int ng, KConstFF kc, double alpha, const int2* __restrict__ ij,
                   const unsigned* count, unsigned cap, double2* __restrict__ out, long long ld,
                   float2* __restrict__ out32, long long ld32, const float* gtab) {
  // one item = one element pair; both orientations share every distance
  // and Bessel evaluation.  Same pair geometry as far_ff_kernel: the centre
  // difference in FP64, node offsets in ff.
  __shared__ float tab[256];
  for (int v = threadIdx.x; v < 256; v += blockDim.x) tab[v] = gtab[v];
  __syncthreads();
  const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= min(*count, cap)) return;
  const int2 e = ij[p];
  const int row = e.x & kDeferIdx, col = e.y;
  const bool want_rc = (e.x & kDeferRC) != 0, want_cr = (e.x & kDeferCR) != 0;
  const double2 cr0 = tf.c[row], cc0 = tf.c[col];
  const ff Dx = ff_from_double(cr0.x - cc0.x), Dy = ff_from_double(cr0.y - cc0.y);
  ffc arc, acr;
  arc.re = arc.im = acr.re = acr.im = ff_make(0.0f, 0.0f);
#pragma unroll 1
  for (int q1 = 0; q1 < ng; ++q1) {
    const size_t a = (size_t)row * ng + q1;
    const float2 a0 = tf.ox[a], a1 = tf.oy[a], a2 = tf.nx[a], a3 = tf.ny[a], a4 = tf.w[a];
    const ff ox1 = ff_make(a0.x, a0.y), oy1 = ff_make(a1.x, a1.y);
    const ff n1x = ff_make(a2.x, a2.y), n1y = ff_make(a3.x, a3.y), w1 = ff_make(a4.x, a4.y);
#pragma unroll 1
    for (int q2 = 0; q2 < ng; ++q2) {
      const size_t b = (size_t)col * ng + q2;
      const float2 b0 = tf.ox[b], b1 = tf.oy[b], b2 = tf.nx[b], b3 = tf.ny[b], b4 = tf.w[b];
      // w = x - y, x a node of the row element, y of the column element
      const ff dx = ff_add_fast(Dx, ff_add_fast(ox1, ff_make(-b0.x, -b0.y)));
      const ff dy = ff_add_fast(Dy, ff_add_fast(oy1, ff_make(-b1.x, -b1.y)));
      const ff d2 = ff_add_fast(ff_sqr(dx), ff_sqr(dy));
      const ff id = ff_rsqrt(d2);  // 1/d
      const ff x = ff_mul(ff_mul(d2, id), kc.k);
      const BesselFF bs = bessel01_ff(x, ff_mul(id, kc.invk), tab);
      const ff ww = ff_mul(w1, ff_make(b4.x, b4.y));
      ff cd_rc = ff_make(0.0f, 0.0f), cd_cr = ff_make(0.0f, 0.0f);
      if (KERNEL != BEM2D_KERNEL_SINGLE) {
        const ff n1w = ff_mul(ff_add_fast(ff_mul(n1x, dx), ff_mul(n1y, dy)), id);
        const ff n2w = ff_mul(ff_add_fast(ff_mul(ff_make(b2.x, b2.y), dx),
                                          ff_mul(ff_make(b3.x, b3.y), dy)), id);
        if (KERNEL == BEM2D_KERNEL_DOUBLE) {
          cd_rc = ff_neg(n2w);  // (row, col): n_y . (y - x) / d
          cd_cr = n1w;          // (col, row): n_x . (x - y) / d
        } else {
          cd_rc = n1w;
          cd_cr = ff_neg(n2w);
        }
      }
      const ffc K1 = kernel_from_bessel<KERNEL>(bs, cd_rc, kc);
      arc.re = ff_add_fast(arc.re, ff_mul(K1.re, ww));
      arc.im = ff_add_fast(arc.im, ff_mul(K1.im, ww));
      if (KERNEL == BEM2D_KERNEL_SINGLE) {
        acr = arc;
      } else {
        const ffc K2 = kernel_from_bessel<KERNEL>(bs, cd_cr, kc);
        acr.re = ff_add_fast(acr.re, ff_mul(K2.re, ww));
        acr.im = ff_add_fast(acr.im, ff_mul(K2.im, ww));
      }
    }
  }
  if (want_rc) {
    const double re = alpha * ff_to_double(arc.re), im = alpha * ff_to_double(arc.im);
    out[(size_t)col * ld + row] = make_double2(re, im);
    out32[(size_t)col * ld32 + row] = make_float2((float)re, (float)im);
  }
  if (want_cr) {
    const double re = alpha * ff_to_double(acr.re), im = alpha * ff_to_double(acr.im);
    out[(size_t)row * ld + col] = make_double2(re, im);
    out32[(size_t)row * ld32 + col] = make_float2((float)re, (float)im);
  }
}

const float* expi_table_dev() {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static float* tab[kMaxDev] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDev) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!tab[dev]) {
    float h[256];
    expi_table(h);
    float* d = nullptr;
    if (cudaMalloc(&d, sizeof h) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice);
    tab[dev] = d;
  }
  return tab[dev];
}

template <int KERNEL>
static int launch_far_ff_k(const DevGeom& g, const NodeTable& t, const NodeTableFF& tf, int ng,
                            double k, double eta, double alpha, double2* out, long long ld,
                            float2* out32, long long ld32, DeferList dl, cudaStream_t s) {
  const KConstFF kc = make_kconst(k, eta);
  const size_t smem = sizeof(double2) * kTileF * (kTileF + 1) + sizeof(unsigned) * kTileF +
                      sizeof(float) * 256 + sizeof(double2) * 2 * kTileF +
                      sizeof(float2) * 10 * ng * kTileF + sizeof(float) * 2 * kTileF +
                      sizeof(long long) * 6 * kTileF;
  const unsigned nt = (unsigned)((g.n_unk + kTileF - 1) / kTileF);
  dim3 grid(nt * (nt + 1) / 2);  // tile pairs (I, J), I <= J
  const float* tab = expi_table_dev();
  if (!tab) return BEM2D_ERR_NOMEM;
  if (ng == 5) {
    far_ff_kernel<KERNEL, 5><<<grid, kFarFFThreads, smem, s>>>(g, t, tf, ng, kc, k, eta, alpha, out,
                                                               ld, out32, ld32, dl, tab);
  } else {
    auto fn = far_ff_kernel<KERNEL, 0>;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    fn<<<grid, kFarFFThreads, smem, s>>>(g, t, tf, ng, kc, k, eta, alpha, out, ld, out32, ld32, dl,
                                         tab);
  }
  return BEM2D_OK;
}

int launch_far_ff(const DevGeom& g, const NodeTable& t, const NodeTableFF& tf, int ng,
                  int kernel, double k, double eta, double alpha, double2* out,
                  long long ld, float2* out32, long long ld32, DeferList dl,
                  cudaStream_t s) {
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      return launch_far_ff_k<BEM2D_KERNEL_SINGLE>(g, t, tf, ng, k, eta, alpha, out, ld, out32,
                                                  ld32, dl, s);
    case BEM2D_KERNEL_DOUBLE:
      return launch_far_ff_k<BEM2D_KERNEL_DOUBLE>(g, t, tf, ng, k, eta, alpha, out, ld, out32,
                                                  ld32, dl, s);
    case BEM2D_KERNEL_CONJDOUBLE:
      return launch_far_ff_k<BEM2D_KERNEL_CONJDOUBLE>(g, t, tf, ng, k, eta, alpha, out, ld, out32,
                                                      ld32, dl, s);
    default:
      return launch_far_ff_k<BEM2D_KERNEL_COMBINED>(g, t, tf, ng, k, eta, alpha, out, ld, out32,
                                                    ld32, dl, s);
  }
}

// Grid sized by the list capacity; threads beyond the device-side count exit.
int launch_deferred(const NodeTableFF& tf, int ng, int kernel, double k, double eta,
                    double alpha, const DeferList& dl, double2* out, long long ld,
                    float2* out32, long long ld32, cudaStream_t s) {
  if (dl.capacity == 0) return BEM2D_OK;
  const float* tab = expi_table_dev();
  if (!tab) return BEM2D_ERR_NOMEM;
  const KConstFF kc = make_kconst(k, eta);
  const unsigned blocks = (dl.capacity + 127) / 128;
  switch (kernel) {
    case BEM2D_KERNEL_SINGLE:
      deferred_ff_kernel<BEM2D_KERNEL_SINGLE><<<blocks, 128, 0, s>>>(tf, ng, kc, alpha, dl.ij, dl.count, dl.capacity, out, ld, out32, ld32, tab);
      break;
    case BEM2D_KERNEL_DOUBLE:
      deferred_ff_kernel<BEM2D_KERNEL_DOUBLE><<<blocks, 128, 0, s>>>(tf, ng, kc, alpha, dl.ij, dl.count, dl.capacity, out, ld, out32, ld32, tab);
      break;
    case BEM2D_KERNEL_CONJDOUBLE:
      deferred_ff_kernel<BEM2D_KERNEL_CONJDOUBLE><<<blocks, 128, 0, s>>>(tf, ng, kc, alpha, dl.ij, dl.count, dl.capacity, out, ld, out32, ld32, tab);
      break;
    default:
      deferred_ff_kernel<BEM2D_KERNEL_COMBINED><<<blocks, 128, 0, s>>>(tf, ng, kc, alpha, dl.ij, dl.count, dl.capacity, out, ld, out32, ld32, tab);
  }
  return BEM2D_OK;
}

}  // namespace bem2d_gpu
