// C ABI of the bem2d GB300 path (include/bem2d_gpu.h): context, device
// workspace, host-side geometry checks, quadrature rules, near-pair lists and
// the orchestration of the assembly and solve kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <functional>
#include <vector>

#include "common.cuh"
#include "dense.cuh"

namespace bem2d_gpu {

// ---------------------------------------------------------------------------
// Context: one stream, a pool of named device buffers that only grow, and
// cached quadrature rules.
struct Buffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct RuleKey {
  int L, N;
  double sigma;
  bool operator<(const RuleKey& o) const {
    if (L != o.L) return L < o.L;
    if (N != o.N) return N < o.N;
    return sigma < o.sigma;
  }
};

struct HostRules {
  std::vector<double> gx, gw, r1, r2, r3;  // r*: (x, y, w) triplets
};

}  // namespace bem2d_gpu

struct bem2d_ctx {
  // per-phase event timers (measurement helpers)
  bool timers = false;
  double phase_ms[4] = {0, 0, 0, 0};
  long long phase_n[4] = {0, 0, 0, 0};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  long long launches = 0;
  std::unordered_map<std::string, bem2d_gpu::Buffer> bufs;
  std::map<bem2d_gpu::RuleKey, std::pair<void*, bem2d_gpu::DevRules>> rules;
  std::vector<bem2d_ctx*> workers;  // per-thread contexts of batched sweeps
  // Sweep workers: a high-priority stream for the factor/solve phase of a
  // scattering solve (the assembly stays on `stream`), ordered by events.
  cudaStream_t stream_hi = nullptr;
  cudaEvent_t ev_asm = nullptr, ev_sol = nullptr;
  int panel_min_rows = 0;  // LuWork::min_rows of this context's factorisations
  int tc_ctas = 0;         // LuWork::tc_ctas of this context's factorisations
  // look-ahead of large complex64 factorisations: a second stream, two events
  cudaStream_t stream_aux = nullptr;
  cudaEvent_t ev_u12 = nullptr, ev_far = nullptr;
};

namespace bem2d_gpu {

static int fail(bem2d_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CUDA_TRY(ctx, expr)                                                        \
  do {                                                                             \
    cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? BEM2D_ERR_NOMEM : BEM2D_ERR_CUDA, \
                  "%s: %s", #expr, cudaGetErrorString(e_));                        \
  } while (0)

#define CHECK_LAUNCH(ctx)                                                          \
  do {                                                                             \
    cudaError_t e_ = cudaGetLastError();                                           \
    if (e_ != cudaSuccess)                                                         \
      return fail(ctx, BEM2D_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

static void* ws(bem2d_ctx* c, const char* name, size_t bytes, int* rc) {
  Buffer& b = c->bufs[name];
  if (b.bytes >= bytes && b.ptr) return b.ptr;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  const size_t sz = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(&b.ptr, sz);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    *rc = fail(c, BEM2D_ERR_NOMEM, "cudaMalloc(%zu) for %s: %s", sz, name, cudaGetErrorString(e));
    return nullptr;
  }
  b.bytes = sz;
  return b.ptr;
}

// Event pair around one phase when timers are on; resolved after a sync.
static int tic(bem2d_ctx* c, int phase) {
  if (!c->timers) return -1;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, c->stream);
  c->pending.push_back(std::make_pair(phase, std::make_pair(a, b)));
  return (int)c->pending.size() - 1;
}
static void toc(bem2d_ctx* c, int id) {
  if (id >= 0) cudaEventRecord(c->pending[id].second.second, c->stream);
}
static void resolve_timers(bem2d_ctx* c) {
  for (auto& p : c->pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      c->phase_ms[p.first] += ms;
      c->phase_n[p.first] += 1;
    }
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  c->pending.clear();
  cudaGetLastError();
}

static bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// ---------------------------------------------------------------------------
// Gauss-Legendre rule on [0,1] by Newton iteration on P_n (nodes ascending,
// weights summing to 1): the rule Gauss() builds by Golub-Welsch
// (lib/bem2d_quadrature.cpp:10-56).
static void gauss01(int n, double* x, double* w) {
  if (n == 1) {
    x[0] = 0.5;
    w[0] = 1.0;
    return;
  }
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    // recompute the derivative at the converged node
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    const double wt = 1.0 / ((1.0 - z * z) * dp * dp);  // = (2/((1-z^2)P'^2)) / 2
    // z descends with i: node i from the right end, mirrored on the left
    x[n - 1 - i] = 0.5 * (1.0 + z);
    x[i] = 0.5 * (1.0 - z);
    w[n - 1 - i] = wt;
    w[i] = wt;
  }
}

// Gauss2D::Rescale (lib/bem2d_quadpoints.cpp:52-73) appended to `out`.
static void append_box(std::vector<double>& out, const std::vector<double>& gx,
                       const std::vector<double>& gw, double a, double b, double c,
                       double d) {
  const int N = (int)gx.size();
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      out.push_back(a + (b - a) * gx[i]);
      out.push_back(c + (d - c) * gx[j]);
      out.push_back((b - a) * (d - c) * (gw[i] * gw[j]));
    }
}

// AdaptedGauss1/2/3 (lib/bem2d_quadpoints.cpp:75-183).
static HostRules make_rules(int L, int N, double sigma) {
  HostRules r;
  r.gx.resize(N);
  r.gw.resize(N);
  gauss01(N, r.gx.data(), r.gw.data());
  std::vector<double> xl;
  for (int i = 0; i < L; ++i) xl.push_back(std::pow(sigma, L - i));
  xl.push_back(1.0);
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) append_box(r.r1, r.gx, r.gw, xl[i], xl[i + 1], xl[j], xl[j + 1]);
  {
    double a = sigma, b = 1;
    for (int l = L; l > 0; --l) {
      append_box(r.r2, r.gx, r.gw, 0, a, 1 - b, 1 - a);
      append_box(r.r2, r.gx, r.gw, a, b, 1 - b, 1 - a);
      append_box(r.r2, r.gx, r.gw, a, b, 1 - a, 1);
      a *= sigma;
      b *= sigma;
    }
  }
  {
    double a = 1, b = sigma;
    for (int l = L; l > 0; --l) {
      append_box(r.r3, r.gx, r.gw, 1 - a, 1 - b, 0, b);
      append_box(r.r3, r.gx, r.gw, 1 - a, 1 - b, b, a);
      append_box(r.r3, r.gx, r.gw, 1 - b, 1, b, a);
      a *= sigma;
      b *= sigma;
    }
  }
  return r;
}

// Distinct x and y values of a rule (exact equality: points of boxes that
// share an interval are computed by the same expression) and, per point,
// their indices packed as x | y << 16.
struct RuleIndex {
  std::vector<double> u, v;
  std::vector<int> k;
};

static RuleIndex index_rule(const std::vector<double>& r) {
  RuleIndex ri;
  std::map<double, int> mu, mv;
  for (size_t p = 0; p + 2 < r.size(); p += 3) {
    const auto a = mu.emplace(r[p], (int)mu.size());
    if (a.second) ri.u.push_back(r[p]);
    const auto b = mv.emplace(r[p + 1], (int)mv.size());
    if (b.second) ri.v.push_back(r[p + 1]);
    ri.k.push_back(a.first->second | (b.first->second << 16));
  }
  return ri;
}

static int get_rules(bem2d_ctx* c, const bem2d_quad* q, DevRules* out) {
  const RuleKey key{q->L, q->N, q->sigma};
  auto it = c->rules.find(key);
  if (it != c->rules.end()) {
    *out = it->second.second;
    return BEM2D_OK;
  }
  const HostRules h = make_rules(q->L, q->N, q->sigma);
  const RuleIndex i1 = index_rule(h.r1), i2 = index_rule(h.r2), i3 = index_rule(h.r3);
  // near-field geometry tables: one warp's must fit in shared memory
  const size_t cap = std::max(2 * i1.u.size(), std::max(i2.u.size(), i3.u.size())) +
                     std::max(i2.v.size(), i3.v.size());
  if (cap > 4096)
    return fail(c, BEM2D_ERR_ARG, "quadrature rule too large for the near-field kernel");
  std::vector<double> all;
  for (const std::vector<double>* v : {&h.gx, &h.gw, &h.r1, &h.r2, &h.r3, &i1.u, &i2.u, &i2.v,
                                       &i3.u, &i3.v})
    all.insert(all.end(), v->begin(), v->end());
  const size_t nd = all.size();
  const size_t nk = i1.k.size() + i2.k.size() + i3.k.size();
  void* d = nullptr;
  CUDA_TRY(c, cudaMalloc(&d, sizeof(double) * std::max<size_t>(nd, 1) + sizeof(int) * nk));
  CUDA_TRY(c, cudaMemcpy(d, all.data(), sizeof(double) * nd, cudaMemcpyHostToDevice));
  std::vector<int> keys;
  for (const RuleIndex* ri : {&i1, &i2, &i3}) keys.insert(keys.end(), ri->k.begin(), ri->k.end());
  int* dk = reinterpret_cast<int*>(static_cast<double*>(d) + nd);
  CUDA_TRY(c, cudaMemcpy(dk, keys.data(), sizeof(int) * nk, cudaMemcpyHostToDevice));
  const double* p = static_cast<const double*>(d);
  DevRules r;
  r.ng = q->N;
  r.gx = p;
  r.gw = p + q->N;
  r.r1 = p + 2 * q->N;
  r.n1 = (int)h.r1.size() / 3;
  r.r2 = r.r1 + h.r1.size();
  r.n2 = (int)h.r2.size() / 3;
  r.r3 = r.r2 + h.r2.size();
  r.n3 = (int)h.r3.size() / 3;
  r.u1 = r.r3 + h.r3.size();
  r.nu1 = (int)i1.u.size();
  r.u2 = r.u1 + i1.u.size();
  r.nu2 = (int)i2.u.size();
  r.v2 = r.u2 + i2.u.size();
  r.nv2 = (int)i2.v.size();
  r.u3 = r.v2 + i2.v.size();
  r.nu3 = (int)i3.u.size();
  r.v3 = r.u3 + i3.u.size();
  r.nv3 = (int)i3.v.size();
  r.k1 = dk;
  r.k2 = dk + i1.k.size();
  r.k3 = r.k2 + i2.k.size();
  c->rules[key] = std::make_pair(d, r);
  *out = r;
  return BEM2D_OK;
}

// ---------------------------------------------------------------------------
// Host-side validation, upload, near-pair list and node table of a geometry.
struct Staged {
  DevGeom g;
  DevRules r;
  NodeTable t;
  NodeTableFF tf;
  bool has_ff = false;
  NearPair* pairs;
  int npairs;
};

static int check_quad(bem2d_ctx* c, const bem2d_quad* q) {
  if (!q) return fail(c, BEM2D_ERR_ARG, "quad is NULL");
  if (q->N < 1 || q->N > 64) return fail(c, BEM2D_ERR_ARG, "QuadOption.N=%d out of [1,64]", q->N);
  if (q->L < 0 || q->L > 64) return fail(c, BEM2D_ERR_ARG, "QuadOption.L=%d out of [0,64]", q->L);
  if (q->L > 0 && !(q->sigma > 0.0 && q->sigma < 1.0))
    return fail(c, BEM2D_ERR_ARG, "QuadOption.sigma=%g not in (0,1)", q->sigma);
  return BEM2D_OK;
}

static int check_geom(bem2d_ctx* c, const bem2d_geometry* g) {
  if (!g) return fail(c, BEM2D_ERR_ARG, "geometry is NULL");
  if (g->n_elem < 1 || g->n_unk < 1)
    return fail(c, BEM2D_ERR_ARG, "empty geometry (n_elem=%d, n_unk=%d)", g->n_elem, g->n_unk);
  if (!g->kind || !g->param || !g->index || !g->next || !g->prev || !g->unk_elem ||
      !g->unk_kind || !g->unk_param)
    return fail(c, BEM2D_ERR_ARG, "geometry has a NULL table");
  for (int e = 0; e < g->n_elem; ++e)
    if (g->kind[e] < BEM2D_ELEM_SEGMENT || g->kind[e] > BEM2D_ELEM_INVELLIPSE)
      return fail(c, BEM2D_ERR_UNSUPPORTED, "element %d has unknown kind %d", e, g->kind[e]);
  for (int u = 0; u < g->n_unk; ++u) {
    if (g->unk_elem[u] < 0 || g->unk_elem[u] >= g->n_elem)
      return fail(c, BEM2D_ERR_ARG, "unknown %d refers to element %d", u, g->unk_elem[u]);
    if (g->unk_kind[u] == BEM2D_BASIS_POLY) {
      const double d = g->unk_param[u];
      if (!(d >= 0 && d <= 64 && d == std::floor(d)))
        return fail(c, BEM2D_ERR_ARG, "unknown %d: polynomial degree %g", u, d);
    } else if (g->unk_kind[u] != BEM2D_BASIS_LIN) {
      return fail(c, BEM2D_ERR_UNSUPPORTED, "unknown %d has basis kind %d", u, g->unk_kind[u]);
    }
  }
  return BEM2D_OK;
}

// Pairs that DiscreteKernel integrates with the graded rules
// (lib/bem2d_quadrature.h:271-282): same element index -> IntegrateIdent,
// else test next() == trial index -> AdaptedGauss3, else prev() -> AdaptedGauss2.
static std::vector<NearPair> near_pairs(const bem2d_geometry* g) {
  std::unordered_map<long long, std::vector<int>> by_index;
  for (int u = 0; u < g->n_unk; ++u) by_index[g->index[g->unk_elem[u]]].push_back(u);
  std::vector<NearPair> out;
  out.reserve((size_t)g->n_unk * 3);
  for (int i = 0; i < g->n_unk; ++i) {
    const int e = g->unk_elem[i];
    const long long keys[3] = {g->index[e], g->next[e], g->prev[e]};
    const int rules[3] = {RULE_SELF, RULE_G3, RULE_G2};
    for (int k = 0; k < 3; ++k) {
      if (k > 0 && keys[k] == keys[0]) continue;
      if (k == 2 && keys[2] == keys[1]) continue;
      auto it = by_index.find(keys[k]);
      if (it == by_index.end()) continue;
      for (int j : it->second) out.push_back(NearPair{i, j, rules[k], k == 0 ? 1 : 0});
    }
  }
  // Pair each (i, j, G3) with its reverse (j, i, G2) when that exists: one
  // warp then integrates both (the rules are mirror images), and the G2
  // entry leaves the list.
  std::unordered_map<long long, size_t> g2;
  auto key = [](int a, int b) { return ((long long)a << 32) | (unsigned)b; };
  for (size_t p = 0; p < out.size(); ++p)
    if (out[p].rule == RULE_G2) g2[key(out[p].i, out[p].j)] = p;
  std::vector<char> drop(out.size(), 0);
  for (auto& pr : out) {
    if (pr.rule != RULE_G3) continue;
    auto it = g2.find(key(pr.j, pr.i));
    if (it == g2.end() || drop[it->second]) continue;
    pr.rule = RULE_G3_PAIR;
    drop[it->second] = 1;
  }
  std::vector<NearPair> kept;
  kept.reserve(out.size());
  for (size_t p = 0; p < out.size(); ++p)
    if (!drop[p]) kept.push_back(out[p]);
  return kept;
}

static int stage(bem2d_ctx* c, const bem2d_geometry* g, const bem2d_quad* q, bool nodes,
                 bool pairs, Staged* st, bool ff_nodes = false) {
  int rc = check_geom(c, g);
  if (rc) return rc;
  if ((rc = check_quad(c, q))) return rc;
  if ((rc = get_rules(c, q, &st->r))) return rc;
  const int ne = g->n_elem, nu = g->n_unk;
  // pack the tables: doubles first (alignment), then 64-bit, then 32-bit
  const size_t b_param = sizeof(double) * 8 * ne, b_up = sizeof(double) * nu;
  const size_t b_links = sizeof(long long) * 3 * ne;
  const size_t b_ints = sizeof(int) * (ne + 2 * nu);
  const size_t total = b_param + b_up + b_links + b_ints;
  std::vector<char> h(total);
  char* p = h.data();
  memcpy(p, g->param, b_param);
  memcpy(p + b_param, g->unk_param, b_up);
  long long* lk = reinterpret_cast<long long*>(p + b_param + b_up);
  for (int e = 0; e < ne; ++e) {
    lk[e] = g->index[e];
    lk[ne + e] = g->next[e];
    lk[2 * ne + e] = g->prev[e];
  }
  int* ints = reinterpret_cast<int*>(p + b_param + b_up + b_links);
  memcpy(ints, g->kind, sizeof(int) * ne);
  memcpy(ints + ne, g->unk_elem, sizeof(int) * nu);
  memcpy(ints + ne + nu, g->unk_kind, sizeof(int) * nu);
  char* d = static_cast<char*>(ws(c, "geom", total, &rc));
  if (!d) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(d, h.data(), total, cudaMemcpyHostToDevice, c->stream));
  DevGeom& dg = st->g;
  dg.n_elem = ne;
  dg.n_unk = nu;
  dg.param = reinterpret_cast<const double*>(d);
  dg.unk_param = reinterpret_cast<const double*>(d + b_param);
  dg.index = reinterpret_cast<const long long*>(d + b_param + b_up);
  dg.next = dg.index + ne;
  dg.prev = dg.index + 2 * ne;
  const int* di = reinterpret_cast<const int*>(d + b_param + b_up + b_links);
  dg.kind = di;
  dg.unk_elem = di + ne;
  dg.unk_kind = di + ne + nu;
  st->pairs = nullptr;
  st->npairs = 0;
  if (pairs) {
    const std::vector<NearPair> np = near_pairs(g);
    st->npairs = (int)np.size();
    st->pairs = static_cast<NearPair*>(ws(c, "pairs", sizeof(NearPair) * np.size(), &rc));
    if (!st->pairs) return rc;
    if (!np.empty())
      CUDA_TRY(c, cudaMemcpyAsync(st->pairs, np.data(), sizeof(NearPair) * np.size(),
                                  cudaMemcpyHostToDevice, c->stream));
  }
  if (nodes) {
    const size_t nn = (size_t)nu * q->N;
    double* t = static_cast<double*>(ws(c, "nodes", sizeof(double) * 5 * nn, &rc));
    if (!t) return rc;
    st->t = NodeTable{t, t + nn, t + 2 * nn, t + 3 * nn, t + 4 * nn};
    st->has_ff = ff_nodes;
    if (ff_nodes) {
      // centres are double2: their offset is rounded up to 16 bytes (5 nn
      // float2 entries end on an 8-byte boundary when nn is odd)
      const size_t b_nodes = (sizeof(float2) * 5 * nn + 15) / 16 * 16;
      const size_t bytes = b_nodes + sizeof(double2) * nu + sizeof(float) * nu;
      char* f = static_cast<char*>(ws(c, "nodes_ff", bytes, &rc));
      if (!f) return rc;
      float2* f2 = reinterpret_cast<float2*>(f);
      double2* cen = reinterpret_cast<double2*>(f + b_nodes);
      st->tf = NodeTableFF{f2, f2 + nn, f2 + 2 * nn, f2 + 3 * nn, f2 + 4 * nn, cen,
                           reinterpret_cast<float*>(cen + nu)};
    }
    launch_node_table(dg, st->r, st->t, ff_nodes ? &st->tf : nullptr, c->stream);
    ++c->launches;
    CHECK_LAUNCH(c);
  }
  // the host table `h` must outlive the async copy
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

// Complex wavenumbers k_re + i k_im (the reference's AMOS branch) are
// accepted with Re k > 0 and arg k >= -pi/3, the domain of the
// complex-argument Hankel evaluator (hankel_c.cuh).
static int check_k(bem2d_ctx* c, double k_re, double k_im) {
  if (!std::isfinite(k_re) || !std::isfinite(k_im))
    return fail(c, BEM2D_ERR_ARG, "wavenumber is not finite");
  if (k_im != 0.0 && !(k_re > 0.0 && k_im >= -std::sqrt(3.0) * k_re))
    return fail(c, BEM2D_ERR_UNSUPPORTED,
                "complex wavenumber %g%+gi is outside Re k > 0, arg k >= -pi/3", k_re, k_im);
  return BEM2D_OK;
}

// Assemble beta*M + alpha*K into a device matrix (ld); ki != 0: complex
// wavenumber k + i ki.
static int assemble_dev(bem2d_ctx* c, const Staged& st, int kernel, double k, double eta,
                        double alpha, double beta, double2* A, long long ld, double ki = 0.0) {
  int t = tic(c, BEM2D_PHASE_FAR);
  if (ki != 0.0)
    launch_far_fp64_ck(st.g, st.t, st.r.ng, kernel, k, ki, eta, alpha, A, ld, c->stream);
  else
    launch_far_fp64(st.g, st.t, st.r.ng, kernel, k, eta, alpha, A, ld, c->stream);
  toc(c, t);
  ++c->launches;
  CHECK_LAUNCH(c);
  t = tic(c, BEM2D_PHASE_NEAR);
  if (ki != 0.0)
    launch_near_ck(st.g, st.r, st.pairs, st.npairs, kernel, k, ki, eta, alpha, beta, A, ld,
                   c->stream);
  else
    launch_near(st.g, st.r, st.pairs, st.npairs, kernel, k, eta, alpha, beta, A, ld, c->stream);
  toc(c, t);
  if (st.npairs) ++c->launches;
  CHECK_LAUNCH(c);
  return BEM2D_OK;
}

// Mixed assembly: Bessel functions in float-float throughout (far field,
// deferred and near-field entries; geometry and quadrature sums in FP64 for
// the near field), into a complex128 (A, ld) and a complex64 (A32, ld32)
// matrix.
static int assemble_mixed_dev(bem2d_ctx* c, const Staged& st, int kernel, double k, double eta,
                              double alpha, double beta, double2* A, long long ld, float2* A32,
                              long long ld32) {
  const long long n = st.g.n_unk;
  const unsigned cap = (unsigned)std::min<long long>(
      n * n, std::max<long long>(1 << 20, n * n / 8));
  int rc = 0;
  char* d = static_cast<char*>(ws(c, "defer", sizeof(int2) * (size_t)cap + 256, &rc));
  if (!d) return rc;
  DeferList dl;
  dl.count = reinterpret_cast<unsigned*>(d);
  dl.ij = reinterpret_cast<int2*>(d + 256);
  dl.capacity = cap;
  CUDA_TRY(c, cudaMemsetAsync(dl.count, 0, sizeof(unsigned), c->stream));
  int t = tic(c, BEM2D_PHASE_FAR);
  if (launch_far_ff(st.g, st.t, st.tf, st.r.ng, kernel, k, eta, alpha, A, ld, A32, ld32, dl,
                    c->stream) != BEM2D_OK)
    return fail(c, BEM2D_ERR_NOMEM, "device table for the far-field kernel");
  if (launch_deferred(st.tf, st.r.ng, kernel, k, eta, alpha, dl, A, ld, A32, ld32,
                      c->stream) != BEM2D_OK)
    return fail(c, BEM2D_ERR_NOMEM, "device table for the deferred far-field kernel");
  toc(c, t);
  c->launches += 2;
  CHECK_LAUNCH(c);
  t = tic(c, BEM2D_PHASE_NEAR);
  if (launch_near(st.g, st.r, st.pairs, st.npairs, kernel, k, eta, alpha, beta, A, ld,
                  c->stream, A32, ld32) != BEM2D_OK)
    return fail(c, BEM2D_ERR_NOMEM, "device table for the near-field kernel");
  toc(c, t);
  if (st.npairs) ++c->launches;
  CHECK_LAUNCH(c);
  return BEM2D_OK;
}

// Output helpers: run `fill` into a device matrix (the caller's, or a
// workspace one that is then copied to the caller's host memory).
template <typename F>
static int with_matrix_out(bem2d_ctx* c, void* out, long long ld, int n, F fill) {
  if (!out) return fail(c, BEM2D_ERR_ARG, "output pointer is NULL");
  if (ld < n) return fail(c, BEM2D_ERR_ARG, "leading dimension %lld < %d", ld, n);
  int rc = 0;
  if (is_device_ptr(out)) {
    if ((rc = fill(static_cast<double2*>(out), ld))) return rc;
  } else {
    double2* d = static_cast<double2*>(ws(c, "out", sizeof(double2) * (size_t)n * n, &rc));
    if (!d) return rc;
    if ((rc = fill(d, (long long)n))) return rc;
    CUDA_TRY(c, cudaMemcpy2DAsync(out, sizeof(double2) * ld, d, sizeof(double2) * n,
                                  sizeof(double2) * n, n, cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  resolve_timers(c);
  return BEM2D_OK;
}

// Non-finite guard of the assembly: nf_clear() before an assembly, nf_scan()
// of each output, nf_check() after a synchronisation of the stream.
static int* nf_flag(bem2d_ctx* c, int* rc) {
  return static_cast<int*>(ws(c, "nf_flag", 256, rc));
}
static int nf_clear(bem2d_ctx* c) {
  int rc = 0;
  int* f = nf_flag(c, &rc);
  if (!f) return rc;
  CUDA_TRY(c, cudaMemsetAsync(f, 0, sizeof(int), c->stream));
  return BEM2D_OK;
}
static int nf_scan(bem2d_ctx* c, const double2* A, long long ld, int rows, int cols) {
  int rc = 0;
  int* f = nf_flag(c, &rc);
  if (!f) return rc;
  launch_nonfinite_scan(A, ld, rows, cols, f, c->stream);
  ++c->launches;
  return BEM2D_OK;
}
static int nf_check(bem2d_ctx* c, const char* what) {
  int rc = 0;
  int* f = nf_flag(c, &rc);
  if (!f) return rc;
  int h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, f, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (h) return fail(c, BEM2D_ERR_NONFINITE, "non-finite entry in the assembled %s", what);
  return BEM2D_OK;
}

}  // namespace bem2d_gpu

using namespace bem2d_gpu;

extern "C" {

int bem2d_ctx_create(int device, bem2d_ctx** out) {
  if (!out) return BEM2D_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return BEM2D_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return BEM2D_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return BEM2D_ERR_CUDA;
  bem2d_ctx* c = new bem2d_ctx;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BEM2D_ERR_CUDA;
  }
  c->own_stream = true;
  *out = c;
  return BEM2D_OK;
}

void bem2d_ctx_destroy(bem2d_ctx* c) {
  if (!c) return;
  for (bem2d_ctx* w : c->workers) bem2d_ctx_destroy(w);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->stream_aux) cudaStreamSynchronize(c->stream_aux);
  for (auto& kv : c->bufs)
    if (kv.second.ptr) cudaFree(kv.second.ptr);
  for (auto& kv : c->rules) cudaFree(kv.second.first);
  if (c->stream_hi) {
    cudaStreamSynchronize(c->stream_hi);
    cudaStreamDestroy(c->stream_hi);
  }
  if (c->ev_asm) cudaEventDestroy(c->ev_asm);
  if (c->ev_sol) cudaEventDestroy(c->ev_sol);
  if (c->stream_aux) {
    cudaStreamSynchronize(c->stream_aux);
    cudaStreamDestroy(c->stream_aux);
  }
  if (c->ev_u12) cudaEventDestroy(c->ev_u12);
  if (c->ev_far) cudaEventDestroy(c->ev_far);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* bem2d_ctx_last_error(const bem2d_ctx* c) { return c ? c->err.c_str() : "no context"; }

void* bem2d_ctx_stream(bem2d_ctx* c) { return c ? (void*)c->stream : nullptr; }

int bem2d_ctx_set_stream(bem2d_ctx* c, void* stream) {
  if (!c) return BEM2D_ERR_ARG;
  if (c->own_stream && c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  c->stream = static_cast<cudaStream_t>(stream);
  c->own_stream = false;
  return BEM2D_OK;
}

int64_t bem2d_ctx_launch_count(const bem2d_ctx* c) { return c ? c->launches : 0; }

int bem2d_ctx_enable_timers(bem2d_ctx* c, int enable) {
  if (!c) return BEM2D_ERR_ARG;
  c->timers = enable != 0;
  for (int i = 0; i < 4; ++i) {
    c->phase_ms[i] = 0;
    c->phase_n[i] = 0;
  }
  return BEM2D_OK;
}

int bem2d_ctx_timer(const bem2d_ctx* c, int phase, double* ms, int64_t* count) {
  if (!c || phase < 0 || phase > 3) return BEM2D_ERR_ARG;
  if (ms) *ms = c->phase_ms[phase];
  if (count) *count = c->phase_n[phase];
  return BEM2D_OK;
}

int bem2d_gauss(int n, double* x, double* w) {
  if (n < 1 || !x || !w) return BEM2D_ERR_ARG;
  gauss01(n, x, w);
  return BEM2D_OK;
}

int bem2d_discrete_kernel(bem2d_ctx* c, const bem2d_geometry* geom, const bem2d_quad* quad,
                          int kernel, double k_re, double k_im, double eta, double alpha,
                          double beta, void* out, int64_t ld) {
  if (!c) return BEM2D_ERR_ARG;
  if (kernel < BEM2D_KERNEL_SINGLE || kernel > BEM2D_KERNEL_COMBINED)
    return fail(c, BEM2D_ERR_ARG, "unknown kernel %d", kernel);
  int rc = check_k(c, k_re, k_im);
  if (rc) return rc;
  cudaSetDevice(c->device);
  Staged st;
  if ((rc = stage(c, geom, quad, true, true, &st))) return rc;
  if ((rc = nf_clear(c))) return rc;
  rc = with_matrix_out(c, out, ld, geom->n_unk, [&](double2* A, long long lda) {
    int r = assemble_dev(c, st, kernel, k_re, eta, alpha, beta, A, lda, k_im);
    return r ? r : nf_scan(c, A, lda, geom->n_unk, geom->n_unk);
  });
  return rc ? rc : nf_check(c, "matrix");
}

int bem2d_discrete_kernel_mixed(bem2d_ctx* c, const bem2d_geometry* geom,
                                const bem2d_quad* quad, int kernel, double k_re, double k_im,
                                double eta, double alpha, double beta, void* out, int64_t ld,
                                void* out32, int64_t ld32) {
  if (!c) return BEM2D_ERR_ARG;
  if (kernel < BEM2D_KERNEL_SINGLE || kernel > BEM2D_KERNEL_COMBINED)
    return fail(c, BEM2D_ERR_ARG, "unknown kernel %d", kernel);
  int rc = check_k(c, k_re, k_im);
  if (rc) return rc;
  if (!(k_re > 0)) return fail(c, BEM2D_ERR_ARG, "mixed assembly needs k > 0");
  if (!out || !out32) return fail(c, BEM2D_ERR_ARG, "output pointer is NULL");
  cudaSetDevice(c->device);
  Staged st;
  if ((rc = stage(c, geom, quad, true, true, &st, true))) return rc;
  const int n = geom->n_unk;
  if (ld < n || ld32 < n) return fail(c, BEM2D_ERR_ARG, "leading dimension < %d", n);
  const bool d64 = is_device_ptr(out), d32 = is_device_ptr(out32);
  double2* A = d64 ? static_cast<double2*>(out)
                   : static_cast<double2*>(ws(c, "out", sizeof(double2) * (size_t)n * n, &rc));
  if (!A) return rc;
  float2* B = d32 ? static_cast<float2*>(out32)
                  : static_cast<float2*>(ws(c, "out32", sizeof(float2) * (size_t)n * n, &rc));
  if (!B) return rc;
  const long long la = d64 ? ld : n, lb = d32 ? ld32 : n;
  if ((rc = nf_clear(c))) return rc;
  if (k_im != 0.0) {
    // complex wavenumber: FP64 assembly (complex-argument Hankel functions),
    // then its complex64 rounding
    if ((rc = assemble_dev(c, st, kernel, k_re, eta, alpha, beta, A, la, k_im))) return rc;
    launch_to_c64(A, la, B, lb, n, n, c->stream);
    ++c->launches;
    CHECK_LAUNCH(c);
  } else if ((rc = assemble_mixed_dev(c, st, kernel, k_re, eta, alpha, beta, A, la, B, lb))) {
    return rc;
  }
  if ((rc = nf_scan(c, A, la, n, n))) return rc;
  if (!d64)
    CUDA_TRY(c, cudaMemcpy2DAsync(out, sizeof(double2) * ld, A, sizeof(double2) * n,
                                  sizeof(double2) * n, n, cudaMemcpyDeviceToHost, c->stream));
  if (!d32)
    CUDA_TRY(c, cudaMemcpy2DAsync(out32, sizeof(float2) * ld32, B, sizeof(float2) * n,
                                  sizeof(float2) * n, n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  resolve_timers(c);
  return nf_check(c, "matrix");
}

int bem2d_eval_ident(bem2d_ctx* c, const bem2d_geometry* geom, const bem2d_quad* quad,
                     void* out, int64_t ld) {
  if (!c) return BEM2D_ERR_ARG;
  cudaSetDevice(c->device);
  Staged st;
  int rc = stage(c, geom, quad, false, true, &st);
  if (rc) return rc;
  const int n = geom->n_unk;
  return with_matrix_out(c, out, ld, n, [&](double2* A, long long lda) {
    CUDA_TRY(c, cudaMemset2DAsync(A, sizeof(double2) * lda, 0, sizeof(double2) * n, n, c->stream));
    launch_ident(st.g, st.r, st.pairs, st.npairs, A, lda, c->stream);
    if (st.npairs) ++c->launches;
    CHECK_LAUNCH(c);
    return BEM2D_OK;
  });
}

int bem2d_dot_prod_basfuns(bem2d_ctx* c, const bem2d_geometry* geom, const bem2d_quad* quad,
                           int fun, double k_re, double k_im, double dir_x, double dir_y,
                           double eta, double scale, void* out) {
  if (!c) return BEM2D_ERR_ARG;
  if (fun < BEM2D_FUN_PLANEWAVE || fun > BEM2D_FUN_COMBINEDPLANEWAVE)
    return fail(c, BEM2D_ERR_ARG, "unknown functional %d", fun);
  if (!out) return fail(c, BEM2D_ERR_ARG, "output pointer is NULL");
  int rc = check_k(c, k_re, k_im);
  if (rc) return rc;
  cudaSetDevice(c->device);
  Staged st;
  if ((rc = stage(c, geom, quad, true, false, &st))) return rc;
  const int n = geom->n_unk;
  const bool dev = is_device_ptr(out);
  double2* b = dev ? static_cast<double2*>(out)
                   : static_cast<double2*>(ws(c, "rhs_out", sizeof(double2) * n, &rc));
  if (!b) return rc;
  launch_rhs(st.g, st.t, st.r.ng, fun, k_re, dir_x, dir_y, eta, scale, b, c->stream, k_im);
  ++c->launches;
  CHECK_LAUNCH(c);
  if (!dev)
    CUDA_TRY(c, cudaMemcpyAsync(out, b, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

}  // extern "C"

namespace bem2d_gpu {

// GMRES-based iterative refinement (GMRES-IR: Carson and Higham,
// "Accelerating the solution of linear systems by iterative refinement in
// three precisions", SIAM J. Sci. Comput. 40, 2018): the fallback of the
// mixed solve when plain refinement with the complex64 factor stalls or
// diverges (cond(A) times the factor's error above one).  Outer steps: r =
// b - A x in FP64; d from GMRES on M^{-1} A d = M^{-1} r, M = the complex64
// factor applied in FP64 arithmetic (left preconditioning), Arnoldi basis
// and Hessenberg matrix in FP64 (two Gram-Schmidt passes), restart length
// kGmresM, inner tolerance 1e-6 relative; x += d.  Stops at
// backward error tol, or when three outer steps in a row have not halved it
// (accepted if at most `accept`).  *solves counts the applications of the
// factor.  Converges in few steps when the factor's errors leave few
// outlying eigenvalues of M^{-1} A (a few near-singular directions).
static constexpr int kGmresM = 64;
static int gmres_ir(bem2d_ctx* c, int n, const double2* A, long long lda, const double2* b,
                    double2* x, const float2* LU, const LuWork& w, double normA, double normb,
                    double tol, double accept, double2* r, double2* part, double* red,
                    double* scal, bem2d_solve_info* rep, int* solves) {
  int rc = 0;
  const int m = std::min(n, kGmresM);
  double2* V = static_cast<double2*>(ws(c, "gm_V", sizeof(double2) * (size_t)n * (m + 1), &rc));
  double2* wv = static_cast<double2*>(ws(c, "gm_w", sizeof(double2) * n, &rc));
  double2* hd = static_cast<double2*>(ws(c, "gm_h", sizeof(double2) * (m + 2) * 2, &rc));
  double* nd = static_cast<double*>(ws(c, "gm_n", sizeof(double) * 4, &rc));
  double2* mvp = static_cast<double2*>(ws(c, "mv_part", mv_part_bytes(n), &rc));
  if (!V || !wv || !hd || !nd || !mvp) return rc;
  using cd = std::complex<double>;
  // out = M^{-1} v, the complex64 factor applied in FP64 arithmetic (GMRES
  // needs a fixed operator: complex64 arithmetic would perturb it by
  // cond(M) times single-precision roundoff)
  auto precond = [&](const double2* v, double2* out) -> int {
    int e = lu_solve_mixed(LU, n, n, w, v, out, c->stream, &c->launches);
    if (e) return fail(c, e, "triangular solve launch: %s", cudaGetErrorString(cudaGetLastError()));
    ++*solves;
    return BEM2D_OK;
  };
  auto host_norm = [&](const double2* v, double* out) -> int {
    launch_batched_norm2(n, v, n, nd, 1, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(out, nd, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *out = std::sqrt(*out);
    ++c->launches;
    return BEM2D_OK;
  };
  auto scale_into = [&](const double2* v, double f, double2* out) -> int {
    CUDA_TRY(c, cudaMemcpyAsync(nd + 2, &f, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    launch_batched_scale(n, v, n, nd + 2, out, n, 1, c->stream);
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // f is host memory
    ++c->launches;
    return BEM2D_OK;
  };
  double best = INFINITY;
  int stall = 0;
  for (int outer = 0; outer < 20; ++outer) {
    // residual and backward error
    launch_residual(A, lda, n, x, b, r, part, c->stream);
    launch_sumsq(r, n, n, 1, red, scal + 2, c->stream);
    launch_sumsq(x, n, n, 1, red, scal + 3, c->stream);
    c->launches += 6;
    double hs[2];
    CUDA_TRY(c, cudaMemcpyAsync(hs, scal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const double rnorm = std::sqrt(hs[0]), xnorm = std::sqrt(hs[1]);
    const double berr = rnorm / (normA * xnorm + normb);
    rep->residual = berr;
    if (!std::isfinite(berr)) return fail(c, BEM2D_ERR_NONFINITE, "non-finite residual in GMRES-IR");
    if (berr <= tol || rnorm == 0.0) return BEM2D_OK;
    if (berr < 0.5 * best) {
      best = berr;
      stall = 0;
    } else if (++stall >= 3) {
      if (berr <= accept) return BEM2D_OK;
      return fail(c, BEM2D_ERR_NOCONV, "GMRES-IR stalled at backward error %.3e", berr);
    }
    // v0 = M^{-1} r / beta
    if ((rc = precond(r, V))) return rc;
    double beta = 0;
    if ((rc = host_norm(V, &beta))) return rc;
    if (!(beta > 0) || !std::isfinite(beta))
      return fail(c, BEM2D_ERR_NONFINITE, "GMRES-IR: bad preconditioned residual");
    if ((rc = scale_into(V, 1.0 / beta, V))) return rc;
    std::vector<cd> H((size_t)(m + 1) * m, 0.0), g(m + 1, 0.0), cs(m), sn(m);
    g[0] = beta;
    int k = 0;
    for (int j = 0; j < m; ++j) {
      double2* vj = V + (size_t)j * n;
      double2* vn = V + (size_t)(j + 1) * n;
      launch_mv(A, lda, n, vj, wv, mvp, c->stream);
      c->launches += 2;
      if ((rc = precond(wv, vn))) return rc;
      std::vector<cd> h(j + 1, 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        launch_batched_dots(V, 0, n, j + 1, vn, 0, hd, 0, 1, c->stream);
        launch_batched_sub(V, 0, n, j + 1, vn, 0, hd, 0, 1, c->stream);
        std::vector<double2> hh(j + 1);
        CUDA_TRY(c, cudaMemcpyAsync(hh.data(), hd, sizeof(double2) * (j + 1),
                                    cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        for (int i = 0; i <= j; ++i) h[i] += cd(hh[i].x, hh[i].y);
        c->launches += 2;
      }
      double hn = 0;
      if ((rc = host_norm(vn, &hn))) return rc;
      for (int i = 0; i <= j; ++i) H[(size_t)j * (m + 1) + i] = h[i];
      H[(size_t)j * (m + 1) + j + 1] = hn;
      // previous rotations on column j, then a new one zeroing H(j+1, j)
      cd* col = &H[(size_t)j * (m + 1)];
      for (int i = 0; i < j; ++i) {
        const cd t = cs[i] * col[i] + sn[i] * col[i + 1];
        col[i + 1] = -std::conj(sn[i]) * col[i] + cs[i] * col[i + 1];
        col[i] = t;
      }
      const double a = std::abs(col[j]), bb = std::abs(col[j + 1]);
      const double rr = std::hypot(a, bb);
      if (rr == 0.0) {
        cs[j] = 1.0;
        sn[j] = 0.0;
      } else {
        const cd ph = a > 0 ? col[j] / a : cd(1.0, 0.0);
        cs[j] = a / rr;
        sn[j] = ph * std::conj(col[j + 1]) / rr;
        col[j] = ph * rr;
        col[j + 1] = 0.0;
      }
      g[j + 1] = -std::conj(sn[j]) * g[j];
      g[j] = cs[j] * g[j];
      k = j + 1;
      if (std::abs(g[j + 1]) <= 1e-6 * beta || !(hn > 1e-300 * beta)) break;
      if ((rc = scale_into(vn, 1.0 / hn, vn))) return rc;
    }
    // y = R^{-1} g (upper triangular k x k), d' = V y, x += (|r| / |A|) d'
    std::vector<cd> y(k);
    for (int i = k - 1; i >= 0; --i) {
      cd t = g[i];
      for (int l = i + 1; l < k; ++l) t -= H[(size_t)l * (m + 1) + i] * y[l];
      const cd dgl = H[(size_t)i * (m + 1) + i];
      y[i] = std::abs(dgl) > 0 ? t / dgl : cd(0.0, 0.0);
    }
    std::vector<double2> yd(k);
    for (int i = 0; i < k; ++i) yd[i] = make_double2(-y[i].real(), -y[i].imag());
    CUDA_TRY(c, cudaMemcpyAsync(hd, yd.data(), sizeof(double2) * k, cudaMemcpyHostToDevice,
                                c->stream));
    // x -= V (-f y)
    launch_batched_sub(V, 0, n, k, x, 0, hd, 0, 1, c->stream);
    ++c->launches;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // yd is host memory
    rep->iterations += k;
  }
  return fail(c, BEM2D_ERR_NOCONV, "GMRES-IR did not reach %.1e", tol);
}

// Look-ahead resources of a complex64 factorisation of order n (none below
// the order that uses outer blocks).
static int attach_lookahead(bem2d_ctx* c, LuWork& w, int n) {
  if (!lu_lookahead(n)) return BEM2D_OK;
  if (!c->stream_aux) {
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->stream_aux, cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_u12, cudaEventDisableTiming));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_far, cudaEventDisableTiming));
  }
  int rc = 0;
  w.pack2_bytes = lu_pack_bytes(n);
  w.pack2 = ws(c, "lu_pack2", w.pack2_bytes, &rc);
  if (!w.pack2) return rc;
  w.aux = c->stream_aux;
  w.ev_u12 = c->ev_u12;
  w.ev_far = c->ev_far;
  w.aux_ctas = lu_lookahead_ctas();
  return BEM2D_OK;
}

// Solve with device-resident A (lda) and b; x written to device memory.
// A32pre: a complex64 copy of A already in the "lu32" workspace (mixed
// assembly writes it); otherwise A is converted here.
static int solve_dev(bem2d_ctx* c, int n, const double2* A, long long lda, const double2* b,
                     double2* x, int precision, double tol, bem2d_solve_info* info,
                     bool a32_ready = false) {
  int rc = 0;
  bem2d_solve_info rep{0, 0, 0.0};
  LuWork w;
  w.min_rows = c->panel_min_rows;
  w.tc_ctas = c->tc_ctas;
  if (precision == BEM2D_PREC_MIXED_TF32) {
    w.tc_passes = 1;
    precision = BEM2D_PREC_MIXED;
  }
  // ints: [0] info [1] status [8, 8+n) ipiv
  int* ints = static_cast<int*>(ws(c, "lu_ints", sizeof(int) * (n + 8), &rc));
  if (!ints) return rc;
  w.ipiv = ints + 8;
  w.info = ints;
  w.status = ints + 1;
  w.scratch_bytes = lu_scratch_bytes(n);
  w.scratch = ws(c, "lu_scratch", w.scratch_bytes, &rc);
  if (!w.scratch) return rc;
  char* aux = static_cast<char*>(
      ws(c, "lu_aux", lu_aux_bytes(n, precision == BEM2D_PREC_FP64 ? sizeof(double2)
                                                                  : sizeof(float2)), &rc));
  if (!aux) return rc;
  w.dinv = aux;
  w.perm = reinterpret_cast<int*>(aux + (lu_aux_bytes(n, precision == BEM2D_PREC_FP64
                                                             ? sizeof(double2)
                                                             : sizeof(float2)) -
                                         256 - sizeof(int) * (size_t)n));
  int hinfo[2] = {0, 0};
  if (precision == BEM2D_PREC_FP64) {
    double2* LU = static_cast<double2*>(ws(c, "lu64", sizeof(double2) * (size_t)n * n, &rc));
    if (!LU) return rc;
    CUDA_TRY(c, cudaMemcpy2DAsync(LU, sizeof(double2) * n, A, sizeof(double2) * lda,
                                  sizeof(double2) * n, n, cudaMemcpyDeviceToDevice, c->stream));
    int t = tic(c, BEM2D_PHASE_LU);
    if ((rc = lu_factor<double2>(LU, n, n, w, c->stream, &c->launches)))
      return fail(c, rc, "LU launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    toc(c, t);
    CHECK_LAUNCH(c);
    CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "LU panel barrier timed out");
    rep.info = hinfo[0];
    if (info) *info = rep;
    if (hinfo[0]) return fail(c, hinfo[0], "zero pivot at column %d", hinfo[0]);
    t = tic(c, BEM2D_PHASE_SOLVE);
    if ((rc = lu_solve<double2>(LU, n, n, w, b, x, c->stream, &c->launches)))
      return fail(c, rc, "triangular solve launch: %s", cudaGetErrorString(cudaGetLastError()));
    toc(c, t);
    CHECK_LAUNCH(c);
    CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "triangular solve wait timed out");
    resolve_timers(c);
    return BEM2D_OK;
  }
  if (precision != BEM2D_PREC_MIXED) return fail(c, BEM2D_ERR_ARG, "unknown precision %d", precision);
  // Refine to backward error `tol` (default 1e-14, a few units of FP64
  // roundoff); if progress stalls first, accept anything at or below 1e-12.
  if (!(tol > 0)) tol = 1e-14;
  const double accept = std::max(tol, 1e-12);
  float2* LU = static_cast<float2*>(ws(c, "lu32", sizeof(float2) * (size_t)n * n, &rc));
  if (!LU) return rc;
  w.pack_bytes = lu_pack_bytes(n);
  w.pack = ws(c, "lu_pack", w.pack_bytes, &rc);
  if (w.pack && (rc = attach_lookahead(c, w, n))) return rc;
  if (!w.pack) return rc;
  double2* r = static_cast<double2*>(ws(c, "ir_r", sizeof(double2) * n, &rc));
  float2* d = static_cast<float2*>(ws(c, "ir_d", sizeof(float2) * n, &rc));
  double2* part = static_cast<double2*>(ws(c, "ir_part", residual_part_bytes(n), &rc));
  double* red = static_cast<double*>(ws(c, "ir_red", sumsq_part_bytes() + 64, &rc));
  if (!r || !d || !part || !red) return rc;
  double* scal = red + sumsq_part_bytes() / sizeof(double);  // [0] |A|^2 [1] |b|^2 [2] |r|^2 [3] |x|^2
  if (!a32_ready) {
    launch_to_c64(A, lda, LU, n, n, n, c->stream);
    ++c->launches;
  }
  launch_sumsq(A, lda, n, n, red, scal, c->stream);
  launch_sumsq(b, n, n, 1, red, scal + 1, c->stream);
  c->launches += 4;
  int tl = tic(c, BEM2D_PHASE_LU);
  if ((rc = lu_factor<float2>(LU, n, n, w, c->stream, &c->launches)))
    return fail(c, rc, "LU launch failed: %s", cudaGetErrorString(cudaGetLastError()));
  toc(c, tl);
  CHECK_LAUNCH(c);
  double hs[4];
  CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(hs, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "LU panel barrier timed out");
  rep.info = hinfo[0];
  if (hinfo[0]) {
    if (info) *info = rep;
    return fail(c, hinfo[0], "zero pivot at column %d (complex64 factor)", hinfo[0]);
  }
  const double normA = std::sqrt(hs[0]), normb = std::sqrt(hs[1]);
  // x0 = 0, r0 = b
  CUDA_TRY(c, cudaMemsetAsync(x, 0, sizeof(double2) * n, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c->stream));
  double rnorm = normb, xnorm = 0.0, best = INFINITY;
  int stall = 0;
  const int max_it = 30;
  for (int it = 0;; ++it) {
    const double berr = rnorm / (normA * xnorm + normb);
    rep.residual = berr;
    rep.iterations = it;
    if (!std::isfinite(berr)) {
      if (info) *info = rep;
      return fail(c, BEM2D_ERR_NONFINITE, "non-finite residual in refinement");
    }
    if (berr <= tol || rnorm == 0.0) break;
    bool fallback = false;
    if (berr < 0.5 * best) {
      best = berr;
      stall = 0;
    } else if (++stall >= 2) {
      if (berr <= accept) break;
      fallback = true;
    }
    if (it >= max_it) {
      if (berr <= accept) break;
      fallback = true;
    }
    if (fallback) {
      // plain refinement cannot converge with this factor: GMRES-IR, from
      // x = 0 if the iterates have grown away from the solution
      if (berr > 1e-2) CUDA_TRY(c, cudaMemsetAsync(x, 0, sizeof(double2) * n, c->stream));
      int solves = 0;
      const int ts = tic(c, BEM2D_PHASE_SOLVE);
      rc = gmres_ir(c, n, A, lda, b, x, LU, w, normA, normb, tol, accept, r, part, red, scal,
                    &rep, &solves);
      toc(c, ts);
      rep.iterations = it + solves;
      if (info) *info = rep;
      if (rc) return rc;
      break;
    }
    // d = LU32^{-1} (r / |r|);  x += |r| d;  r = b - A x
    const int ts = tic(c, BEM2D_PHASE_SOLVE);
    launch_scale_to_c64(n, r, 1.0 / rnorm, d, c->stream);
    if ((rc = lu_solve<float2>(LU, n, n, w, d, d, c->stream, &c->launches)))
      return fail(c, rc, "triangular solve launch: %s", cudaGetErrorString(cudaGetLastError()));
    launch_axpy_c64(n, rnorm, d, x, c->stream);
    launch_residual(A, lda, n, x, b, r, part, c->stream);
    launch_sumsq(r, n, n, 1, red, scal + 2, c->stream);
    launch_sumsq(x, n, n, 1, red, scal + 3, c->stream);
    toc(c, ts);
    c->launches += 8;
    CHECK_LAUNCH(c);
    CUDA_TRY(c, cudaMemcpyAsync(hs, scal, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "triangular solve wait timed out");
    rnorm = std::sqrt(hs[2]);
    xnorm = std::sqrt(hs[3]);
  }
  resolve_timers(c);
  if (info) *info = rep;
  return BEM2D_OK;
}

// Copy host data to a workspace buffer unless it is already on the device.
static const double2* dev_in(bem2d_ctx* c, const void* p, size_t rows, size_t cols, long long ld,
                             const char* name, long long* ld_out, int* rc) {
  if (is_device_ptr(p)) {
    *ld_out = ld;
    return static_cast<const double2*>(p);
  }
  double2* d = static_cast<double2*>(ws(c, name, sizeof(double2) * rows * cols, rc));
  if (!d) return nullptr;
  cudaError_t e = cudaMemcpy2DAsync(d, sizeof(double2) * rows, p, sizeof(double2) * ld,
                                    sizeof(double2) * rows, cols, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    *rc = fail(c, BEM2D_ERR_CUDA, "host-to-device copy: %s", cudaGetErrorString(e));
    return nullptr;
  }
  *ld_out = (long long)rows;
  return d;
}

}  // namespace bem2d_gpu

extern "C" {

int bem2d_solve_system(bem2d_ctx* c, int n, const void* A, int64_t lda, const void* b, void* x,
                       int precision, double tol, bem2d_solve_info* info) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !b || !x) return fail(c, BEM2D_ERR_ARG, "bad arguments (n=%d)", n);
  if (lda < n) return fail(c, BEM2D_ERR_ARG, "lda %lld < n %d", (long long)lda, n);
  cudaSetDevice(c->device);
  int rc = 0;
  long long ldA = 0, ldb = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "in_A", &ldA, &rc);
  if (!dA) return rc;
  const double2* db = dev_in(c, b, n, 1, n, "in_b", &ldb, &rc);
  if (!db) return rc;
  const bool xdev = is_device_ptr(x);
  double2* dx = xdev ? static_cast<double2*>(x)
                     : static_cast<double2*>(ws(c, "out_x", sizeof(double2) * n, &rc));
  if (!dx) return rc;
  rc = solve_dev(c, n, dA, ldA, db, dx, precision, tol, info);
  if (rc) return rc;
  if (!xdev) {
    CUDA_TRY(c, cudaMemcpyAsync(x, dx, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  return BEM2D_OK;
}

// Switches c->stream to c->stream_hi (if the context has one) after the
// work queued so far, and back on end() or destruction; the low stream then
// waits for everything queued on the high one.
struct PhaseStream {
  bem2d_ctx* c;
  cudaStream_t lo = nullptr;
  explicit PhaseStream(bem2d_ctx* ctx) : c(ctx) {}
  int begin() {
    if (!c->stream_hi) return BEM2D_OK;
    CUDA_TRY(c, cudaEventRecord(c->ev_asm, c->stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream_hi, c->ev_asm, 0));
    lo = c->stream;
    c->stream = c->stream_hi;
    return BEM2D_OK;
  }
  int end() {
    if (!lo) return BEM2D_OK;
    c->stream = lo;
    lo = nullptr;
    CUDA_TRY(c, cudaEventRecord(c->ev_sol, c->stream_hi));
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_sol, 0));
    return BEM2D_OK;
  }
  ~PhaseStream() { end(); }
};

int bem2d_scattering_solve(bem2d_ctx* c, const bem2d_geometry* geom, const bem2d_quad* quad,
                           double k_re, double k_im, double eta, double dir_x, double dir_y,
                           int precision, double tol, void* x, bem2d_solve_info* info) {
  if (!c) return BEM2D_ERR_ARG;
  if (!x) return fail(c, BEM2D_ERR_ARG, "output pointer is NULL");
  int rc = check_k(c, k_re, k_im);
  if (rc) return rc;
  cudaSetDevice(c->device);
  Staged st;
  const bool mixed = precision == BEM2D_PREC_MIXED || precision == BEM2D_PREC_MIXED_TF32;
  if ((rc = stage(c, geom, quad, true, true, &st, mixed))) return rc;
  const int n = geom->n_unk;
  double2* A = static_cast<double2*>(ws(c, "sys_A", sizeof(double2) * (size_t)n * n, &rc));
  if (!A) return rc;
  double2* b = static_cast<double2*>(ws(c, "sys_b", sizeof(double2) * n, &rc));
  if (!b) return rc;
  // complex wavenumbers: FP64 assembly; the mixed solver converts A itself
  const bool mixed_asm = mixed && k_im == 0.0;
  if ((rc = nf_clear(c))) return rc;
  if (mixed_asm) {
    float2* A32 = static_cast<float2*>(ws(c, "lu32", sizeof(float2) * (size_t)n * n, &rc));
    if (!A32) return rc;
    if ((rc = assemble_mixed_dev(c, st, BEM2D_KERNEL_COMBINED, k_re, eta, 2.0, 1.0, A, n, A32, n)))
      return rc;
  } else if ((rc = assemble_dev(c, st, BEM2D_KERNEL_COMBINED, k_re, eta, 2.0, 1.0, A, n, k_im))) {
    return rc;
  }
  launch_rhs(st.g, st.t, st.r.ng, BEM2D_FUN_COMBINEDPLANEWAVE, k_re, dir_x, dir_y, eta, 2.0, b,
             c->stream, k_im);
  ++c->launches;
  CHECK_LAUNCH(c);
  // NaN or Inf in A or b (a degenerate element, say) would otherwise reach
  // the caller as a zero pivot or a non-finite solution
  if ((rc = nf_scan(c, A, n, n, n)) || (rc = nf_scan(c, b, n, n, 1))) return rc;
  const bool xdev = is_device_ptr(x);
  double2* dx = xdev ? static_cast<double2*>(x)
                     : static_cast<double2*>(ws(c, "out_x", sizeof(double2) * n, &rc));
  if (!dx) return rc;
  // Sweep workers factor and solve on their high-priority stream, so that
  // these latency-bound chains get SM slots ahead of other workers'
  // assembly grids; the next call's assembly waits for this phase.
  PhaseStream ps(c);
  if ((rc = ps.begin())) return rc;
  if ((rc = solve_dev(c, n, A, n, b, dx, precision, tol, info, mixed_asm))) {
    const int nf = nf_check(c, "matrix or right-hand side");
    return nf ? nf : rc;
  }
  if ((rc = nf_check(c, "matrix or right-hand side"))) return rc;
  if (!xdev) {
    CUDA_TRY(c, cudaMemcpyAsync(x, dx, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  return ps.end();
}

}  // extern "C"

// ===========================================================================
// Norms, change of basis, numerical range, potentials
// ===========================================================================
namespace bem2d_gpu {

static double2* dev_out(bem2d_ctx* c, void* p, size_t elems, const char* name, int* rc) {
  if (is_device_ptr(p)) return static_cast<double2*>(p);
  return static_cast<double2*>(ws(c, name, sizeof(double2) * elems, rc));
}

// Deterministic start vector of unit norm (the same on every run).
static std::vector<std::complex<double>> start_vector(int n) {
  std::vector<std::complex<double>> v(n);
  unsigned long long s = 0x9E3779B97F4A7C15ull;
  double nrm = 0;
  for (int i = 0; i < n; ++i) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    const double a = ((s >> 11) & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0) - 0.5;
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    const double b = ((s >> 11) & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0) - 0.5;
    v[i] = std::complex<double>(a + 1.0, b);
    nrm += std::norm(v[i]);
  }
  nrm = std::sqrt(nrm);
  for (auto& x : v) x /= nrm;
  return v;
}

template <typename T>
struct LzNames;
template <>
struct LzNames<double2> {
  static constexpr const char* Q = "nr_Q";
  static constexpr const char* Y1 = "nr_Y1";
  static constexpr const char* Y2 = "nr_Y2";
  static constexpr const char* W = "nr_W";
  static constexpr const char* h = "nr_h";
  static constexpr const char* sc = "nr_sc";
  static constexpr const char* Q2 = "nr_Q2";
  static constexpr const char* W2 = "nr_W2";
  static constexpr const char* Z = "nr_Z";
};
template <>
struct LzNames<float2> {
  static constexpr const char* Q = "nr32_Q";
  static constexpr const char* Y1 = "nr32_Y1";
  static constexpr const char* Y2 = "nr32_Y2";
  static constexpr const char* W = "nr32_W";
  static constexpr const char* h = "nr32_h";
  static constexpr const char* sc = "nr32_sc";
  static constexpr const char* Q2 = "nr32_Q2";
  static constexpr const char* W2 = "nr32_W2";
  static constexpr const char* Z = "nr32_Z";
};

// Batched Lanczos (full reorthogonalisation, two Gram-Schmidt passes) for
// lambda_max of H_a = (e^{i th_a} A + e^{-i th_a} A^H) / 2, every angle at
// once: one product with A and one with A^H per step for all angles.  An
// angle has converged when its lambda_max moved by at most tol (relative)
// in two consecutive steps.  start (complex128, n per angle): start vectors
// (normalised here); else the deterministic start vector.  ritz (optional):
// the Ritz vector of lambda_max per angle on return.
template <typename T>
static int numrange_lanczos(bem2d_ctx* c, int n, const T* dA, long long la, int nang,
                            const double* dth, double tol, int mmax, const double2* start,
                            double* lam_out, T* ritz, bool full_reorth = true,
                            double rtol = 0.0, double etol = 0.0,
                            const double* gap_in = nullptr, double* gap_out = nullptr,
                            const float2* ffhi = nullptr, const float2* fflo = nullptr) {
  int rc = 0;
  const long long qs = (long long)n * (mmax + 1);  // per-angle basis stride
  T* Q = static_cast<T*>(ws(c, LzNames<T>::Q, sizeof(T) * (size_t)qs * nang, &rc));
  T* Y1 = static_cast<T*>(ws(c, LzNames<T>::Y1, sizeof(T) * (size_t)n * nang, &rc));
  T* Y2 = static_cast<T*>(ws(c, LzNames<T>::Y2, sizeof(T) * (size_t)n * nang, &rc));
  T* W = static_cast<T*>(ws(c, LzNames<T>::W, sizeof(T) * (size_t)n * nang, &rc));
  T* h = static_cast<T*>(ws(c, LzNames<T>::h, sizeof(T) * (size_t)(mmax + 2) * nang, &rc));
  double* sc = static_cast<double*>(ws(c, LzNames<T>::sc, sizeof(double) * 2 * nang + 64, &rc));
  if (!Q || !Y1 || !Y2 || !W || !h || !sc) return rc;
  std::vector<double> nn(nang), inv(nang);
  if (start) {
    if constexpr (sizeof(T) == sizeof(double2)) {
      launch_batched_norm2(n, start, n, sc, nang, c->stream);
      CUDA_TRY(c, cudaMemcpyAsync(nn.data(), sc, sizeof(double) * nang, cudaMemcpyDeviceToHost, c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      for (int a = 0; a < nang; ++a) inv[a] = nn[a] > 0 ? 1.0 / std::sqrt(nn[a]) : 0.0;
      CUDA_TRY(c, cudaMemcpyAsync(sc, inv.data(), sizeof(double) * nang, cudaMemcpyHostToDevice, c->stream));
      launch_batched_scale(n, start, n, sc, Q, qs, nang, c->stream);
      c->launches += 2;
    } else {
      return fail(c, BEM2D_ERR_ARG, "start vectors are complex128");
    }
  } else {
    const std::vector<std::complex<double>> v0 = start_vector(n);
    std::vector<T> v0t(n);
    for (int r = 0; r < n; ++r) v0t[r] = {(decltype(v0t[r].x))v0[r].real(), (decltype(v0t[r].x))v0[r].imag()};
    for (int a = 0; a < nang; ++a)
      CUDA_TRY(c, cudaMemcpyAsync(Q + (size_t)a * qs, v0t.data(), sizeof(T) * n,
                                  cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // v0t is released below
  }
  std::vector<std::vector<double>> al(nang), be(nang);
  std::vector<double> lam(nang, 0.0), prev(nang, NAN), dlam(nang, 0.0);
  std::vector<int> stable(nang, 0);
  std::vector<T> hh((size_t)(mmax + 2) * nang);
  const int ldh = mmax + 2;
  int steps = 0;
  // Deflation: an angle whose value has converged leaves the batch (its
  // Ritz vector, if wanted, is formed on the way out), and the others are
  // gathered to the front slots (basis and next vector, into a second
  // buffer), so later steps cost in proportion to the angles still
  // iterating.  slot_angle[s]: the angle of slot s; na: slots in use.
  std::vector<int> slot_angle(nang);
  for (int a = 0; a < nang; ++a) slot_angle[a] = a;
  int na = nang;
  T* Qalt = static_cast<T*>(ws(c, LzNames<T>::Q2, sizeof(T) * (size_t)qs * nang, &rc));
  T* Walt = static_cast<T*>(ws(c, LzNames<T>::W2, sizeof(T) * (size_t)n * nang, &rc));
  int* dmap = static_cast<int*>(ws(c, "nr_map", sizeof(int) * 2 * nang, &rc));
  double* dthc = static_cast<double*>(ws(c, "nr_thc", sizeof(double) * nang, &rc));
  if (!Qalt || !Walt || !dmap || !dthc) return rc;
  // K-split partials of the products: the most any batch width needs
  size_t zwork_bytes = 0;
  for (int m = 1; m <= nang; ++m) zwork_bytes = std::max(zwork_bytes, zgemm_work_bytes(n, m, sizeof(T)));
  void* zwork = zwork_bytes ? ws(c, LzNames<T>::Z, zwork_bytes, &rc) : nullptr;
  if (zwork_bytes && !zwork) return rc;
  float2* ffb = nullptr;  // B's float-float split for the products
  if (ffhi) {
    ffb = static_cast<float2*>(ws(c, "nr_ffb", 2 * sizeof(float2) * (size_t)n * nang, &rc));
    if (!ffb) return rc;
  }
  std::vector<double> th_h(nang);
  CUDA_TRY(c, cudaMemcpyAsync(th_h.data(), dth, sizeof(double) * nang, cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dthc, dth, sizeof(double) * nang, cudaMemcpyDeviceToDevice,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const double* theta = dthc;
  // Ritz vectors u = Q_s y_s of slots sl (y the unit eigenvector of T_s for
  // lambda_max, st steps) into ritz[angle]: the slots' bases gathered to
  // Qalt, W' = 0 - Qalt (-y), scattered to the angles' columns
  auto emit_ritz = [&](const std::vector<int>& sl, int st) -> int {
    const int m = (int)sl.size();
    if (!ritz || m == 0) return BEM2D_OK;
    std::vector<int> ang(m);
    for (int i = 0; i < m; ++i) {
      const int a = sl[i];
      std::vector<double> e(be[a].begin(), be[a].begin() + (st - 1));
      const std::vector<double> sv = tridiag_eigenvector(al[a], e, lam[a]);
      if (gap_out)
        gap_out[slot_angle[a]] =
            st > 1 ? lam[a] - tridiag_kth_largest(al[a], e, 2, 1e-6) : 0.0;
      for (int r = 0; r < st; ++r)
        hh[(size_t)i * ldh + r] = {(decltype(hh[0].x))(-sv[r]), (decltype(hh[0].x))0};
      ang[i] = slot_angle[a];
    }
    CUDA_TRY(c, cudaMemcpyAsync(h, hh.data(), sizeof(T) * (size_t)ldh * m, cudaMemcpyHostToDevice,
                                c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(dmap, sl.data(), sizeof(int) * m, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(dmap + nang, ang.data(), sizeof(int) * m, cudaMemcpyHostToDevice,
                                c->stream));
    launch_gather_slots(Q, qs, Qalt, qs, (long long)st * n, dmap, m, c->stream);
    CUDA_TRY(c, cudaMemsetAsync(Walt, 0, sizeof(T) * (size_t)n * m, c->stream));
    launch_batched_sub(Qalt, qs, n, st, Walt, n, h, ldh, m, c->stream);
    launch_scatter_slots(Walt, (long long)n, ritz, (long long)n, (long long)n, dmap + nang, m,
                         c->stream);
    c->launches += 3;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // hh, sl, ang are host memory
    return BEM2D_OK;
  };
  for (int j = 0; j < mmax; ++j) {
    const T* Qj = Q + (size_t)j * n;
    if constexpr (sizeof(T) == sizeof(double2)) {
      if (ffhi) {  // the products in float-float on the FP32 pipe
        launch_zgemm_ff(false, ffhi, fflo, n, Qj, qs, na, Y1, n, zwork, zwork_bytes, ffb,
                        c->stream);
        launch_zgemm_ff(true, ffhi, fflo, n, Qj, qs, na, Y2, n, zwork, zwork_bytes, ffb,
                        c->stream);
      } else {
        launch_zgemm(false, dA, la, n, Qj, qs, na, Y1, n, zwork, zwork_bytes, c->stream);
        launch_zgemm(true, dA, la, n, Qj, qs, na, Y2, n, zwork, zwork_bytes, c->stream);
      }
    } else {
      launch_zgemm(false, dA, la, n, Qj, qs, na, Y1, n, zwork, zwork_bytes, c->stream);
      launch_zgemm(true, dA, la, n, Qj, qs, na, Y2, n, zwork, zwork_bytes, c->stream);
    }
    launch_herm_combine(n, Y1, Y2, n, theta, W, n, na, c->stream);
    // Gram-Schmidt (two passes) against q_0..q_j, or, without full
    // reorthogonalisation, against q_{j-1}, q_j only (the three-term
    // recurrence: the extreme Ritz value converges all the same)
    const int w0 = full_reorth ? 0 : std::max(0, j - 1), nw = j + 1 - w0;
    const T* Qw = Q + (size_t)w0 * n;
    launch_batched_dots(Qw, qs, n, nw, W, n, h, ldh, na, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(hh.data(), h, sizeof(T) * (size_t)ldh * na, cudaMemcpyDeviceToHost, c->stream));
    launch_batched_sub(Qw, qs, n, nw, W, n, h, ldh, na, c->stream);
    launch_batched_dots(Qw, qs, n, nw, W, n, h, ldh, na, c->stream);
    launch_batched_sub(Qw, qs, n, nw, W, n, h, ldh, na, c->stream);
    launch_batched_norm2(n, W, n, sc, na, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(nn.data(), sc, sizeof(double) * na, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->launches += 8;
    CHECK_LAUNCH(c);
    steps = j + 1;
    for (int a = 0; a < na; ++a) {
      al[a].push_back(hh[(size_t)a * ldh + (j - w0)].x);
      const double b = std::sqrt(nn[a]);
      inv[a] = b > 1e-300 ? 1.0 / b : 0.0;
      // Ritz values interlace: the previous value bounds the new one below.
      // The value is resolved to 1e-4 of its last change (to roundoff once
      // it has settled), which is all the convergence tests need.
      {
        const double lp = lam[a];
        lam[a] = j == 0 ? al[a][0]
                        : tridiag_lmax_from(al[a], be[a], lp, 2.0 * dlam[a], 1e-4 * dlam[a]);
        dlam[a] = j == 0 ? std::fabs(lam[a]) : std::fabs(lam[a] - lp);
      }
      const double scale = std::max(std::fabs(lam[a]), 1e-300);
      if (rtol > 0 || etol > 0) {
        // Ritz-pair criteria, relative to the size of H seen so far
        // (hs = max |lambda|, |alpha_i|, beta_i), with r = beta_{j+1} |s_j|
        // the residual estimate (s the unit eigenvector of T for
        // lambda_max), computed once the value has settled to 1e-5:
        //  rtol: r <= rtol hs (the Ritz vector has converged);
        //  etol: the value has moved by at most etol hs in this step and
        //        the error estimate min(r, r^2 / (theta_1 - theta_2)) is at
        //        most etol hs (for Hermitian H an eigenvalue lies within r
        //        of the Ritz value, within r^2 / gap for an isolated one).
        bool conv = b <= 1e-300;
        const bool warm = gap_in != nullptr;
        if (!conv && (warm || (j >= 3 && std::fabs(lam[a] - prev[a]) <= 1e-5 * scale))) {
          double hs = scale;
          for (const double v : al[a]) hs = std::max(hs, std::fabs(v));
          for (const double v : be[a]) hs = std::max(hs, v);
          const std::vector<double> sv = tridiag_eigenvector(al[a], be[a], lam[a]);
          const double r = b * std::fabs(sv[j]);
          if (rtol > 0) {
            conv = r <= rtol * hs;
          } else if (warm || std::fabs(lam[a] - prev[a]) <= etol * hs) {
            // gap to the rest of the spectrum: the smaller of the warm
            // start's estimate and this tridiagonal's theta_1 - theta_2
            double gap = warm ? gap_in[slot_angle[a]] : INFINITY;
            if (j >= 1) gap = std::min(gap, lam[a] - tridiag_kth_largest(al[a], be[a], 2, 1e-6));
            conv = std::min(r, gap > 0 ? r * r / gap : r) <= etol * hs;
          }
        }
        stable[a] = conv ? 2 : 0;
      } else if (std::fabs(lam[a] - prev[a]) <= tol * scale || b <= 1e-300) {
        ++stable[a];
      } else {
        stable[a] = 0;
      }
      prev[a] = lam[a];
      be[a].push_back(b);
    }
    {
      std::vector<int> keep, done;
      keep.reserve(na);
      for (int a = 0; a < na; ++a) {
        if (stable[a] >= 2 && (j >= 3 || gap_in)) {
          lam[a] = tridiag_lmax_from(al[a], be[a], lam[a], 0.0, 0.0);  // to roundoff
          lam_out[slot_angle[a]] = lam[a];
          done.push_back(a);
        } else {
          keep.push_back(a);
        }
      }
      if ((rc = emit_ritz(done, j + 1))) return rc;
      if (keep.empty()) {
        na = 0;
        break;
      }
      if ((int)keep.size() < na) {
        const int nk = (int)keep.size();
        for (int i = 0; i < nk; ++i) {
          const int a = keep[i];
          if (a == i) continue;
          al[i] = std::move(al[a]);
          be[i] = std::move(be[a]);
          lam[i] = lam[a];
          dlam[i] = dlam[a];
          prev[i] = prev[a];
          stable[i] = stable[a];
          inv[i] = inv[a];
          slot_angle[i] = slot_angle[a];
          th_h[i] = th_h[a];
        }
        CUDA_TRY(c, cudaMemcpyAsync(dmap, keep.data(), sizeof(int) * nk, cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(dthc, th_h.data(), sizeof(double) * nk,
                                    cudaMemcpyHostToDevice, c->stream));
        launch_gather_slots(Q, qs, Qalt, qs, (long long)(j + 1) * n, dmap, nk, c->stream);
        launch_gather_slots(W, (long long)n, Walt, (long long)n, (long long)n, dmap, nk,
                            c->stream);
        c->launches += 2;
        std::swap(Q, Qalt);
        std::swap(W, Walt);
        na = nk;
        // keep.data() and th_h are read by the copies above
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      }
    }
    // q_{j+1} = w / beta
    CUDA_TRY(c, cudaMemcpyAsync(sc, inv.data(), sizeof(double) * na, cudaMemcpyHostToDevice, c->stream));
    launch_batched_scale(n, W, n, sc, Q + (size_t)(j + 1) * n, qs, na, c->stream);
    ++c->launches;
  }
  // mmax reached: the angles still iterating report their last values
  std::vector<int> rest;
  for (int a = 0; a < na; ++a) {
    lam[a] = tridiag_lmax_from(al[a], be[a], lam[a], 0.0, 0.0);
    lam_out[slot_angle[a]] = lam[a];
    rest.push_back(a);
  }
  if ((rc = emit_ritz(rest, steps))) return rc;
  return BEM2D_OK;
}

// Largest singular value of an operator given y = op(x) and y = op^H(x), by
// Golub-Kahan-Lanczos bidiagonalisation with two-pass Gram-Schmidt
// reorthogonalisation of both bases, until the Ritz residual bound
// min(r, r^2 / gap) of the largest Ritz value bounds its relative error by
// tol (at most 300 steps).  v0: start vector (device, need not be
// normalised; null: the deterministic default); ritz: if not null,
// receives the unit right Ritz vector of the final estimate (device, n
// entries).
template <typename Op, typename OpH>
static int gk_sigma_max(bem2d_ctx* c, int n, Op op, OpH oph, double tol, const char* tag,
                        double* sigma, const double2* v0 = nullptr, double2* ritz = nullptr) {
  int rc = 0;
  const int mmax = std::min(n, 300);
  double2* V = static_cast<double2*>(ws(c, (std::string(tag) + "V").c_str(),
                                         sizeof(double2) * (size_t)n * (mmax + 1), &rc));
  double2* U = static_cast<double2*>(ws(c, (std::string(tag) + "U").c_str(),
                                         sizeof(double2) * (size_t)n * (mmax + 1), &rc));
  double2* h = static_cast<double2*>(ws(c, "gk_h", sizeof(double2) * (mmax + 2), &rc));
  double* nrm = static_cast<double*>(ws(c, "gk_nrm", sizeof(double) * 4, &rc));
  if (!V || !U || !h || !nrm) return rc;
  if (v0) {
    CUDA_TRY(c, cudaMemcpyAsync(V, v0, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c->stream));
  } else {
    const std::vector<std::complex<double>> sv = start_vector(n);
    CUDA_TRY(c, cudaMemcpyAsync(V, sv.data(), sizeof(double2) * n, cudaMemcpyHostToDevice,
                                c->stream));
  }
  std::vector<double> alpha, beta;
  auto norm_of = [&](double2* w, double* out) -> int {
    launch_batched_norm2(n, w, n, nrm, 1, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(out, nrm, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *out = std::sqrt(*out);
    return BEM2D_OK;
  };
  auto reorth = [&](double2* Q, int j, double2* w) {
    for (int pass = 0; pass < 2; ++pass) {
      launch_batched_dots(Q, 0, n, j, w, 0, h, 0, 1, c->stream);
      launch_batched_sub(Q, 0, n, j, w, 0, h, 0, 1, c->stream);
    }
  };
  auto normalize = [&](double2* w, double a) -> int {
    std::vector<double> inv(1, 1.0 / a);
    CUDA_TRY(c, cudaMemcpyAsync(nrm + 2, inv.data(), sizeof(double), cudaMemcpyHostToDevice, c->stream));
    launch_batched_scale(n, w, 0, nrm + 2, w, 0, 1, c->stream);
    return BEM2D_OK;
  };
  if (v0) {  // normalise the given start vector
    double a0 = 0;
    if ((rc = norm_of(V, &a0))) return rc;
    if (!(a0 > 0) || !std::isfinite(a0)) return fail(c, BEM2D_ERR_NONFINITE, "bad start vector");
    if ((rc = normalize(V, a0))) return rc;
  }
  // u_0 = op(v_0) / alpha_0
  if ((rc = op(V, U))) return rc;
  double a = 0;
  if ((rc = norm_of(U, &a))) return rc;
  if (!(a > 0) || !std::isfinite(a)) {
    *sigma = a;
    return std::isfinite(a) ? BEM2D_OK : fail(c, BEM2D_ERR_NONFINITE, "non-finite operator norm");
  }
  alpha.push_back(a);
  if ((rc = normalize(U, a))) return rc;
  double sig = a;
  for (int j = 0; j < mmax; ++j) {
    double2* vn = V + (size_t)(j + 1) * n;
    double2* un = U + (size_t)(j + 1) * n;
    // v_{j+1} = (op^H u_j - alpha_j v_j) / beta_j
    if ((rc = oph(U + (size_t)j * n, vn))) return rc;
    launch_axpy_real(n, alpha[j], V + (size_t)j * n, vn, c->stream);
    reorth(V, j + 1, vn);
    double b = 0;
    if ((rc = norm_of(vn, &b))) return rc;
    {
      // the largest Ritz value theta^2 of T = B^H B (alpha_0..j, beta_0..j-1)
      // with unit eigenvector y has residual r = |beta_j alpha_j y_j| as an
      // eigenpair of A^H A, so |sigma^2 - theta^2| <= min(r, r^2 / gap)
      // (gap: to the next Ritz value); stop when that bounds the relative
      // error of sigma by tol
      const int k = (int)alpha.size();
      std::vector<double> d(k), e(k, 0.0), e1(k > 1 ? k - 1 : 0), ev;
      for (int i = 0; i < k; ++i) {
        d[i] = alpha[i] * alpha[i] + (i > 0 ? beta[i - 1] * beta[i - 1] : 0.0);
        if (i + 1 < k) e[i] = e1[i] = alpha[i] * beta[i];
      }
      if (!tridiag_eigenvalues(d, e, &ev)) return fail(c, BEM2D_ERR_NOCONV, "tridiagonal QL failed");
      std::sort(ev.begin(), ev.end());
      const double l1 = ev.back(), l2 = k > 1 ? ev[k - 2] : 0.0;
      sig = std::sqrt(l1);
      const std::vector<double> y = tridiag_eigenvector(d, e1, l1);
      const double r = std::fabs(b * alpha[k - 1] * y[k - 1]);
      const double gap = l1 - l2;
      const double err = (k > 1 && gap > 0) ? std::min(r, r * r / gap) : r;
      if (!(b > 1e-300) || err <= 2.0 * tol * l1) break;
    }
    beta.push_back(b);
    if ((rc = normalize(vn, b))) return rc;
    // u_{j+1} = (op v_{j+1} - beta_j u_j) / alpha_{j+1}
    if ((rc = op(vn, un))) return rc;
    launch_axpy_real(n, b, U + (size_t)j * n, un, c->stream);
    reorth(U, j + 1, un);
    if ((rc = norm_of(un, &a))) return rc;
    if (!(a > 1e-300)) break;
    alpha.push_back(a);
    if ((rc = normalize(un, a))) return rc;
  }
  *sigma = sig;
  if (ritz) {
    // right Ritz vector V y, y the top eigenvector of B^T B (the
    // tridiagonal of the last step), over the k vectors v_0 .. v_{k-1}
    const int k = (int)alpha.size();
    std::vector<double> d(k), e(k > 1 ? k - 1 : 0);
    for (int i = 0; i < k; ++i) {
      d[i] = alpha[i] * alpha[i] + (i > 0 ? beta[i - 1] * beta[i - 1] : 0.0);
      if (i + 1 < k) e[i] = alpha[i] * beta[i];
    }
    const std::vector<double> y = tridiag_eigenvector(d, e, sig * sig);
    std::vector<std::complex<double>> yc(k);
    for (int i = 0; i < k; ++i) yc[i] = y[i];
    double2* yd = static_cast<double2*>(ws(c, "gk_y", sizeof(double2) * (mmax + 2), &rc));
    if (!yd) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(yd, yc.data(), sizeof(double2) * k, cudaMemcpyHostToDevice,
                                c->stream));
    launch_zgemm_rect(V, n, n, k, yd, k, 1, ritz, n, c->stream);
    ++c->launches;
    double rn = 0;
    if ((rc = norm_of(ritz, &rn))) return rc;
    if (!(rn > 0)) return fail(c, BEM2D_ERR_NONFINITE, "zero Ritz vector");
    if ((rc = normalize(ritz, rn))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // host vectors above are freed on return
  }
  return BEM2D_OK;
}

}  // namespace bem2d_gpu

extern "C" {

int bem2d_change_basis(bem2d_ctx* c, int n, const void* K, int64_t ldk, const void* M,
                       int64_t ldm, const int32_t* bstart, int nblk, void* out, int64_t ldo) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !K || !M || !out || !bstart || nblk < 1 || ldk < n || ldm < n || ldo < n)
    return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (bstart[0] != 0 || bstart[nblk] != n) return fail(c, BEM2D_ERR_ARG, "blocks must cover 0..n");
  std::vector<int> bs_of(n), bz_of(n);
  for (int b = 0; b < nblk; ++b) {
    const int s0 = bstart[b], s1 = bstart[b + 1];
    if (s1 <= s0 || s1 - s0 > 16) return fail(c, BEM2D_ERR_ARG, "block %d has size %d", b, s1 - s0);
    for (int i = s0; i < s1; ++i) {
      bs_of[i] = s0;
      bz_of[i] = s1 - s0;
    }
  }
  cudaSetDevice(c->device);
  int rc = 0;
  int* dmeta = static_cast<int*>(ws(c, "cb_meta", sizeof(int) * 2 * (size_t)n, &rc));
  double2* blk = static_cast<double2*>(ws(c, "cb_blk", sizeof(double2) * 16 * (size_t)n, &rc));
  if (!dmeta || !blk) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(dmeta, bs_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dmeta + n, bz_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
  // the mass blocks on the host (columns: hb[i*16 + p] = M[start_i + p, i])
  std::vector<std::complex<double>> hb((size_t)16 * n);
  if (is_device_ptr(M)) {
    launch_gather_blocks(n, static_cast<const double2*>(M), ldm, dmeta, dmeta + n, blk, c->stream);
    ++c->launches;
    CUDA_TRY(c, cudaMemcpyAsync(hb.data(), blk, sizeof(double2) * 16 * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  } else {
    const std::complex<double>* Mh = static_cast<const std::complex<double>*>(M);
    for (int i = 0; i < n; ++i)
      for (int p = 0; p < bz_of[i]; ++p) hb[(size_t)i * 16 + p] = Mh[(size_t)i * ldm + bs_of[i] + p];
  }
  // per block: M_b = U^H U (upper Cholesky), then U^{-1}
  std::vector<std::complex<double>> ui((size_t)16 * n);
  for (int b = 0; b < nblk; ++b) {
    const int s0 = bstart[b], m = bstart[b + 1] - s0;
    std::complex<double> Uc[16][16] = {}, Ui[16][16] = {};
    auto Mb = [&](int r, int col) { return hb[(size_t)(s0 + col) * 16 + r]; };
    for (int j = 0; j < m; ++j) {
      double dj = Mb(j, j).real();
      for (int k = 0; k < j; ++k) dj -= std::norm(Uc[k][j]);
      if (!(dj > 0)) return fail(c, BEM2D_ERR_ARG, "mass block %d is not positive definite", b);
      Uc[j][j] = std::sqrt(dj);
      for (int l = j + 1; l < m; ++l) {
        std::complex<double> v = Mb(j, l);
        for (int k = 0; k < j; ++k) v -= std::conj(Uc[k][j]) * Uc[k][l];
        Uc[j][l] = v / Uc[j][j];
      }
    }
    for (int j = 0; j < m; ++j) {  // column j of U^{-1}
      Ui[j][j] = 1.0 / Uc[j][j];
      for (int i = j - 1; i >= 0; --i) {
        std::complex<double> v = 0;
        for (int k = i + 1; k <= j; ++k) v += Uc[i][k] * Ui[k][j];
        Ui[i][j] = -v / Uc[i][i];
      }
    }
    for (int j = 0; j < m; ++j)
      for (int p = 0; p < m; ++p) ui[(size_t)(s0 + j) * 16 + p] = Ui[p][j];
  }
  double2* dui = static_cast<double2*>(ws(c, "cb_uinv", sizeof(double2) * 16 * (size_t)n, &rc));
  if (!dui) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(dui, ui.data(), sizeof(double2) * 16 * n, cudaMemcpyHostToDevice, c->stream));
  long long lk = 0;
  const double2* dK = dev_in(c, K, n, n, ldk, "in_A", &lk, &rc);
  if (!dK) return rc;
  const bool odev = is_device_ptr(out);
  double2* dO = dev_out(c, out, (size_t)n * n, "out", &rc);
  if (!dO) return rc;
  const long long lo = odev ? ldo : n;
  launch_change_basis(n, dK, lk, dmeta, dmeta + n, dui, dO, lo, c->stream);
  ++c->launches;
  CHECK_LAUNCH(c);
  if (!odev)
    CUDA_TRY(c, cudaMemcpy2DAsync(out, sizeof(double2) * ldo, dO, sizeof(double2) * n,
                                  sizeof(double2) * n, n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

int bem2d_l2_norm_cond(bem2d_ctx* c, int n, const void* A, int64_t lda, double tol, double* norm,
                       double* cond) {
  return bem2d_l2_norm_cond_prec(c, n, A, lda, tol, BEM2D_PREC_FP64, norm, cond);
}

// Order from which the mixed norm / condition number iterates with the
// explicit complex64 inverse instead of triangular solves.
static constexpr int kInverseMinN = 1024;

int bem2d_l2_norm_cond_prec(bem2d_ctx* c, int n, const void* A, int64_t lda, double tol,
                            int precision, double* norm, double* cond) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !norm || !cond || lda < n) return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (precision != BEM2D_PREC_FP64 && precision != BEM2D_PREC_MIXED)
    return fail(c, BEM2D_ERR_ARG, "unknown precision %d", precision);
  if (!(tol > 0)) tol = 1e-13;
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "nc_A", &la, &rc);
  if (!dA) return rc;
  double2* part = static_cast<double2*>(ws(c, "mv_part", mv_part_bytes(n), &rc));
  if (!part) return rc;
  const bool mixed = precision == BEM2D_PREC_MIXED;
  // sigma_max: products with A in FP64 (the FP64 pipe), or, in mixed
  // precision, in float-float on the FP32 pipe (~1e-13 relative to |A| |x|:
  // A split once, 16 n^2 bytes)
  float2* Ahi = nullptr;
  float2* Alo = nullptr;
  float2* ffb = nullptr;
  void* ffw = nullptr;
  const size_t ffw_bytes = zgemm_work_bytes(n, 1, sizeof(double2));
  if (mixed) {
    Ahi = static_cast<float2*>(ws(c, "nc_Ahi", sizeof(float2) * (size_t)n * n, &rc));
    Alo = static_cast<float2*>(ws(c, "nc_Alo", sizeof(float2) * (size_t)n * n, &rc));
    ffb = static_cast<float2*>(ws(c, "nc_ffb", 2 * sizeof(float2) * (size_t)n, &rc));
    ffw = ws(c, "nc_ffw", ffw_bytes + 256, &rc);
    if (!Ahi || !Alo || !ffb || !ffw) return rc;
    launch_split_ff(dA, la, n, Ahi, Alo, c->stream);
    ++c->launches;
  }
  auto op = [&](const double2* x, double2* y) -> int {
    if (mixed) {
      launch_zgemm_ff(false, Ahi, Alo, n, x, n, 1, y, n, ffw, ffw_bytes, ffb, c->stream);
      c->launches += 3;
    } else {
      launch_mv(dA, la, n, x, y, part, c->stream);
      c->launches += 2;
    }
    return BEM2D_OK;
  };
  auto oph = [&](const double2* x, double2* y) -> int {
    if (mixed) {
      launch_zgemm_ff(true, Ahi, Alo, n, x, n, 1, y, n, ffw, ffw_bytes, ffb, c->stream);
      c->launches += 3;
    } else {
      launch_mvh(dA, la, n, x, y, c->stream);
      c->launches += 1;
    }
    return BEM2D_OK;
  };
  double smax = 0, inv_smin = 0;
  if ((rc = gk_sigma_max(c, n, op, oph, tol, "gka", &smax))) return rc;
  // sigma_min = 1 / sigma_max(A^{-1}): complex128 LU, or complex64 LU with
  // FP64 refinement of every product with A^{-1} / A^{-H}
  const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
  LuWork w;
  int* ints = static_cast<int*>(ws(c, "lu_ints", sizeof(int) * (n + 8), &rc));
  if (!ints) return rc;
  w.ipiv = ints + 8;
  w.info = ints;
  w.status = ints + 1;
  w.scratch_bytes = lu_scratch_bytes(n);
  w.scratch = ws(c, "lu_scratch", w.scratch_bytes, &rc);
  char* aux = static_cast<char*>(ws(c, "lu_aux", lu_aux_bytes(n, esz), &rc));
  void* LU = ws(c, mixed ? "lu32" : "lu64", esz * (size_t)n * n, &rc);
  if (!w.scratch || !aux || !LU) return rc;
  w.dinv = aux;
  w.perm = reinterpret_cast<int*>(aux + (lu_aux_bytes(n, esz) - 256 - sizeof(int) * (size_t)n));
  const int tl = tic(c, BEM2D_PHASE_LU);
  if (mixed) {
    w.pack_bytes = lu_pack_bytes(n);
    w.pack = ws(c, "lu_pack", w.pack_bytes, &rc);
    if (!w.pack) return rc;
    if ((rc = attach_lookahead(c, w, n))) return rc;
    launch_to_c64(dA, la, static_cast<float2*>(LU), n, n, n, c->stream);
    ++c->launches;
    rc = lu_factor<float2>(static_cast<float2*>(LU), n, n, w, c->stream, &c->launches);
  } else {
    CUDA_TRY(c, cudaMemcpy2DAsync(LU, sizeof(double2) * n, dA, sizeof(double2) * la,
                                  sizeof(double2) * n, n, cudaMemcpyDeviceToDevice, c->stream));
    rc = lu_factor<double2>(static_cast<double2*>(LU), n, n, w, c->stream, &c->launches);
  }
  toc(c, tl);
  if (rc) return fail(c, rc, "LU launch failed: %s", cudaGetErrorString(cudaGetLastError()));
  int hinfo[2];
  CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "LU panel wait timed out");
  if (hinfo[0]) {
    // singular: sigma_min = 0
    *norm = smax;
    *cond = INFINITY;
    return fail(c, hinfo[0], "zero pivot at column %d", hinfo[0]);
  }
  double2* tmp = static_cast<double2*>(ws(c, "nc_tmp", sizeof(double2) * n, &rc));
  if (!tmp) return rc;
  if (!mixed) {
    double2* LU64 = static_cast<double2*>(LU);
    auto iop = [&, LU64](const double2* x, double2* y) -> int {
      int r = lu_solve<double2>(LU64, n, n, w, x, y, c->stream, &c->launches);
      return r ? fail(c, r, "triangular solve launch failed") : BEM2D_OK;
    };
    auto ioph = [&, LU64](const double2* x, double2* y) -> int {
      int r = lu_solve_h<double2>(LU64, n, n, w, x, y, c->stream, &c->launches);
      return r ? fail(c, r, "triangular solve launch failed") : BEM2D_OK;
    };
    if ((rc = gk_sigma_max(c, n, iop, ioph, tol, "gkb", &inv_smin))) return rc;
    *norm = smax;
    *cond = smax * inv_smin;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    resolve_timers(c);
    return BEM2D_OK;
  }
  float2* LU32 = static_cast<float2*>(LU);
  double2* r = static_cast<double2*>(ws(c, "nc_r", sizeof(double2) * n, &rc));
  float2* d = static_cast<float2*>(ws(c, "nc_d", 3 * sizeof(float2) * n, &rc));
  if (!d) return rc;
  // From kInverseMinN unknowns on, every product with A^{-1} / A^{-H} is a
  // complex64 matrix-vector product with the explicit inverse W = U^{-1}
  // L^{-1} (one pass over N^2 entries) instead of two triangular solves (a
  // chain of 2N/64 dependent block steps); the iterations below need
  // hundreds of such products.
  float2* Winv = nullptr;
  void* zw = nullptr;
  const size_t zw_bytes = mv_part_bytes(n);
  if (n >= kInverseMinN) {
    Winv = static_cast<float2*>(ws(c, "lu_inv32", sizeof(float2) * (size_t)n * n, &rc));
    zw = ws(c, "inv_zw", zw_bytes + 256, &rc);
    if (!Winv || !zw) return rc;
    const int ti = tic(c, BEM2D_PHASE_LU);
    if ((rc = lu_inverse_c64(LU32, n, n, w, Winv, n, c->stream, &c->launches)))
      return fail(c, rc, "inverse launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    toc(c, ti);
    CHECK_LAUNCH(c);
  }
  // out = op(A)^{-1} (scale x) in complex64 (out: d + n; d, d + 2n: scratch)
  auto inv32 = [&](bool herm, const double2* x, double scale) -> int {
    const int ts = tic(c, BEM2D_PHASE_SOLVE);
    struct Toc {
      bem2d_ctx* c;
      int t;
      ~Toc() { toc(c, t); }
    } toc_on_return{c, ts};
    if (Winv) {
      if (herm) {
        launch_scale_to_c64(n, x, scale, d, c->stream);
        launch_mvh(Winv, n, n, d, d + 2 * n, c->stream);
        launch_scatter_c64(n, d + 2 * n, w.perm, d + n, c->stream);
        c->launches += 3;
      } else {
        launch_gather_to_c64(n, x, w.perm, scale, d, c->stream);
        launch_mv(Winv, n, n, d, d + n, static_cast<float2*>(zw), c->stream);
        c->launches += 3;
      }
      return BEM2D_OK;
    }
    launch_scale_to_c64(n, x, scale, d, c->stream);
    ++c->launches;
    const int e = herm ? lu_solve_h<float2>(LU32, n, n, w, d, d + n, c->stream, &c->launches)
                       : lu_solve<float2>(LU32, n, n, w, d, d + n, c->stream, &c->launches);
    return e ? fail(c, e, "triangular solve launch failed") : BEM2D_OK;
  };
  double2* rpart = static_cast<double2*>(ws(c, "ir_part", residual_part_bytes(n), &rc));
  double* red = static_cast<double*>(ws(c, "ir_red", sumsq_part_bytes() + 64, &rc));
  double2* v1 = static_cast<double2*>(ws(c, "nc_v1", sizeof(double2) * n, &rc));
  if (!r || !rpart || !red || !v1) return rc;
  double* scal = red + sumsq_part_bytes() / sizeof(double);  // [0] |A|^2 [1] |x|^2 [2] |r|^2 [3] |y|^2
  launch_sumsq(dA, la, n, n, red, scal, c->stream);
  c->launches += 2;
  double hA = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&hA, scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const double normA = std::sqrt(hA);
  // y = op(A)^{-1} x: corrections from the complex64 factor, residuals
  // x - op(A) y in FP64, until the backward error
  // ||x - op(A) y|| / (||A||_F ||y|| + ||x||) is at FP64 roundoff (2e-16)
  // or stops halving; at most 10 corrections
  auto refine = [&](bool herm, const double2* x, double2* y) -> int {
    CUDA_TRY(c, cudaMemsetAsync(y, 0, sizeof(double2) * n, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(r, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c->stream));
    launch_sumsq(x, n, n, 1, red, scal + 1, c->stream);
    c->launches += 2;
    double hs[4];
    CUDA_TRY(c, cudaMemcpyAsync(hs + 1, scal + 1, sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const double xnorm = std::sqrt(hs[1]);
    double rnorm = xnorm, ynorm = 0.0, best = INFINITY;
    for (int it = 0; it < 10; ++it) {
      if (rnorm == 0.0 || rnorm <= 2.2e-16 * (normA * ynorm + xnorm)) break;
      if (!(rnorm < 0.5 * best)) break;
      best = rnorm;
      if ((rc = inv32(herm, r, 1.0 / rnorm))) return rc;
      launch_axpy_c64(n, rnorm, d + n, y, c->stream);
      if (herm) {
        launch_mvh(dA, la, n, y, tmp, c->stream);
        CUDA_TRY(c, cudaMemcpyAsync(r, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice,
                                    c->stream));
        launch_axpy_real(n, 1.0, tmp, r, c->stream);
      } else {
        launch_residual(dA, la, n, y, x, r, rpart, c->stream);
      }
      launch_sumsq(r, n, n, 1, red, scal + 2, c->stream);
      launch_sumsq(y, n, n, 1, red, scal + 3, c->stream);
      c->launches += 8;
      CUDA_TRY(c, cudaMemcpyAsync(hs + 2, scal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                  c->stream));
      CUDA_TRY(c, cudaMemcpyAsync(hinfo, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                                  c->stream));
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      if (hinfo[1]) return fail(c, BEM2D_ERR_TIMEOUT, "triangular solve wait timed out");
      rnorm = std::sqrt(hs[2]);
      ynorm = std::sqrt(hs[3]);
      if (!std::isfinite(rnorm))
        return fail(c, BEM2D_ERR_NONFINITE, "non-finite residual in a refined solve");
    }
    return BEM2D_OK;
  };
  // phase 1: the same iteration with unrefined complex64 solves (an
  // operator accurate to ~1e-7), until its estimate settles to 1e-10: its
  // Ritz vector starts the refined phase, which then needs only a few steps
  auto op32 = [&](bool herm, const double2* x, double2* y) -> int {
    if ((rc = inv32(herm, x, 1.0))) return rc;
    launch_widen(n, d + n, n, y, n, 1, c->stream);
    ++c->launches;
    return BEM2D_OK;
  };
  double s32 = 0;
  if ((rc = gk_sigma_max(
           c, n, [&](const double2* x, double2* y) { return op32(false, x, y); },
           [&](const double2* x, double2* y) { return op32(true, x, y); }, 1e-10, "gkb", &s32,
           nullptr, v1)))
    return rc;
  if ((rc = gk_sigma_max(
           c, n, [&](const double2* x, double2* y) { return refine(false, x, y); },
           [&](const double2* x, double2* y) { return refine(true, x, y); }, tol, "gkb",
           &inv_smin, v1)))
    return rc;
  *norm = smax;
  *cond = smax * inv_smin;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  resolve_timers(c);
  return BEM2D_OK;
}

int bem2d_matmul(bem2d_ctx* c, int m, int n, int k, const void* A, int64_t lda, const void* B,
                 int64_t ldb, void* C, int64_t ldc) {
  if (!c) return BEM2D_ERR_ARG;
  if (m < 1 || n < 1 || k < 1 || !A || !B || !C || lda < m || ldb < k || ldc < m)
    return fail(c, BEM2D_ERR_ARG, "bad arguments (m=%d n=%d k=%d)", m, n, k);
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0, lb = 0;
  const double2* dA = dev_in(c, A, m, k, lda, "mm_A", &la, &rc);
  if (!dA) return rc;
  const double2* dB = dev_in(c, B, k, n, ldb, "mm_B", &lb, &rc);
  if (!dB) return rc;
  const bool cdev = is_device_ptr(C);
  double2* dC = cdev ? static_cast<double2*>(C)
                     : static_cast<double2*>(ws(c, "mm_C", sizeof(double2) * (size_t)m * n, &rc));
  if (!dC) return rc;
  const long long lc = cdev ? ldc : m;
  launch_zgemm_rect(dA, la, m, k, dB, lb, n, dC, lc, c->stream);
  ++c->launches;
  CHECK_LAUNCH(c);
  if (!cdev)
    CUDA_TRY(c, cudaMemcpy2DAsync(C, sizeof(double2) * ldc, dC, sizeof(double2) * m,
                                  sizeof(double2) * m, n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

int bem2d_debug_panel_timeout(bem2d_ctx* c, int n, int polls) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 256 || n > 4096 || polls < 1)
    return fail(c, BEM2D_ERR_ARG, "timeout probe: n in [256, 4096], polls >= 1");
  cudaSetDevice(c->device);
  int rc = 0;
  int* ints = static_cast<int*>(ws(c, "lu_ints", sizeof(int) * (n + 8), &rc));
  if (!ints) return rc;
  LuWork w;
  w.ipiv = ints + 8;
  w.info = ints;
  w.status = ints + 1;
  w.scratch_bytes = lu_scratch_bytes(n);
  w.scratch = ws(c, "lu_scratch", w.scratch_bytes, &rc);
  float2* P = static_cast<float2*>(ws(c, "probe_panel", sizeof(float2) * (size_t)n * 64, &rc));
  if (!w.scratch || !P) return rc;
  CUDA_TRY(c, cudaMemsetAsync(P, 0, sizeof(float2) * (size_t)n * 64, c->stream));
  if ((rc = lu_panel_timeout_probe(P, n, n, w, (unsigned)polls, c->stream)))
    return fail(c, rc, "timeout probe launch: %s", cudaGetErrorString(cudaGetLastError()));
  ++c->launches;
  int h[2] = {0, 0};
  CUDA_TRY(c, cudaMemcpyAsync(h, w.info, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (h[1])
    return fail(c, BEM2D_ERR_TIMEOUT, "panel wait gave up after %d polls on a slot never posted",
                polls);
  return BEM2D_OK;
}

int bem2d_debug_tc_update(bem2d_ctx* c, int M, int N, int K, void* C, int64_t ldc,
                          const void* A, int64_t lda, const void* B, int64_t ldb) {
  if (!c) return BEM2D_ERR_ARG;
  if (M < 1 || N < 1 || K < 1 || !C || !A || !B || ldc < M || lda < M || ldb < K)
    return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (!is_device_ptr(C) || !is_device_ptr(A) || !is_device_ptr(B))
    return fail(c, BEM2D_ERR_ARG, "the tensor-core update takes device pointers");
  cudaSetDevice(c->device);
  int rc = 0;
  const size_t pb = tc_pack_bytes(M, N, K);
  void* pack = ws(c, "dbg_pack", pb, &rc);
  int* st = static_cast<int*>(ws(c, "dbg_status", 256, &rc));
  if (!pack || !st) return rc;
  CUDA_TRY(c, cudaMemsetAsync(st, 0, sizeof(int), c->stream));
  if ((rc = launch_tc_cgemm_sub(static_cast<float2*>(C), ldc, static_cast<const float2*>(A), lda,
                                static_cast<const float2*>(B), ldb, M, N, K, pack, pb, st,
                                c->stream)))
    return fail(c, rc, "tensor-core update launch: %s", cudaGetErrorString(cudaGetLastError()));
  c->launches += 3;
  int h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, st, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (h) return fail(c, BEM2D_ERR_TIMEOUT, "tensor-core update wait timed out");
  return BEM2D_OK;
}

int bem2d_num_range(bem2d_ctx* c, int n, const void* A, int64_t lda, int nang,
                    const double* theta, double tol, int precision, double* lmax) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || nang < 1 || !theta || !lmax || lda < n)
    return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (precision != BEM2D_PREC_FP64 && precision != BEM2D_PREC_MIXED)
    return fail(c, BEM2D_ERR_ARG, "unknown precision %d", precision);
  if (!(tol > 0)) tol = 1e-13;
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "nr_A", &la, &rc);
  if (!dA) return rc;
  double* dth = static_cast<double*>(ws(c, "nr_th", sizeof(double) * nang, &rc));
  if (!dth) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(dth, theta, sizeof(double) * nang, cudaMemcpyHostToDevice, c->stream));
  const int mmax = std::min(n, 160);
  if (precision == BEM2D_PREC_FP64)
    return numrange_lanczos<double2>(c, n, dA, la, nang, dth, tol, mmax, nullptr, lmax, nullptr,
                                     true, 0.0, tol);
  // mixed: complex64 Lanczos (full reorthogonalisation, cold start: every
  // angle's largest eigenvalue is found from its own Krylov space) until
  // each Ritz pair's residual is below 1e-7 |H| (a Ritz vector converged
  // near single precision, whose Rayleigh quotient is already within
  // ~1e-14 |H|^2 / gap), then complex128 Lanczos (full reorthogonalisation)
  // started from those Ritz vectors, all angles in one batch, each until
  // its error estimate min(r, r^2 / gap) is below tol times |H| (r the
  // complex128 residual, gap the smaller of the complex64 estimate and the
  // current tridiagonal's): with a complex64 residual near 1e-6, most angles
  // are done after the first complex128 product
  float2* A32 = static_cast<float2*>(ws(c, "nr_A32", sizeof(float2) * (size_t)n * n, &rc));
  float2* R32 = static_cast<float2*>(ws(c, "nr_R32", sizeof(float2) * (size_t)n * nang, &rc));
  double2* S64 = static_cast<double2*>(ws(c, "nr_S64", sizeof(double2) * (size_t)n * nang, &rc));
  if (!A32 || !R32 || !S64) return rc;
  launch_to_c64(dA, la, A32, n, n, n, c->stream);
  ++c->launches;
  std::vector<double> l32(nang), gap(nang);
  if ((rc = numrange_lanczos<float2>(c, n, A32, n, nang, dth, 1e-6, mmax, nullptr, l32.data(), R32,
                                     true, 1e-7, 0.0, nullptr, gap.data())))
    return rc;
  // the complex64 gap theta_1 - theta_2 over-estimates the true gap while
  // theta_2 is still rising: a quarter of it, less the complex64 noise
  double hs = 0.0;
  for (int a = 0; a < nang; ++a) hs = std::max(hs, std::fabs(l32[a]));
  for (int a = 0; a < nang; ++a) gap[a] = std::max(0.0, 0.25 * gap[a] - 1e-6 * hs);
  launch_widen(n, R32, n, S64, n, nang, c->stream);
  ++c->launches;
  // the complex128 phase's products in float-float (~1e-13 relative to
  // |A| |x|, a hundred times below tol): A split once into fl32(A) and the
  // rest, 16 N^2 bytes
  float2* Ahi = static_cast<float2*>(ws(c, "nr_Ahi", sizeof(float2) * (size_t)n * n, &rc));
  float2* Alo = static_cast<float2*>(ws(c, "nr_Alo", sizeof(float2) * (size_t)n * n, &rc));
  if (!Ahi || !Alo) return rc;
  launch_split_ff(dA, la, n, Ahi, Alo, c->stream);
  ++c->launches;
  return numrange_lanczos<double2>(c, n, dA, la, nang, dth, tol, mmax, S64, lmax, nullptr, true,
                                   0.0, tol, gap.data(), nullptr, Ahi, Alo);
}

}  // extern "C"

namespace bem2d_gpu {

// Eigenvalues of the Hermitian M (N x N, device, overwritten): `count`
// ascending from the smallest or descending from the largest, into out
// (host or device, count doubles).
static int spectra_run(bem2d_ctx* c, double2* M, int N, int count, int descending, double* out) {
  int rc = 0;
  void* work = ws(c, "sp_work", spectra_work_bytes(N), &rc);
  if (!work) return rc;
  const bool odev = is_device_ptr(out);
  double* dout = odev ? out : static_cast<double*>(ws(c, "sp_out", sizeof(double) * count, &rc));
  if (!dout) return rc;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      sms < 1)
    sms = 1;
  c->launches += launch_tridiag_eigs(M, N, count, descending, work, dout, sms, c->stream);
  CHECK_LAUNCH(c);
  if (!odev)
    CUDA_TRY(c, cudaMemcpyAsync(out, dout, sizeof(double) * count, cudaMemcpyDeviceToHost,
                                c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

}  // namespace bem2d_gpu

extern "C" {

int bem2d_hermitian_eigenvalues(bem2d_ctx* c, int n, const void* A, int64_t lda, double* w) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !w || lda < n) return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (n > BEM2D_SPECTRA_MAX_N)
    return fail(c, BEM2D_ERR_ARG, "order %d above BEM2D_SPECTRA_MAX_N = %d", n,
                BEM2D_SPECTRA_MAX_N);
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "sp_A", &la, &rc);
  if (!dA) return rc;
  double2* M = static_cast<double2*>(ws(c, "sp_M", sizeof(double2) * (size_t)n * n, &rc));
  if (!M) return rc;
  launch_herm_from_upper(dA, la, n, M, c->stream);
  ++c->launches;
  CHECK_LAUNCH(c);
  return spectra_run(c, M, n, n, 0, w);
}

int bem2d_singular_values(bem2d_ctx* c, int n, const void* A, int64_t lda, double* s) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !s || lda < n) return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (n > BEM2D_SPECTRA_MAX_N / 2)
    return fail(c, BEM2D_ERR_ARG, "order %d above BEM2D_SPECTRA_MAX_N / 2 = %d", n,
                BEM2D_SPECTRA_MAX_N / 2);
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "sp_A", &la, &rc);
  if (!dA) return rc;
  const int N = 2 * n;
  double2* M = static_cast<double2*>(ws(c, "sp_M", sizeof(double2) * (size_t)N * N, &rc));
  if (!M) return rc;
  launch_jordan_wielandt(dA, la, n, M, c->stream);
  ++c->launches;
  CHECK_LAUNCH(c);
  return spectra_run(c, M, N, n, 1, s);
}

int bem2d_eigenvalues(bem2d_ctx* c, int n, const void* A, int64_t lda, void* w) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !w || lda < n) return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (n > BEM2D_EIG_MAX_N)
    return fail(c, BEM2D_ERR_ARG, "order %d above BEM2D_EIG_MAX_N = %d", n, BEM2D_EIG_MAX_N);
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "eig_in", &la, &rc);
  if (!dA) return rc;
  double2* H = static_cast<double2*>(ws(c, "eig_H", sizeof(double2) * (size_t)n * n, &rc));
  void* work = ws(c, "eig_work", eig_work_bytes(n), &rc);
  if (!H || !work) return rc;
  const bool odev = is_device_ptr(w);
  double2* dw = odev ? static_cast<double2*>(w)
                     : static_cast<double2*>(ws(c, "eig_w", sizeof(double2) * n, &rc));
  if (!dw) return rc;
  CUDA_TRY(c, cudaMemcpy2DAsync(H, sizeof(double2) * n, dA, sizeof(double2) * la,
                                sizeof(double2) * n, n, cudaMemcpyDeviceToDevice, c->stream));
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      sms < 1)
    sms = 1;
  c->launches += launch_eigenvalues(H, n, work, dw, sms, c->stream);
  CHECK_LAUNCH(c);
  int status = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&status, eig_status_ptr(work, n), sizeof(int),
                              cudaMemcpyDeviceToHost, c->stream));
  if (!odev)
    CUDA_TRY(c, cudaMemcpyAsync(w, dw, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (status)
    return fail(c, BEM2D_ERR_NOCONV, "QR iteration: %d eigenvalues not found within the limit",
                status);
  return BEM2D_OK;
}

int bem2d_eigenvectors(bem2d_ctx* c, int n, const void* A, int64_t lda, void* w, void* vr,
                       int64_t ldvr) {
  if (!c) return BEM2D_ERR_ARG;
  if (n < 1 || !A || !w || !vr || lda < n || ldvr < n)
    return fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (n > BEM2D_EIG_MAX_N)
    return fail(c, BEM2D_ERR_ARG, "order %d above BEM2D_EIG_MAX_N = %d", n, BEM2D_EIG_MAX_N);
  cudaSetDevice(c->device);
  int rc = 0;
  long long la = 0;
  const double2* dA = dev_in(c, A, n, n, lda, "eig_in", &la, &rc);
  if (!dA) return rc;
  const size_t nn = sizeof(double2) * (size_t)n * n;
  double2* H = static_cast<double2*>(ws(c, "eig_H", nn, &rc));
  double2* Z = static_cast<double2*>(ws(c, "eig_Z", nn, &rc));
  double2* Y = static_cast<double2*>(ws(c, "eig_Y", nn, &rc));
  void* work = ws(c, "eig_work", eig_work_bytes(n), &rc);
  if (!H || !Z || !Y || !work) return rc;
  const bool wdev = is_device_ptr(w), vdev = is_device_ptr(vr) && ldvr == n;
  double2* dw = wdev ? static_cast<double2*>(w)
                     : static_cast<double2*>(ws(c, "eig_w", sizeof(double2) * n, &rc));
  double2* X = vdev ? static_cast<double2*>(vr) : static_cast<double2*>(ws(c, "eig_X", nn, &rc));
  if (!dw || !X) return rc;
  CUDA_TRY(c, cudaMemcpy2DAsync(H, sizeof(double2) * n, dA, sizeof(double2) * la,
                                sizeof(double2) * n, n, cudaMemcpyDeviceToDevice, c->stream));
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      sms < 1)
    sms = 1;
  c->launches += launch_eigenvalues(H, n, work, dw, sms, c->stream, Z);
  CHECK_LAUNCH(c);
  int status = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&status, eig_status_ptr(work, n), sizeof(int),
                              cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (status)
    return fail(c, BEM2D_ERR_NOCONV, "QR iteration: %d eigenvalues not found within the limit",
                status);
  c->launches += launch_eigenvectors(H, Z, n, Y, X, c->stream);
  CHECK_LAUNCH(c);
  if (!wdev)
    CUDA_TRY(c, cudaMemcpyAsync(w, dw, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
  if (!vdev)
    CUDA_TRY(c, cudaMemcpy2DAsync(vr, sizeof(double2) * ldvr, X, sizeof(double2) * n,
                                  sizeof(double2) * n, n, cudaMemcpyDefault, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

int bem2d_eval_kernel(bem2d_ctx* c, const bem2d_geometry* geom, const bem2d_quad* quad,
                      int kernel, double k_re, double k_im, double eta, const void* coeffs,
                      int npts, const double* points, void* out) {
  if (!c) return BEM2D_ERR_ARG;
  if (kernel < BEM2D_KERNEL_SINGLE || kernel > BEM2D_KERNEL_COMBINED)
    return fail(c, BEM2D_ERR_ARG, "unknown kernel %d", kernel);
  if (npts < 0 || (npts > 0 && (!points || !out)) || !coeffs)
    return fail(c, BEM2D_ERR_ARG, "bad arguments");
  int rc = check_k(c, k_re, k_im);
  if (rc) return rc;
  if (npts == 0) return BEM2D_OK;
  cudaSetDevice(c->device);
  Staged st;
  if ((rc = stage(c, geom, quad, true, false, &st))) return rc;
  long long l = 0;
  const double2* dc = dev_in(c, coeffs, geom->n_unk, 1, geom->n_unk, "ek_c", &l, &rc);
  if (!dc) return rc;
  double* dp = static_cast<double*>(ws(c, "ek_p", sizeof(double) * 2 * (size_t)npts, &rc));
  if (!dp) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(dp, points, sizeof(double) * 2 * npts, cudaMemcpyDefault, c->stream));
  const bool odev = is_device_ptr(out);
  double2* dO = dev_out(c, out, (size_t)npts, "ek_o", &rc);
  if (!dO) return rc;
  launch_potential(st.g, st.t, st.r.ng, kernel, k_re, eta, dc, npts, dp, dO, c->stream, k_im);
  ++c->launches;
  CHECK_LAUNCH(c);
  if (!odev)
    CUDA_TRY(c, cudaMemcpyAsync(out, dO, sizeof(double2) * npts, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return BEM2D_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Context accessors for entry points defined in other translation units.
namespace bem2d_gpu {
int ctx_device(const bem2d_ctx* c) { return c->device; }
cudaStream_t ctx_stream(const bem2d_ctx* c) { return c->stream; }
long long* ctx_launches(bem2d_ctx* c) { return &c->launches; }
std::vector<bem2d_ctx*>& ctx_workers(bem2d_ctx* c) { return c->workers; }
// Sweep workers factor with full 256-row panel CTAs (measured on the
// ellipse sweep, 16 workers: 636 ms with 64-row, 614 ms with 256-row CTAs).
#ifndef BEM2D_SWEEP_PANEL_ROWS
#define BEM2D_SWEEP_PANEL_ROWS 256
#endif
// Persistent CTAs of a sweep worker's tensor-core updates (0: one per SM).
#ifndef BEM2D_SWEEP_TC_CTAS
#define BEM2D_SWEEP_TC_CTAS 0
#endif
bool ctx_timers_on(const bem2d_ctx* c) { return c->timers; }
void ctx_add_timers(bem2d_ctx* dst, const bem2d_ctx* src) {
  for (int i = 0; i < 4; ++i) {
    dst->phase_ms[i] += src->phase_ms[i];
    dst->phase_n[i] += src->phase_n[i];
  }
}
int ctx_make_sweep_worker(bem2d_ctx* c) {
  c->panel_min_rows = BEM2D_SWEEP_PANEL_ROWS;
  c->tc_ctas = BEM2D_SWEEP_TC_CTAS;
  if (c->stream_hi) return BEM2D_OK;
  cudaSetDevice(c->device);
  int least = 0, greatest = 0;
  CUDA_TRY(c, cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CUDA_TRY(c, cudaStreamCreateWithPriority(&c->stream_hi, cudaStreamNonBlocking, greatest));
  CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_asm, cudaEventDisableTiming));
  CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_sol, cudaEventDisableTiming));
  return BEM2D_OK;
}
int ctx_fail(bem2d_ctx* c, int code, const char* msg) { return fail(c, code, "%s", msg); }
}  // namespace bem2d_gpu
