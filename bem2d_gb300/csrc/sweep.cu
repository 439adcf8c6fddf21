// Batched wavenumber sweep: many independent sound-soft scattering solves
// (one geometry and one wavenumber each, sizes uneven) run concurrently.
//
// The reference runs such sweeps as a serial loop over k that rebuilds the
// geometry and calls DiscreteKernel / EvalIdent / the solver once per k
// (normcomps/ellipsenormcond.cpp:66-128; SoundSoftScattering::Discretize and
// Solve, lib/bem2d_soundsoftscattering.h:95-126).  Here every problem is a
// work item; W host workers, each owning a context (its own CUDA stream and
// device workspace), pull items largest-first (longest-processing-time
// order) and run the complete single-problem path on their stream.  Small
// problems do not fill the 152 SMs on their own (their LU is bound by the
// latency of the panel steps), so several in flight at once keep the GPU
// busy; the largest items start first so the tail is short.  A worker's
// assembly kernels (grids of thousands of CTAs) run on its normal stream,
// its factorisation and solve on a high-priority one: the block scheduler
// then gives SM slots freed by one worker's assembly to another worker's
// panel chain first, instead of queueing that chain behind the whole grid.
//
// The worker contexts live in the parent context and keep their workspaces
// between calls, so a repeated sweep allocates nothing after the first.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace {
constexpr int kDefaultWorkers = 16;
constexpr int kMaxWorkers = 32;
}  // namespace

extern "C" int bem2d_sweep_solve(bem2d_ctx* c, int nk, const bem2d_geometry* geoms,
                                 const bem2d_quad* quad, const double* k, const double* eta,
                                 double dir_x, double dir_y, int precision, double tol,
                                 int nworkers, void* const* x, bem2d_solve_info* infos) {
  using namespace bem2d_gpu;
  if (!c) return BEM2D_ERR_ARG;
  if (nk < 0 || (nk > 0 && (!geoms || !quad || !k || !x)))
    return ctx_fail(c, BEM2D_ERR_ARG, "bad arguments");
  if (nk == 0) return BEM2D_OK;
  if (precision != BEM2D_PREC_FP64 && precision != BEM2D_PREC_MIXED &&
      precision != BEM2D_PREC_MIXED_TF32)
    return ctx_fail(c, BEM2D_ERR_ARG, "unknown precision");
  for (int i = 0; i < nk; ++i)
    if (!x[i]) return ctx_fail(c, BEM2D_ERR_ARG, "an output pointer is NULL");
  const int W = std::max(1, std::min({nworkers > 0 ? nworkers : kDefaultWorkers, kMaxWorkers, nk}));
  std::vector<bem2d_ctx*>& workers = ctx_workers(c);
  while ((int)workers.size() < W) {
    bem2d_ctx* w = nullptr;
    const int rc = bem2d_ctx_create(ctx_device(c), &w);
    if (rc) return ctx_fail(c, rc, "could not create a sweep worker context");
    workers.push_back(w);
    if (ctx_make_sweep_worker(w) != BEM2D_OK)
      return ctx_fail(c, BEM2D_ERR_CUDA, bem2d_ctx_last_error(w));
  }
  // largest problems first
  std::vector<int> order(nk);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return geoms[a].n_unk > geoms[b].n_unk; });
  std::vector<long long> launches0(W);
  const bool timed = ctx_timers_on(c);  // phase timers: summed over the problems
  for (int w = 0; w < W; ++w) {
    launches0[w] = bem2d_ctx_launch_count(workers[w]);
    bem2d_ctx_enable_timers(workers[w], timed ? 1 : 0);
  }

  std::atomic<int> next{0};
  std::atomic<bool> stop{false};
  std::mutex err_mu;
  int err_rc = BEM2D_OK, err_item = -1;
  std::string err_msg;
  auto work = [&](int wi) {
    bem2d_ctx* wc = workers[wi];
    for (;;) {
      if (stop.load()) return;
      const int j = next.fetch_add(1);
      if (j >= nk) return;
      const int i = order[j];
      bem2d_solve_info rep{0, 0, 0.0};
      const int rc = bem2d_scattering_solve(wc, &geoms[i], quad, k[i], 0.0, eta ? eta[i] : k[i],
                                            dir_x, dir_y, precision, tol, x[i], &rep);
      if (infos) infos[i] = rep;
      if (rc != BEM2D_OK) {
        std::lock_guard<std::mutex> lock(err_mu);
        if (err_rc == BEM2D_OK) {
          err_rc = rc;
          err_item = i;
          err_msg = bem2d_ctx_last_error(wc);
        }
        stop = true;
        return;
      }
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(W - 1);
  for (int w = 1; w < W; ++w) pool.emplace_back(work, w);
  work(0);
  for (auto& t : pool) t.join();
  long long* total = ctx_launches(c);
  for (int w = 0; w < W; ++w) {
    *total += bem2d_ctx_launch_count(workers[w]) - launches0[w];
    if (timed) ctx_add_timers(c, workers[w]);
  }
  if (err_rc != BEM2D_OK) {
    const std::string msg = "problem " + std::to_string(err_item) + ": " + err_msg;
    return ctx_fail(c, err_rc, msg.c_str());
  }
  return BEM2D_OK;
}
