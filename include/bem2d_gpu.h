/*
 * bem2d_gpu.h -- C ABI of the GB300 (sm_103a) Galerkin assembly and dense
 * solve path of bem2d.
 *
 * Every entry point replaces one routine of the reference library; the
 * comment above each names it (file:line in the reference project).  The C++
 * API in bem2d_gb300/lib (same class and function names as the reference's
 * lib/) is written on top of these calls, and so is the Python test/bench
 * binding (bem2d_gb300/capi.py).
 *
 * Conventions
 *  - Matrices are complex128 (interleaved re, im), column-major, entry (i,j)
 *    at index i + j*ld: the reference's Matrix layout
 *    (lib/bem2d_mathroutines.cpp:78-140).
 *  - Matrix/vector pointers may be host or device memory; the library looks
 *    the pointer up and copies host data through its own device workspace.
 *    Calls are stream-ordered on the context's stream and return after the
 *    results are in place (host results copied back).
 *  - Return values: 0 = success; > 0 = LAPACK-style info (a zero pivot at
 *    column `info`, 1-based: the reference throws LapackError); < 0 = one of
 *    the BEM2D_ERR_* codes.  bem2d_ctx_last_error() gives a message.
 *  - A context is not thread-safe; use one per host thread.
 *  - Wavenumbers are k_re + i k_im.  A complex k (the reference's AMOS zbesh
 *    branch, lib/bem2d_mathroutines.cpp:44-75) is evaluated in FP64 by the
 *    complex-argument Hankel evaluator (csrc/hankel_c.cuh) and must satisfy
 *    k_re > 0 and arg k >= -pi/3 (k_im >= -sqrt(3) k_re), else
 *    BEM2D_ERR_UNSUPPORTED.  eta stays real, as in the reference.
 */
#ifndef BEM2D_GPU_H
#define BEM2D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define BEM2D_OK 0
#define BEM2D_ERR_ARG (-1)         /* bad argument: reference ParameterException / SizeError / ArrayMismatch */
#define BEM2D_ERR_CUDA (-2)        /* CUDA runtime error */
#define BEM2D_ERR_NOMEM (-3)       /* device allocation failed */
#define BEM2D_ERR_NONFINITE (-4)   /* NaN/Inf in an assembled entry or a residual */
#define BEM2D_ERR_NOCONV (-5)      /* iterative refinement / iteration did not converge */
#define BEM2D_ERR_TIMEOUT (-6)     /* a bounded device-side wait gave up */
#define BEM2D_ERR_UNSUPPORTED (-7) /* k outside arg k >= -pi/3, unknown element or basis kind */

/* ---- element kinds (lib/bem2d_element.h:72-116, lib/bem2d_curvetypes.h) -
 * param row (8 doubles) per element:
 *   SEGMENT     p1x p1y p2x p2y                 ConstElement(p1, p2)
 *   curves      t1 t2 c0 c1 c2 c3               AnalyticCurveElement(t1, t2, curve)
 *     CIRCLE, TREFOIL, KITE: no curve parameters
 *     ELLIPSE: c0 = rho;  ELLIPSEARC: c0..c3 = a, b, theta1, theta2
 *     INVELLIPSE: c0 = alpha                                                  */
#define BEM2D_ELEM_SEGMENT 0
#define BEM2D_ELEM_CIRCLE 1
#define BEM2D_ELEM_TREFOIL 2
#define BEM2D_ELEM_KITE 3
#define BEM2D_ELEM_ELLIPSE 4
#define BEM2D_ELEM_ELLIPSEARC 5
#define BEM2D_ELEM_INVELLIPSE 6

/* ---- basis kinds (lib/bem2d_basistypes.h:28-62) ------------------------ */
#define BEM2D_BASIS_POLY 0 /* PolBasis(degree): t^degree; param = degree */
#define BEM2D_BASIS_LIN 1  /* LinBasis(sign): t or 1-t; param = sign     */

/* ---- kernels (lib/bem2d_kernel.h:12-88) -------------------------------- */
#define BEM2D_KERNEL_SINGLE 0     /* SingleLayer               */
#define BEM2D_KERNEL_DOUBLE 1     /* DoubleLayer               */
#define BEM2D_KERNEL_CONJDOUBLE 2 /* ConjDoubleLayer           */
#define BEM2D_KERNEL_COMBINED 3   /* CombinedSingleConjDouble  */

/* ---- incident-field functionals (lib/bem2d_fun.h:14-93) ---------------- */
#define BEM2D_FUN_PLANEWAVE 0
#define BEM2D_FUN_NORMALPLANEWAVE 1
#define BEM2D_FUN_COMBINEDPLANEWAVE 2

/* ---- solver precision -------------------------------------------------- */
#define BEM2D_PREC_FP64 0  /* complex128 LU, FP64 throughout                 */
#define BEM2D_PREC_MIXED 1 /* complex64 LU + FP64 iterative refinement      */
/* As BEM2D_PREC_MIXED, with the LU's tensor-core trailing updates as one
 * TF32 product per term (1xTF32: operands rounded to 10 mantissa bits, a
 * third of the 3xTF32 tensor work).  The factor is then accurate to about
 * 1e-3 relative instead of 1e-6, so refinement contracts the error by about
 * cond(A) 1e-3 per step: for systems with cond(A) up to ~100; beyond that
 * GMRES-IR takes over (see bem2d_solve_system).  Accepted by
 * bem2d_solve_system, bem2d_scattering_solve and bem2d_sweep_solve. */
#define BEM2D_PREC_MIXED_TF32 2

/* QuadOption (lib/bem2d_quadrature.h:26-30). */
typedef struct {
  int32_t L;
  int32_t N;
  double sigma;
} bem2d_quad;

/* Geometry in flat form: the element list of Geometry (lib/bem2d_geometry.h)
 * with each element's index()/next()/prev() (lib/bem2d_element.h:36-58;
 * -1 = unset), and the (element, basis) list of Geometry::FlatMap()
 * (lib/bem2d_geometry.h:48-57) whose order numbers the unknowns. */
typedef struct {
  int32_t n_elem;
  const int32_t* kind;    /* [n_elem]     BEM2D_ELEM_*                      */
  const double* param;    /* [n_elem * 8] see above                         */
  const int64_t* index;   /* [n_elem]                                       */
  const int64_t* next;    /* [n_elem]                                       */
  const int64_t* prev;    /* [n_elem]                                       */
  int32_t n_unk;
  const int32_t* unk_elem;  /* [n_unk] element position (0..n_elem-1)     */
  const int32_t* unk_kind;  /* [n_unk] BEM2D_BASIS_*                       */
  const double* unk_param;  /* [n_unk] degree or sign                      */
} bem2d_geometry;

/* Solver report. */
typedef struct {
  int32_t info;         /* LAPACK-style info of the factorisation (0 = ok)   */
  int32_t iterations;   /* refinement steps taken (mixed precision)          */
  double residual;      /* final ||b - A x||_2 / (||A||_F ||x||_2 + ||b||_2) */
} bem2d_solve_info;

typedef struct bem2d_ctx bem2d_ctx;

/* ---- context ----------------------------------------------------------- */
int bem2d_ctx_create(int device, bem2d_ctx** ctx);
void bem2d_ctx_destroy(bem2d_ctx* ctx);
const char* bem2d_ctx_last_error(const bem2d_ctx* ctx);
/* cudaStream_t the context issues its work on (default: its own stream). */
void* bem2d_ctx_stream(bem2d_ctx* ctx);
int bem2d_ctx_set_stream(bem2d_ctx* ctx, void* stream);
/* Number of kernels this context has launched so far. */
int64_t bem2d_ctx_launch_count(const bem2d_ctx* ctx);

/* ---- quadrature rules -------------------------------------------------- */
/* Gauss(x, w, N) on [0,1]: replaces lib/bem2d_quadrature.cpp:10-56 (host). */
int bem2d_gauss(int n, double* x, double* w);

/* ---- assembly ---------------------------------------------------------- */
/* out = beta * EvalIdent(geom) + alpha * DiscreteKernel(geom, quad, kernel):
 * replaces DiscreteKernel<kernel> (lib/bem2d_quadrature.h:231-294) and, with
 * alpha = 2, beta = 1, kernel = COMBINED, the matrix of
 * SoundSoftScattering::DiscretizeMatrix (lib/bem2d_soundsoftscattering.h:95-103).
 * eta is the coupling of COMBINED (CombinedSingleConjDouble(k) uses eta = k).
 * All arithmetic FP64.  out: complex128 n_unk x n_unk, ld >= n_unk. */
int bem2d_discrete_kernel(bem2d_ctx* ctx, const bem2d_geometry* geom,
                          const bem2d_quad* quad, int kernel, double k_re,
                          double k_im, double eta, double alpha, double beta,
                          void* out, int64_t ld);

/* Mixed-precision variant of bem2d_discrete_kernel: same matrix, with the
 * Bessel functions of every entry evaluated in compensated single-single
 * (float-float) arithmetic on the FP32 pipe (~1e-14 relative per kernel
 * evaluation); the near-field geometry and quadrature sums stay FP64.
 * Writes complex128 (out, ld) and its complex64 rounding (out32, ld32):
 * the residual and LU inputs of the mixed solver.  Requires k_re > 0.  A
 * complex k assembles in FP64 (as bem2d_discrete_kernel) and rounds. */
int bem2d_discrete_kernel_mixed(bem2d_ctx* ctx, const bem2d_geometry* geom,
                                const bem2d_quad* quad, int kernel, double k_re,
                                double k_im, double eta, double alpha, double beta,
                                void* out, int64_t ld, void* out32, int64_t ld32);

/* out = mass matrix: replaces EvalIdent (lib/bem2d_quadrature.cpp:79-127). */
int bem2d_eval_ident(bem2d_ctx* ctx, const bem2d_geometry* geom,
                     const bem2d_quad* quad, void* out, int64_t ld);

/* out[i] = scale * sum_q fun(x_q) |J| phi_i(x_q) w_q: replaces DotProdBasFuns
 * (lib/bem2d_quadrature.h:130-156) with PlaneWave / NormalPlaneWave /
 * CombinedPlaneWave (lib/bem2d_fun.h:14-93); SoundSoftScattering::
 * DiscretizeRhs uses COMBINEDPLANEWAVE with scale = 2. */
int bem2d_dot_prod_basfuns(bem2d_ctx* ctx, const bem2d_geometry* geom,
                           const bem2d_quad* quad, int fun, double k_re,
                           double k_im, double dir_x, double dir_y, double eta,
                           double scale, void* out);

/* ---- dense solve ------------------------------------------------------- */
/* x = A^{-1} b: replaces SolveSystem (lib/bem2d_mathroutines.cpp:323-351,
 * LAPACK zgetrf + zgetrs).  A (n x n, lda) and b are not modified.
 * BEM2D_PREC_FP64: blocked complex128 LU with partial pivoting.
 * BEM2D_PREC_MIXED: complex64 LU with partial pivoting (tournament
 *   pivoting for panels taller than 4096 rows), then FP64 iterative
 *   refinement with the complex128 A until the backward error
 *   ||b - A x|| / (||A||_F ||x|| + ||b||) <= tol (tol <= 0 selects 1e-14);
 *   at most 30 steps.  If plain refinement stalls or diverges above
 *   max(tol, 1e-12) (cond(A) too large for the complex64 factor), GMRES-IR
 *   takes over (GMRES in FP64 preconditioned by the complex64 factor, FP64
 *   residuals); BEM2D_ERR_NOCONV if that stalls too.  info->iterations:
 *   refinement steps, plus the factor's applications inside GMRES-IR. */
int bem2d_solve_system(bem2d_ctx* ctx, int n, const void* A, int64_t lda,
                       const void* b, void* x, int precision, double tol,
                       bem2d_solve_info* info);

/* Largest n bem2d_solve_system_noalloc accepts. */
#define BEM2D_NOALLOC_MAX_N 1024

/* x = A^{-1} b as bem2d_solve_system with BEM2D_PREC_FP64, without allocating
 * device memory.  No counterpart in the reference.  For callers that may not
 * call cudaMalloc: a solver inside an application whose memory pool owns the
 * device, or a loop that cannot afford cudaMalloc/cudaFree synchronising the
 * device.  It calls no cudaMalloc, cudaFree or allocating library routine;
 * its work buffers live in one static device array of 21 MiB that the CUDA
 * runtime reserves with this library's device code.
 *   n <= BEM2D_NOALLOC_MAX_N, else BEM2D_ERR_ARG (message names the limit).
 *   A, b, x: host or device memory; A and b are not modified.
 *   The first call on each device looks up the array's address
 *   (cudaGetSymbolAddress) and caches it; make that call before any stream
 *   capture.  The array is shared by all calls on a device and keeps the
 *   last call's contents (what must start at zero is cleared on every
 *   call): calls whose GPU work overlaps race, so serialise them.
 *   The context supplies the stream and the error message; it must have
 *   been created beforehand (bem2d_ctx_create allocates no device memory). */
int bem2d_solve_system_noalloc(bem2d_ctx* ctx, int n, const void* A, int64_t lda,
                               const void* b, void* x, bem2d_solve_info* info);

/* Host-side layout check of bem2d_solve_system_noalloc (no counterpart in
 * the reference): 1 if every work buffer of the largest accepted order
 * BEM2D_NOALLOC_MAX_N fits the static array, else 0; *total and *capacity
 * (may be NULL) receive the bytes needed and the array's size.  No GPU
 * work. */
int bem2d_noalloc_scratch_fits(int64_t* total, int64_t* capacity);

/* C = A B (complex128; C m x n, A m x k, B k x n, column-major, host or
 * device): replaces Matrix * Matrix (lib/bem2d_mathroutines.cpp:190-206,
 * cblas_zgemm).  FP64 on the CUDA cores (64 x 64 tiles). */
int bem2d_matmul(bem2d_ctx* ctx, int m, int n, int k, const void* A, int64_t lda, const void* B,
                 int64_t ldb, void* C, int64_t ldc);

/* ---- norms, change of basis, numerical range, potentials --------------- */
/* out = U^{-H} K U^{-1} where M = U^H U: replaces ChangeBasis
 * (lib/bem2d_mathroutines.cpp:534-588, zpotrf + two ztrsm).  M must be block
 * diagonal, as mass matrices are: nblk blocks starting at bstart[0..nblk-1]
 * (bstart[0] = 0, bstart[nblk] = n, block sizes 1..16); entries of M outside
 * the blocks are ignored.  BEM2D_ERR_ARG if a block is not positive
 * definite (the reference would throw LapackError from zpotrf). */
int bem2d_change_basis(bem2d_ctx* ctx, int n, const void* K, int64_t ldk, const void* M,
                       int64_t ldm, const int32_t* bstart, int nblk, void* out,
                       int64_t ldo);

/* norm = sigma_max(A), cond = sigma_max / sigma_min: replaces L2NormCond
 * (lib/bem2d_mathroutines.cpp:208-266, zgesvd).  Golub-Kahan-Lanczos
 * bidiagonalisation with full reorthogonalisation, on A for sigma_max and on
 * A^{-1} (complex128 LU, solves with A and A^H) for sigma_min, each until
 * the Ritz residual bound min(r, r^2 / gap) of the largest Ritz value bounds
 * its relative error by tol (tol <= 0 selects 1e-13; at most 300 steps). */
int bem2d_l2_norm_cond(bem2d_ctx* ctx, int n, const void* A, int64_t lda, double tol,
                       double* norm, double* cond);

/* bem2d_l2_norm_cond with a choice of arithmetic for sigma_min (the same
 * routine of the reference, lib/bem2d_mathroutines.cpp:208-266):
 * BEM2D_PREC_FP64: as bem2d_l2_norm_cond (complex128 LU);
 * BEM2D_PREC_MIXED: complex64 LU (tensor-core trailing updates); the Lanczos
 *   iteration on A^{-1} first runs with unrefined complex64 solves (to
 *   1e-10), then again from that Ritz vector with every product with A^{-1}
 *   or A^{-H} refined with FP64 residuals of A until its backward error
 *   reaches FP64 roundoff or stops halving, so the final iteration sees the
 *   operator to FP64 accuracy.  From n = 1024 on the complex64 solves are
 *   products with the explicit inverse U^{-1} L^{-1} (formed once from the
 *   factor, n^2 complex64 of device memory more).  The Lanczos arithmetic
 *   is FP64 in both modes. */
int bem2d_l2_norm_cond_prec(bem2d_ctx* ctx, int n, const void* A, int64_t lda, double tol,
                            int precision, double* norm, double* cond);

/* Largest order bem2d_hermitian_eigenvalues accepts (its workspace holds an
 * n x n complex128 matrix: 4.3 GB at the limit); bem2d_singular_values
 * accepts half of it. */
#define BEM2D_SPECTRA_MAX_N 16384

/* w[0..n-1] = eigenvalues, ascending, of the Hermitian matrix whose upper
 * triangle A holds (the diagonal's real part is used): replaces
 * HermitianEigenvalues (lib/bem2d_mathroutines.cpp:353-433, zheev with
 * jobz 'N', uplo 'U').  Householder reduction to real tridiagonal form on
 * the GPU (four kernels per column), then bisection on Sturm counts, one
 * thread per eigenvalue; absolute accuracy ~ n eps ||A||.  A: host or
 * device; w: host or device. */
int bem2d_hermitian_eigenvalues(bem2d_ctx* ctx, int n, const void* A, int64_t lda, double* w);

/* s[0..n-1] = singular values of A, descending: replaces SingularValues
 * (lib/bem2d_mathroutines.cpp:268-320, zgesvd without vectors).  They are
 * the n largest eigenvalues of the Hermitian [0 A; A^H 0], computed as in
 * bem2d_hermitian_eigenvalues (absolute accuracy ~ n eps ||A||).
 * n <= BEM2D_SPECTRA_MAX_N / 2. */
int bem2d_singular_values(bem2d_ctx* ctx, int n, const void* A, int64_t lda, double* s);

/* Largest order bem2d_eigenvalues accepts: its QR iteration runs on one
 * CTA, about n^2 dependent rotation steps of a few microseconds each. */
#define BEM2D_EIG_MAX_N 4096

/* w[0..n-1] (complex128) = eigenvalues of the general complex A: replaces
 * Eigenvalues(const Matrix&, pcvector&) (lib/bem2d_mathroutines.cpp:437-466,
 * zgeev without eigenvectors).  Householder reduction to upper Hessenberg
 * form on the GPU (six kernels per column), then implicitly shifted QR
 * (Wilkinson shifts, exceptional shifts, closed-form 2 x 2 blocks) in one
 * CTA; no balancing.  Eigenvalues come in the order they deflate (bottom of
 * the matrix first), as in LAPACK's QR.  BEM2D_ERR_NOCONV if the iteration
 * limit 30 max(10, n) is reached.  A: host or device (not modified);
 * w: host or device. */
int bem2d_eigenvalues(bem2d_ctx* ctx, int n, const void* A, int64_t lda, void* w);

/* w[0..n-1] (complex128) and the right eigenvectors vr (n x n, ldvr,
 * complex128, column i for w[i]) of the general complex A: replaces
 * Eigenvalues(const Matrix&, pcvector&, pMatrix&)
 * (lib/bem2d_mathroutines.cpp:468-528, zgeev with jobvr = 'V').  The
 * reduction's reflectors and the QR rotations are accumulated into the
 * Schur vectors Z (A = Z T Z^H, T upper triangular, w[i] = T(i, i)); the
 * eigenvectors of T by back substitution (ztrevc's scheme), X = Z Y, each
 * column scaled to unit 2-norm with its largest entry real and positive
 * (zgeev's normalisation).  Limits and order as bem2d_eigenvalues; A, w, vr
 * host or device. */
int bem2d_eigenvectors(bem2d_ctx* ctx, int n, const void* A, int64_t lda, void* w, void* vr,
                       int64_t ldvr);

/* lmax[j] = largest eigenvalue of (e^{i th_j} A + e^{-i th_j} A^H) / 2 for
 * nang angles th_j: the eigenvalue step of NumRange
 * (lib/bem2d_mathroutines.cpp:590-653, zheev per angle; the smallest
 * eigenvalue at th is -lmax at th + pi).  Lanczos with full
 * reorthogonalisation, all angles in one block of matrix products; an angle
 * leaves the block once its error estimate min(r, r^2 / gap) is below tol
 * times the size of the Hermitian part seen so far (tol <= 0 selects
 * 1e-13; r the Ritz pair's residual, which bounds the distance to an
 * eigenvalue, gap the distance to the next Ritz value).  BEM2D_PREC_FP64:
 * complex128 throughout.  BEM2D_PREC_MIXED: complex64 Lanczos (cold start)
 * to a residual of 1e-7 |H|, then complex128 Lanczos started from its Ritz
 * vectors, with the complex64 gap estimates (same tolerance). */
int bem2d_num_range(bem2d_ctx* ctx, int n, const void* A, int64_t lda, int nang,
                    const double* theta, double tol, int precision, double* lmax);

/* out[j] = sum_u c_u sum_q K(p_j, y_uq) |J(y_uq)| phi_u(y_uq) w_q: the
 * potential of the density c at npts points p (x0 y0 x1 y1 ...): replaces
 * EvalKernel (lib/bem2d_quadrature.h:184-228; both normals are the source
 * element's, as there).  out is complex128[npts], overwritten. */
int bem2d_eval_kernel(bem2d_ctx* ctx, const bem2d_geometry* geom, const bem2d_quad* quad,
                      int kernel, double k_re, double k_im, double eta, const void* coeffs,
                      int npts, const double* points, void* out);

/* SoundSoftScattering::Discretize() + Solve() in one call
 * (lib/bem2d_soundsoftscattering.h:95-126): A = Id + 2 K_combined(k, eta),
 * b = 2 <CombinedPlaneWave(dir, k, eta), phi_i>, x = A^{-1} b.  A and b stay
 * in the context's device workspace; only x (n_unk complex128) is written.
 * BEM2D_PREC_MIXED assembles with bem2d_discrete_kernel_mixed's arithmetic
 * and solves as bem2d_solve_system's mixed mode (a complex k: FP64 assembly,
 * then the mixed solve). */
int bem2d_scattering_solve(bem2d_ctx* ctx, const bem2d_geometry* geom,
                           const bem2d_quad* quad, double k_re, double k_im,
                           double eta, double dir_x, double dir_y,
                           int precision, double tol, void* x,
                           bem2d_solve_info* info);

/* Batched sweep of nk independent bem2d_scattering_solve problems
 * (geoms[i], k[i], eta[i] or k[i] if eta is NULL; one incident direction):
 * replaces the serial per-wavenumber loop of the reference's sweeps
 * (normcomps/ellipsenormcond.cpp:66-128, which rebuilds the geometry and
 * the system for every k).  nworkers (<= 0: 16) host workers, each with its
 * own streams and workspace, run the problems concurrently, largest first;
 * a worker's factorisation and solve run on a high-priority stream.
 * x[i] (geoms[i].n_unk complex128, host or device) and infos[i] (may be
 * NULL) receive each solution; results equal bem2d_scattering_solve's.
 * Returns when every problem is done; on failure the first error (the
 * message names the problem) and unfinished problems are skipped. */
int bem2d_sweep_solve(bem2d_ctx* ctx, int nk, const bem2d_geometry* geoms,
                      const bem2d_quad* quad, const double* k, const double* eta,
                      double dir_x, double dir_y, int precision, double tol,
                      int nworkers, void* const* x, bem2d_solve_info* infos);

/* ---- measurement helpers (no counterpart in the reference) ------------ */
/* Sustained FMA throughput of the FP64 (BEM2D_PREC_FP64) or FP32
 * (BEM2D_PREC_MIXED) pipe of the current device in TFLOP/s (2 flops per
 * FMA): the roofline denominator of the assembly kernels. */
int bem2d_fma_peak(int precision, double* tflops);

/* Per-phase device timers (CUDA events on the context's stream).  Phases:
 * 0 far-field assembly kernel, 1 near-field kernel, 2 LU factorisation,
 * 3 triangular solves and refinement.  Enabling resets the totals. */
#define BEM2D_PHASE_FAR 0
#define BEM2D_PHASE_NEAR 1
#define BEM2D_PHASE_LU 2
#define BEM2D_PHASE_SOLVE 3
int bem2d_ctx_enable_timers(bem2d_ctx* ctx, int enable);
int bem2d_ctx_timer(const bem2d_ctx* ctx, int phase, double* ms, int64_t* count);

/* Failure-detection check of the bounded device waits (no counterpart in
 * the reference; its LAPACK calls cannot time out).  Runs one complex64 LU
 * panel of order n (256 <= n <= 4096) on the cooperative-grid panel kernel
 * with two blocks whose waits expect a third block's candidate, which is
 * never posted; every wait gives up after `polls` polls and the kernel
 * returns.  Returns BEM2D_ERR_TIMEOUT when the waits gave up (the expected
 * outcome), BEM2D_OK if they did not.  The context stays usable: the next
 * factorisation clears the status word. */
int bem2d_debug_panel_timeout(bem2d_ctx* ctx, int n, int polls);

/* C -= A B for complex64 column-major device matrices (C M x N, A M x K,
 * B K x N) through the complex64 LU's tensor-core trailing update
 * (tcgen05 kind::tf32, 3xTF32 split): the update of zgetrf's right-looking
 * step (lib/bem2d_mathroutines.cpp:345) exposed for its own parity test. */
int bem2d_debug_tc_update(bem2d_ctx* ctx, int M, int N, int K, void* C, int64_t ldc,
                          const void* A, int64_t lda, const void* B, int64_t ldb);

#ifdef __cplusplus
}
#endif
#endif /* BEM2D_GPU_H */
