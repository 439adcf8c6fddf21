// Launch interfaces of dense.cu (dense operators and Lanczos helpers).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace bem2d_gpu {

void launch_change_basis(int n, const double2* K, long long ldk, const int* bstart_of,
                         const int* bsize_of, const double2* uinv, double2* out, long long ldo,
                         cudaStream_t s);
void launch_gather_blocks(int n, const double2* M, long long ldm, const int* bstart_of,
                          const int* bsize_of, double2* blk, cudaStream_t s);
size_t mv_part_bytes(int n);
void launch_mv(const double2* A, long long lda, int n, const double2* x, double2* y,
               double2* part, cudaStream_t s);
void launch_mvh(const double2* A, long long lda, int n, const double2* x, double2* y,
                cudaStream_t s);
// complex64 versions (part: mv_part_bytes(n) bytes suffice)
void launch_mv(const float2* A, long long lda, int n, const float2* x, float2* y, float2* part,
               cudaStream_t s);
void launch_mvh(const float2* A, long long lda, int n, const float2* x, float2* y,
                cudaStream_t s);
// C (n x m, ldc) = op(A) B, op = A or A^H (herm).  work: room for the K-split
// partial products (zgemm_work_bytes); with less, one pass over K.
void launch_zgemm(bool herm, const double2* A, long long lda, int n, const double2* B,
                  long long ldb, int m, double2* C, long long ldc, void* work,
                  size_t work_bytes, cudaStream_t s);
void launch_zgemm(bool herm, const float2* A, long long lda, int n, const float2* B,
                  long long ldb, int m, float2* C, long long ldc, void* work,
                  size_t work_bytes, cudaStream_t s);
size_t zgemm_work_bytes(int n, int m, size_t elem);
// C (n x m, ldc) = op(A) B in float-float on the FP32 pipe (~1e-13 relative
// to |A| |B|): A (n x n) given as hi = fl32(A), lo = fl32(A - hi), ld n;
// B, C complex128.  work: zgemm_work_bytes(n, m, sizeof(double2));
// bsplit: 2 n m float2 of scratch for B's split.
void launch_zgemm_ff(bool herm, const float2* Ahi, const float2* Alo, int n, const double2* B,
                     long long ldb, int m, double2* C, long long ldc, void* work,
                     size_t work_bytes, float2* bsplit, cudaStream_t s);
// hi / lo (n x n, ld n) = the float-float split of A (complex128, ld lda)
void launch_split_ff(const double2* A, long long lda, int n, float2* hi, float2* lo,
                     cudaStream_t s);
// C (rows x m, ldc) = A (rows x k, lda) B (k x m, ldb), complex128
void launch_zgemm_rect(const double2* A, long long lda, int rows, int k, const double2* B,
                       long long ldb, int m, double2* C, long long ldc, cudaStream_t s);
#define BEM2D_BATCHED_DECLS(T)                                                                \
  void launch_batched_dots(const T* Q, long long qstride, int n, int j, const T* W,           \
                           long long wstride, T* h, int ldh, int nb, cudaStream_t s);         \
  void launch_batched_sub(const T* Q, long long qstride, int n, int j, T* W, long long wstride, \
                          const T* h, int ldh, int nb, cudaStream_t s);                       \
  void launch_batched_norm2(int n, const T* W, long long wstride, double* out, int nb,        \
                            cudaStream_t s);                                                  \
  void launch_batched_scale(int n, const T* src, long long sstride, const double* scale,      \
                            T* dst, long long dstride, int nb, cudaStream_t s);               \
  void launch_herm_combine(int n, const T* Y1, const T* Y2, long long stride,                 \
                           const double* theta, T* W, long long wstride, int nb, cudaStream_t s); \
  /* dst slot i (stride dstride) = the first len entries of src slot map[i] */               \
  void launch_gather_slots(const T* src, long long sstride, T* dst, long long dstride,        \
                           long long len, const int* map, int nmap, cudaStream_t s);          \
  /* dst slot map[i] = the first len entries of src slot i */                                \
  void launch_scatter_slots(const T* src, long long sstride, T* dst, long long dstride,       \
                            long long len, const int* map, int nmap, cudaStream_t s);
BEM2D_BATCHED_DECLS(double2)
BEM2D_BATCHED_DECLS(float2)
#undef BEM2D_BATCHED_DECLS
// dst (complex128) = src (complex64), nb columns of n
void launch_widen(int n, const float2* src, long long sstride, double2* dst, long long dstride,
                  int nb, cudaStream_t s);
void launch_axpy_real(int n, double a, const double2* x, double2* y, cudaStream_t s);
bool tridiag_eigenvalues(std::vector<double> d, std::vector<double> e, std::vector<double>* ev);
// Largest eigenvalue of the symmetric tridiagonal (d, e) (e: n-1 entries).
double tridiag_lmax(const std::vector<double>& d, const std::vector<double>& e);
// Largest eigenvalue given a lower bound lo (for a Lanczos tridiagonal, the
// previous step's value: Ritz values interlace) and a guess of the distance
// to it: the step grows fourfold until lo + step bounds the spectrum, then
// bisection to max(atol, 2.2e-16 times the Gershgorin bound); returns the
// lower end of the final bracket, so a result is again a valid lower bound
// (a value above the true one would stall the next calls at itself).  Far
// fewer Sturm sweeps than bisection from the Gershgorin interval once the
// value has settled.
double tridiag_lmax_from(const std::vector<double>& d, const std::vector<double>& e, double lo,
                         double step, double atol);
// k-th largest eigenvalue (k = 1: the largest) by Sturm bisection, to rel
// times the Gershgorin bound of the spectrum.
double tridiag_kth_largest(const std::vector<double>& d, const std::vector<double>& e, int k,
                           double rel);
// Unit eigenvector of the symmetric tridiagonal (d, e) for its eigenvalue
// lambda (inverse iteration).
std::vector<double> tridiag_eigenvector(const std::vector<double>& d, const std::vector<double>& e,
                                        double lambda);

}  // namespace bem2d_gpu
