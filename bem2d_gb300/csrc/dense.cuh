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
void launch_zgemm(bool herm, const double2* A, long long lda, int n, const double2* B,
                  long long ldb, int m, double2* C, long long ldc, cudaStream_t s);
void launch_batched_dots(const double2* Q, long long qstride, int n, int j, const double2* W,
                         long long wstride, double2* h, int ldh, int nb, cudaStream_t s);
void launch_batched_sub(const double2* Q, long long qstride, int n, int j, double2* W,
                        long long wstride, const double2* h, int ldh, int nb, cudaStream_t s);
void launch_batched_norm2(int n, const double2* W, long long wstride, double* out, int nb,
                          cudaStream_t s);
void launch_batched_scale(int n, const double2* src, long long sstride, const double* scale,
                          double2* dst, long long dstride, int nb, cudaStream_t s);
void launch_herm_combine(int n, const double2* Y1, const double2* Y2, long long stride,
                         const double* theta, double2* W, long long wstride, int nb,
                         cudaStream_t s);
void launch_axpy_real(int n, double a, const double2* x, double2* y, cudaStream_t s);
bool tridiag_eigenvalues(std::vector<double> d, std::vector<double> e, std::vector<double>* ev);

}  // namespace bem2d_gpu
