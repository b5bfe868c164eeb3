// sod_dense.h -- FP64 dense linear algebra of the solves (sod_dense_kernels.cu): GEMM, LU with partial
// pivoting, Cholesky and their triangular solves.  Row-major device buffers, work on the context's
// stream.
#pragma once
#include "sod_internal.h"

namespace sod {

// C[M x N] = alpha op(A) op(B) + beta C, op(X) = X^T when the flag is set (row-major storage, leading
// dimensions in elements).  lower_only: only the lower triangle (and the diagonal tiles) of C.
int dgemm(sod_context *ctx, bool ta, bool tb, int M, int N, int K, double alpha, const double *A, long long lda,
          const double *B, long long ldb, double beta, double *C, long long ldc, bool lower_only);
// P A = L U in place (unit lower L below the diagonal, U on and above); ipiv[i] = the row interchanged
// with row i at step i; perm[i] = the original row now at position i; *info = 1-based index of the
// first exactly zero pivot, 0 if none (device ints)
int lu_factor(sod_context *ctx, double *A, int n, int *ipiv, int *perm, int *info);
// X = A^-1 B (n x nrhs); X must not alias B
int lu_solve(sod_context *ctx, const double *LU, int n, const int *perm, int nrhs, const double *B, double *X);
// A = L L^T in place from A's lower triangle; *info = 1-based column of the first non-positive pivot
int chol_factor(sod_context *ctx, double *A, int n, int *info);
// X = A^-1 B for the factored A (n x nrhs); X may alias B
int chol_solve(sod_context *ctx, const double *L, int n, int nrhs, const double *B, double *X);

}  // namespace sod
