// sod_dense.h -- cuSOLVER / cuBLAS entry points of the dense solves (LU, Cholesky, FP64 GEMM).
//
// Both libraries are loaded with dlopen at first use, so only the dense-solve entry points depend on
// them; the assembly, transform and history paths never load them.
#pragma once
#include <cublas_api.h>
#include <cusolverDn.h>

#include <string>

#include "sod_internal.h"

namespace sod {

struct DenseApi {
    // cuSOLVER (dense)
    cusolverStatus_t (*dn_create)(cusolverDnHandle_t *) = nullptr;
    cusolverStatus_t (*dn_destroy)(cusolverDnHandle_t) = nullptr;
    cusolverStatus_t (*dn_set_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
    cusolverStatus_t (*getrf_buf)(cusolverDnHandle_t, int, int, double *, int, int *) = nullptr;
    cusolverStatus_t (*getrf)(cusolverDnHandle_t, int, int, double *, int, double *, int *, int *) = nullptr;
    cusolverStatus_t (*getrs)(cusolverDnHandle_t, cublasOperation_t, int, int, const double *, int, const int *,
                              double *, int, int *) = nullptr;
    cusolverStatus_t (*potrf_buf)(cusolverDnHandle_t, cublasFillMode_t, int, double *, int, int *) = nullptr;
    cusolverStatus_t (*potrf)(cusolverDnHandle_t, cublasFillMode_t, int, double *, int, double *, int, int *) = nullptr;
    cusolverStatus_t (*potrs)(cusolverDnHandle_t, cublasFillMode_t, int, int, const double *, int, double *, int,
                              int *) = nullptr;
    // cuBLAS
    cublasStatus_t (*blas_create)(cublasHandle_t *) = nullptr;
    cublasStatus_t (*blas_destroy)(cublasHandle_t) = nullptr;
    cublasStatus_t (*blas_set_stream)(cublasHandle_t, cudaStream_t) = nullptr;
    cublasStatus_t (*dgemm)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int, const double *,
                            const double *, int, const double *, int, const double *, double *, int) = nullptr;
    cublasStatus_t (*dsyrk)(cublasHandle_t, cublasFillMode_t, cublasOperation_t, int, int, const double *,
                            const double *, int, const double *, double *, int) = nullptr;
    bool solver_ok = false, blas_ok = false;
    std::string why_solver, why_blas;
};
const DenseApi &dense_api();

// out[c][r] = in[r][c] for an R x C row-major FP64 matrix, on the context's stream
int transpose_f64(sod_context *ctx, const double *in, int R, int C, double *out);

}  // namespace sod
