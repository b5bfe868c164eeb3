// sod_solve.cu -- dense LU solves downstream of the assembly, on the device.
//
// Replaces the Eigen::PartialPivLU uses of ElastodynamicsCQBEMMatrixCollection::init
// (src/elastodynamics_cqbem_matrix_collection.cpp:200-214: H_inv.compute(H_0), u_p = H_inv.solve(G'),
// H_inv_B_trans, H_inv_B_euler, H_inv.inverse()) and the per-step u = H_inv.solve(b) of
// ElastodynamicsCQBEMObject (src/elastodynamics_cqbem_object.cpp:63), fused after the history
// convolution so the served time step stays on the device.
//
// The factorisation is LU with partial pivoting in FP64 (P A = L U on the row-major matrix, with
// LAPACK's pivot choice; sod_dense_kernels.cu).
#include <memory>
#include <string>

#include "sod_dense.h"

using namespace sod;

namespace {

// X[r][j] = sum_c Ai[r][c] B[c][j] (FP64): one warp per row, lanes over the columns in a fixed
// stride, FP64 xor tree over the lanes (deterministic).  B (n x R) stays in L2.
template <int R>
__global__ void __launch_bounds__(256) inv_gemv_kernel(const double *__restrict__ Ai, const double *__restrict__ B,
                                                       int n, double *__restrict__ X) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    const double *a = Ai + (size_t)row * n;
    double acc[R];
#pragma unroll
    for (int j = 0; j < R; j++) acc[j] = 0.0;
    for (int c = lane; c < n; c += 32) {
        const double v = __ldg(a + c);
#pragma unroll
        for (int j = 0; j < R; j++) acc[j] = fma(v, __ldg(B + (size_t)c * R + j), acc[j]);
    }
#pragma unroll
    for (int j = 0; j < R; j++) {
        double v = acc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) X[(size_t)row * R + j] = v;
    }
}

__global__ void identity_kernel(double *I, int n) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < (size_t)n * n) I[e] = (e / n == e % n) ? 1.0 : 0.0;
}

}  // namespace

struct sod_solver {
    sod_context *ctx = nullptr;
    int n = 0;
    DevBuf lu, ipiv, perm, info, rhs, tmp;
    DevBuf inv;         // A^-1 (row-major) once sod_solver_keep_inverse ran
    bool has_inv = false;
};

namespace sod {
int solver_size(const sod_solver *s) { return s->n; }
// per-step form: with a kept inverse, X = A^-1 B as an FP64 GEMV (one pass over A^-1) instead of
// the two triangular solves; X must not alias B
int solver_apply_device(sod_solver *s, int nrhs, const double *B, double *X) {
    if (!s->has_inv || (nrhs != 1 && nrhs != 16)) return solver_solve_device(s, nrhs, B, X);
    sod_context *ctx = s->ctx;
    const int blocks = (int)(((long long)s->n * 32 + 255) / 256);
    if (nrhs == 1)
        inv_gemv_kernel<1><<<blocks, 256, 0, ctx->stream>>>(s->inv.as<double>(), B, s->n, X);
    else
        inv_gemv_kernel<16><<<blocks, 256, 0, ctx->stream>>>(s->inv.as<double>(), B, s->n, X);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}
// X (row-major n x nrhs, device) = A^-1 B (row-major n x nrhs, device); X may alias B
int solver_solve_device(sod_solver *s, int nrhs, const double *B, double *X) {
    sod_context *ctx = s->ctx;
    const int n = s->n;
    const size_t bytes = sizeof(double) * (size_t)n * nrhs;
    if (X != B) return lu_solve(ctx, s->lu.as<double>(), n, s->perm.as<int>(), nrhs, B, X);
    SOD_TRY(s->rhs.ensure(bytes));
    SOD_TRY(lu_solve(ctx, s->lu.as<double>(), n, s->perm.as<int>(), nrhs, B, s->rhs.as<double>()));
    SOD_CHECK_CUDA(cudaMemcpyAsync(X, s->rhs.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return SOD_OK;
}
}  // namespace sod

extern "C" {

int sod_solver_create(sod_context *ctx, int n, const double *A, sod_solver **out) {
    SOD_REQUIRE(ctx && A && out, "null argument");
    SOD_REQUIRE(n >= 1, "matrix size must be >= 1");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    auto s = std::make_unique<sod_solver>();
    s->ctx = ctx;
    s->n = n;
    const size_t bytes = sizeof(double) * (size_t)n * n;
    SOD_TRY(s->lu.ensure(bytes));
    SOD_CHECK_CUDA(cudaMemcpyAsync(s->lu.p, A, bytes, cudaMemcpyDefault, ctx->stream));
    SOD_TRY(s->ipiv.ensure(sizeof(int) * (size_t)n));
    SOD_TRY(s->perm.ensure(sizeof(int) * (size_t)n));
    SOD_TRY(s->info.ensure(sizeof(int)));
    SOD_TRY(lu_factor(ctx, s->lu.as<double>(), n, s->ipiv.as<int>(), s->perm.as<int>(), s->info.as<int>()));
    int info = 0;
    SOD_CHECK_CUDA(cudaMemcpyAsync(&info, s->info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    if (info != 0) {
        set_error("LU factorisation: the matrix is singular (zero pivot " + std::to_string(info) + ")");
        return SOD_ERR_INVALID_ARG;
    }
    *out = s.release();
    return SOD_OK;
}

int sod_solver_solve(sod_solver *s, int nrhs, const double *B, double *X) {
    SOD_REQUIRE(s && B && X, "null argument");
    SOD_REQUIRE(nrhs >= 1, "nrhs must be >= 1");
    sod_context *ctx = s->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t bytes = sizeof(double) * (size_t)s->n * nrhs;
    const bool hb = !is_device_pointer(B), hx = !is_device_pointer(X);
    const double *db = B;
    double *dx = X;
    if (hb || hx) SOD_TRY(s->tmp.ensure(bytes));
    if (hb) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(s->tmp.p, B, bytes, cudaMemcpyHostToDevice, ctx->stream));
        db = s->tmp.as<double>();
    }
    if (hx) dx = s->tmp.as<double>();
    SOD_TRY(solver_solve_device(s, nrhs, db, dx));
    if (hx) SOD_CHECK_CUDA(cudaMemcpyAsync(X, dx, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (hb || hx) SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return SOD_OK;
}

int sod_solver_inverse(sod_solver *s, double *Ainv) {
    SOD_REQUIRE(s && Ainv, "null argument");
    sod_context *ctx = s->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const int n = s->n;
    const size_t bytes = sizeof(double) * (size_t)n * n;
    const bool host = !is_device_pointer(Ainv);
    double *d = Ainv;
    if (host) {
        SOD_TRY(ctx->staging.ensure(bytes));
        d = ctx->staging.as<double>();
    }
    const size_t nn = (size_t)n * n;
    SOD_TRY(s->rhs.ensure(bytes));
    identity_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx->stream>>>(s->rhs.as<double>(), n);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    SOD_TRY(lu_solve(ctx, s->lu.as<double>(), n, s->perm.as<int>(), n, s->rhs.as<double>(), d));  // A X = I
    if (host) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(Ainv, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return SOD_OK;
}

int sod_solver_keep_inverse(sod_solver *s) {
    SOD_REQUIRE(s, "null solver");
    if (s->has_inv) return SOD_OK;
    SOD_CHECK_CUDA(cudaSetDevice(s->ctx->device));
    SOD_TRY(s->inv.ensure(sizeof(double) * (size_t)s->n * s->n));
    SOD_TRY(sod_solver_inverse(s, s->inv.as<double>()));
    s->has_inv = true;
    return SOD_OK;
}

int sod_solver_destroy(sod_solver *s) {
    if (s) {
        cudaSetDevice(s->ctx->device);
        delete s;
    }
    return SOD_OK;
}

}  // extern "C"
