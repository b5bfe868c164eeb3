// sod_solve.cu -- dense LU solves downstream of the assembly, on the device.
//
// Replaces the Eigen::PartialPivLU uses of ElastodynamicsCQBEMMatrixCollection::init
// (src/elastodynamics_cqbem_matrix_collection.cpp:200-214: H_inv.compute(H_0), u_p = H_inv.solve(G'),
// H_inv_B_trans, H_inv_B_euler, H_inv.inverse()) and the per-step u = H_inv.solve(b) of
// ElastodynamicsCQBEMObject (src/elastodynamics_cqbem_object.cpp:63), fused after the history
// convolution so the served time step stays on the device.
//
// The factorisation is LAPACK-style LU with partial pivoting in FP64 (cuSOLVER getrf / getrs: a plain
// library factorisation; the library is loaded at first use, so the rest of this library does not
// depend on it).  Matrices are row-major at the interface; a row-major A is the column-major A^T, so
// the buffer is factored as it is (P A^T = L U) and solves use the transposed form, A X = B.
// Right-hand sides are transposed to column-major and back by a tiled shared-memory kernel.
#include <dlfcn.h>

#include <mutex>
#include <string>

#include "sod_dense.h"

using namespace sod;

namespace sod {

const DenseApi &dense_api() {
    static DenseApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        auto open = [](const char *const *names, int n) -> void * {
            for (int i = 0; i < n; i++)
                if (void *h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL)) return h;
            return nullptr;
        };
        const char *sol[] = {"libcusolver.so.12", "libcusolver.so", "/usr/local/cuda/lib64/libcusolver.so.12"};
        if (void *h = open(sol, 3)) {
            auto sym = [&](const char *s) { return dlsym(h, s); };
            api.dn_create = reinterpret_cast<decltype(api.dn_create)>(sym("cusolverDnCreate"));
            api.dn_destroy = reinterpret_cast<decltype(api.dn_destroy)>(sym("cusolverDnDestroy"));
            api.dn_set_stream = reinterpret_cast<decltype(api.dn_set_stream)>(sym("cusolverDnSetStream"));
            api.getrf_buf = reinterpret_cast<decltype(api.getrf_buf)>(sym("cusolverDnDgetrf_bufferSize"));
            api.getrf = reinterpret_cast<decltype(api.getrf)>(sym("cusolverDnDgetrf"));
            api.getrs = reinterpret_cast<decltype(api.getrs)>(sym("cusolverDnDgetrs"));
            api.potrf_buf = reinterpret_cast<decltype(api.potrf_buf)>(sym("cusolverDnDpotrf_bufferSize"));
            api.potrf = reinterpret_cast<decltype(api.potrf)>(sym("cusolverDnDpotrf"));
            api.potrs = reinterpret_cast<decltype(api.potrs)>(sym("cusolverDnDpotrs"));
            api.solver_ok = api.dn_create && api.dn_destroy && api.dn_set_stream && api.getrf_buf && api.getrf &&
                            api.getrs && api.potrf_buf && api.potrf && api.potrs;
            if (!api.solver_ok) api.why_solver = "cuSOLVER is missing dense LU / Cholesky entry points";
        } else {
            api.why_solver = std::string("cuSOLVER not found (") + dlerror() + ")";
        }
        const char *blas[] = {"libcublas.so.13", "libcublas.so", "/usr/local/cuda/lib64/libcublas.so.13"};
        if (void *h = open(blas, 3)) {
            auto sym = [&](const char *s) { return dlsym(h, s); };
            api.blas_create = reinterpret_cast<decltype(api.blas_create)>(sym("cublasCreate_v2"));
            api.blas_destroy = reinterpret_cast<decltype(api.blas_destroy)>(sym("cublasDestroy_v2"));
            api.blas_set_stream = reinterpret_cast<decltype(api.blas_set_stream)>(sym("cublasSetStream_v2"));
            api.dgemm = reinterpret_cast<decltype(api.dgemm)>(sym("cublasDgemm_v2"));
            api.dsyrk = reinterpret_cast<decltype(api.dsyrk)>(sym("cublasDsyrk_v2"));
            api.blas_ok = api.blas_create && api.blas_destroy && api.blas_set_stream && api.dgemm && api.dsyrk;
            if (!api.blas_ok) api.why_blas = "cuBLAS is missing FP64 GEMM entry points";
        } else {
            api.why_blas = std::string("cuBLAS not found (") + dlerror() + ")";
        }
    });
    return api;
}

}  // namespace sod

namespace {

// out[c][r] = in[r][c] for an R x C row-major matrix (32 x 32 tiles through shared memory)
__global__ void transpose_kernel(const double *__restrict__ in, int R, int C, double *__restrict__ out) {
    __shared__ double tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        if (r < R && c < C) tile[k][threadIdx.x] = in[(size_t)r * C + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (r < R && c < C) out[(size_t)c * R + r] = tile[threadIdx.x][k];
    }
}


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

int sod::transpose_f64(sod_context *ctx, const double *in, int R, int C, double *out) {
    const dim3 grid((C + 31) / 32, (R + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, ctx->stream>>>(in, R, C, out);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

struct sod_solver {
    sod_context *ctx = nullptr;
    int n = 0;
    cusolverDnHandle_t h = nullptr;
    DevBuf lu, ipiv, info, work, rhs, tmp;
    DevBuf inv;         // A^-1 (row-major) once sod_solver_keep_inverse ran
    bool has_inv = false;
    ~sod_solver() {
        if (h) dense_api().dn_destroy(h);
    }
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
    const DenseApi &api = dense_api();
    const size_t bytes = sizeof(double) * (size_t)n * nrhs;
    SOD_TRY(s->rhs.ensure(bytes));
    double *cm = s->rhs.as<double>();
    if (nrhs == 1) {
        if (cm != B) SOD_CHECK_CUDA(cudaMemcpyAsync(cm, B, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SOD_TRY(transpose_f64(ctx, B, n, nrhs, cm));  // -> column-major n x nrhs
    }
    if (api.getrs(s->h, CUBLAS_OP_T, n, nrhs, s->lu.as<double>(), n, s->ipiv.as<int>(), cm, n, s->info.as<int>()) !=
        CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDgetrs failed");
        return SOD_ERR_CUDA;
    }
    ctx->count();
    if (nrhs == 1) {
        if (X != cm) SOD_CHECK_CUDA(cudaMemcpyAsync(X, cm, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        SOD_TRY(transpose_f64(ctx, cm, nrhs, n, X));  // column-major n x nrhs is row-major nrhs x n
    }
    return SOD_OK;
}
}  // namespace sod

extern "C" {

int sod_solver_create(sod_context *ctx, int n, const double *A, sod_solver **out) {
    SOD_REQUIRE(ctx && A && out, "null argument");
    SOD_REQUIRE(n >= 1, "matrix size must be >= 1");
    const DenseApi &api = dense_api();
    if (!api.solver_ok) {
        set_error(api.why_solver);
        return SOD_ERR_UNSUPPORTED;
    }
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    auto s = std::make_unique<sod_solver>();
    s->ctx = ctx;
    s->n = n;
    if (api.dn_create(&s->h) != CUSOLVER_STATUS_SUCCESS || api.dn_set_stream(s->h, ctx->stream) != CUSOLVER_STATUS_SUCCESS) {
        s->h = nullptr;
        set_error("cusolverDnCreate failed");
        return SOD_ERR_CUDA;
    }
    const size_t bytes = sizeof(double) * (size_t)n * n;
    SOD_TRY(s->lu.ensure(bytes));
    SOD_CHECK_CUDA(cudaMemcpyAsync(s->lu.p, A, bytes, cudaMemcpyDefault, ctx->stream));
    SOD_TRY(s->ipiv.ensure(sizeof(int) * (size_t)n));
    SOD_TRY(s->info.ensure(sizeof(int)));
    int lwork = 0;
    if (api.getrf_buf(s->h, n, n, s->lu.as<double>(), n, &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDgetrf_bufferSize failed");
        return SOD_ERR_CUDA;
    }
    SOD_TRY(s->work.ensure(sizeof(double) * (size_t)std::max(lwork, 1)));
    // the row-major buffer is the column-major A^T: P A^T = L U
    if (api.getrf(s->h, n, n, s->lu.as<double>(), n, s->work.as<double>(), s->ipiv.as<int>(), s->info.as<int>()) !=
        CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDgetrf failed");
        return SOD_ERR_CUDA;
    }
    ctx->count();
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
    identity_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx->stream>>>(d, n);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    SOD_TRY(solver_solve_device(s, n, d, d));  // A X = I, row-major
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
