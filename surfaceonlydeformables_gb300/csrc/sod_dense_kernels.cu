// sod_dense_kernels.cu -- FP64 dense linear algebra of the solves downstream of the assembly:
// GEMM, LU with partial pivoting and its solves, Cholesky and its solves.  Row-major throughout.
//
// GB300 runs FP64 at about 4 flop per clock per SM (1/64 of the FP32 rate), so these kernels are
// bound by the FP64 pipe, not by memory: a 64 x 64 output tile per CTA with a 4 x 4 register tile
// per thread reads 16 KB of operands per 16 K-columns from shared memory against 65536 FP64 FMAs,
// which keeps the pipe busy with any occupancy above one CTA per SM.
//
// LU (P A = L U, the factorisation of Eigen::PartialPivLU / LAPACK getrf): right-looking, 64-column
// panels.  A panel is factored recursively (left half, triangular solve of the right half's top rows,
// GEMM update of the right half, right half), down to 8-column leaves factored by one CTA: pivot search
// over the leaf's column (largest magnitude, smallest row index on ties, as LAPACK's idamax), swap of
// the two whole rows (all n columns, so the interchanges reach the factored and the trailing parts
// at once), scaling by the pivot and the rank-1 updates of the leaf.  After each panel the trailing
// matrix is updated by a triangular solve (U12 = L11^-1 A12) and a GEMM (A22 -= L21 U12).
// Cholesky (A = L L^T, the regularised elastostatic system): the same blocking without pivoting.
// The solves are blocked right-looking substitutions: each diagonal block is solved, then the rows
// below (or above) are updated by one GEMM, which spreads the work over the whole GPU even for one
// right-hand side.  Every sum runs in a fixed order, so results are deterministic.
#include <algorithm>

#include "sod_dense.h"

namespace sod {
namespace {

constexpr int GT = 64;  // GEMM output tile
constexpr int GK = 16;  // GEMM K step

// C[M x N] = alpha op(A) op(B) + beta C.  op(A)[i][k] = TA ? A[k * lda + i] : A[i * lda + k];
// op(B)[k][j] = TB ? B[j * ldb + k] : B[k * ldb + j].  256 threads, 4 x 4 outputs each.
// LOWER: only tiles with a row block >= the column block are computed (the lower triangle of a
// symmetric product, diagonal tiles in full).
template <bool TA, bool TB, bool LOWER>
__global__ void __launch_bounds__(256) dgemm_kernel(int M, int N, int K, double alpha, const double *__restrict__ A,
                                                    long long lda, const double *__restrict__ B, long long ldb,
                                                    double beta, double *__restrict__ C, long long ldc) {
    const int bm = blockIdx.y, bn = blockIdx.x;
    if (LOWER && bn > bm) return;
    __shared__ double As[GK][GT + 1];
    __shared__ double Bs[GK][GT + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = bm * GT, j0 = bn * GT;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
    for (int k0 = 0; k0 < K; k0 += GK) {
        // 64 x 16 tile of op(A) and 16 x 64 tile of op(B), 4 elements per thread each
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int e = tid + 256 * t;
            int i, k;
            if (TA) {  // contiguous along i
                i = e & 63, k = e >> 6;
            } else {  // contiguous along k
                k = e & 15, i = e >> 4;
            }
            const int gi = i0 + i, gk = k0 + k;
            As[k][i] = (gi < M && gk < K) ? (TA ? A[(long long)gk * lda + gi] : A[(long long)gi * lda + gk]) : 0.0;
            int j, kb;
            if (TB) {  // contiguous along k
                kb = e & 15, j = e >> 4;
            } else {  // contiguous along j
                j = e & 63, kb = e >> 6;
            }
            const int gj = j0 + j, gkb = k0 + kb;
            Bs[kb][j] = (gj < N && gkb < K) ? (TB ? B[(long long)gj * ldb + gkb] : B[(long long)gkb * ldb + gj]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < GK; k++) {
            double a[4], b[4];
#pragma unroll
            for (int t = 0; t < 4; t++) a[t] = As[k][ty * 4 + t], b[t] = Bs[k][tx * 4 + t];
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = fma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const int gi = i0 + ty * 4 + p;
        if (gi >= M) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int gj = j0 + tx * 4 + q;
            if (gj >= N) continue;
            double *c = C + (long long)gi * ldc + gj;
            *c = beta == 0.0 ? alpha * acc[p][q] : fma(alpha, acc[p][q], beta * *c);
        }
    }
}

// The same product for thin shapes (fewer than 32 rows or columns: the updates of the right-hand sides
// and of the narrow panel halves): one thread per output element, K summed in order.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) dgemm_small_kernel(int M, int N, int K, double alpha, const double *__restrict__ A,
                                                          long long lda, const double *__restrict__ B, long long ldb,
                                                          double beta, double *__restrict__ C, long long ldc) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)M * N) return;
    const int i = (int)(e / N), j = (int)(e % N);
    double acc = 0.0;
    for (int k = 0; k < K; k++) {
        const double a = TA ? A[(long long)k * lda + i] : A[(long long)i * lda + k];
        const double b = TB ? B[(long long)j * ldb + k] : B[(long long)k * ldb + j];
        acc = fma(a, b, acc);
    }
    double *c = C + (long long)i * ldc + j;
    *c = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * *c);
}

// ---- LU leaf: columns [c0, c0 + w) of rows [c0, n), one CTA --------------------------------------------
constexpr int LEAF = 8;
constexpr int LEAF_THREADS = 1024;

__global__ void __launch_bounds__(LEAF_THREADS) lu_leaf_kernel(double *__restrict__ A, int n, long long lda, int c0,
                                                               int w, int *__restrict__ ipiv, int *__restrict__ info) {
    __shared__ double wv[32];
    __shared__ int wi[32];
    __shared__ double prow[LEAF];
    __shared__ int piv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = c0; c < c0 + w; c++) {
        // pivot: largest |A[r][c]| over r >= c, smallest r on ties
        double best = -1.0;
        int br = n;
        for (int r = c + tid; r < n; r += LEAF_THREADS) {
            const double v = fabs(A[(long long)r * lda + c]);
            if (v > best) best = v, br = r;  // rows visited in increasing order: the first maximum stays
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int orow = __shfl_xor_sync(0xffffffffu, br, o);
            if (ov > best || (ov == best && orow < br)) best = ov, br = orow;
        }
        if (lane == 0) wv[warp] = best, wi[warp] = br;
        __syncthreads();
        if (tid == 0) {
            double b = wv[0];
            int r = wi[0];
            for (int k = 1; k < LEAF_THREADS / 32; k++)
                if (wv[k] > b || (wv[k] == b && wi[k] < r)) b = wv[k], r = wi[k];
            if (r >= n) r = c;
            piv = r;
            ipiv[c] = r;
            if (b == 0.0 && *info == 0) *info = c + 1;  // exactly singular: the first zero pivot, 1-based
        }
        __syncthreads();
        const int p = piv;
        if (p != c)  // interchange the whole rows
            for (int j = tid; j < n; j += LEAF_THREADS) {
                const double t = A[(long long)c * lda + j];
                A[(long long)c * lda + j] = A[(long long)p * lda + j];
                A[(long long)p * lda + j] = t;
            }
        __syncthreads();
        const double d = A[(long long)c * lda + c];
        if (tid < c0 + w - c - 1) prow[tid] = A[(long long)c * lda + c + 1 + tid];
        __syncthreads();
        if (d != 0.0) {
            const double rd = 1.0 / d;
            const int nj = c0 + w - c - 1;
            for (int r = c + 1 + tid; r < n; r += LEAF_THREADS) {
                double *row = A + (long long)r * lda;
                const double l = row[c] * rd;
                row[c] = l;
                for (int j = 0; j < nj; j++) row[c + 1 + j] = fma(-l, prow[j], row[c + 1 + j]);
            }
        }
        __syncthreads();
    }
}

// ---- triangular solves on a diagonal block (w <= W), L or U in shared memory ---------------------------
// X = L^-1 X for the w x w unit lower triangle at T (ld ldt), X = rows [0, w) x columns [0, ncol) at X
// (ld ldx); one thread per column.
template <int W>
__global__ void __launch_bounds__(256) trsm_unit_lower_kernel(const double *__restrict__ T, long long ldt, int w,
                                                              double *__restrict__ X, long long ldx, int ncol) {
    __shared__ double Ls[W][W + 1];
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) Ls[e / w][e % w] = T[(long long)(e / w) * ldt + e % w];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncol) return;
    double x[W];
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) x[i] = X[(long long)i * ldx + j];
#pragma unroll
    for (int i = 0; i < W; i++) {
        if (i >= w) break;
        double s = x[i];
#pragma unroll
        for (int k = 0; k < W; k++)
            if (k < i) s = fma(-Ls[i][k], x[k], s);
        x[i] = s;
    }
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) X[(long long)i * ldx + j] = x[i];
}

// X = U^-1 X for the w x w non-unit upper triangle at T (ld ldt); one thread per column.
template <int W>
__global__ void __launch_bounds__(256) trsm_upper_kernel(const double *__restrict__ T, long long ldt, int w,
                                                         double *__restrict__ X, long long ldx, int ncol) {
    __shared__ double Us[W][W + 1];
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) Us[e / w][e % w] = T[(long long)(e / w) * ldt + e % w];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncol) return;
    double x[W];
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) x[i] = X[(long long)i * ldx + j];
#pragma unroll
    for (int ii = W - 1; ii >= 0; ii--) {
        if (ii >= w) continue;
        double s = x[ii];
#pragma unroll
        for (int k = 0; k < W; k++)
            if (k > ii && k < w) s = fma(-Us[ii][k], x[k], s);
        x[ii] = s / Us[ii][ii];
    }
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) X[(long long)i * ldx + j] = x[i];
}

// X = L^-1 X (TRANS false) or X = L^-T X (TRANS true) for the non-unit lower (Cholesky) triangle L
template <bool TRANS, int W>
__global__ void __launch_bounds__(256) trsm_chol_kernel(const double *__restrict__ T, long long ldt, int w,
                                                        double *__restrict__ X, long long ldx, int ncol) {
    __shared__ double Ls[W][W + 1];
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) Ls[e / w][e % w] = T[(long long)(e / w) * ldt + e % w];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncol) return;
    double x[W];
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) x[i] = X[(long long)i * ldx + j];
    if (!TRANS) {
#pragma unroll
        for (int i = 0; i < W; i++) {
            if (i >= w) break;
            double s = x[i];
#pragma unroll
            for (int k = 0; k < W; k++)
                if (k < i) s = fma(-Ls[i][k], x[k], s);
            x[i] = s / Ls[i][i];
        }
    } else {  // L^T is upper: (L^T)[i][k] = L[k][i]
#pragma unroll
        for (int ii = W - 1; ii >= 0; ii--) {
            if (ii >= w) continue;
            double s = x[ii];
#pragma unroll
            for (int k = 0; k < W; k++)
                if (k > ii && k < w) s = fma(-Ls[k][ii], x[k], s);
            x[ii] = s / Ls[ii][ii];
        }
    }
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) X[(long long)i * ldx + j] = x[i];
}

// L21 = A21 L11^-T: each row x of A21 (nrow x w at X, ld ldx) solves y L11^T = x, i.e. L11 y^T = x^T
// (forward substitution with the non-unit lower L11); one thread per row.
template <int W>
__global__ void __launch_bounds__(128) trsm_right_lt_kernel(const double *__restrict__ T, long long ldt, int w,
                                                            double *__restrict__ X, long long ldx, int nrow) {
    __shared__ double Ls[W][W + 1];
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) Ls[e / w][e % w] = T[(long long)(e / w) * ldt + e % w];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrow) return;
    double *row = X + (long long)r * ldx;
    double x[W];
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) x[i] = row[i];
#pragma unroll
    for (int i = 0; i < W; i++) {
        if (i >= w) break;
        double s = x[i];
#pragma unroll
        for (int k = 0; k < W; k++)
            if (k < i) s = fma(-Ls[i][k], x[k], s);
        x[i] = s / Ls[i][i];
    }
#pragma unroll
    for (int i = 0; i < W; i++)
        if (i < w) row[i] = x[i];
}

// Cholesky of the w x w (w <= 64) diagonal block at T in place (lower; its strict upper part is zeroed),
// one CTA.  info = global column + 1 of the first non-positive pivot.
__global__ void __launch_bounds__(256) potrf_block_kernel(double *__restrict__ T, long long ldt, int w, int col0,
                                                          int *__restrict__ info) {
    __shared__ double S[64][65];
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) S[e / w][e % w] = T[(long long)(e / w) * ldt + e % w];
    __syncthreads();
    for (int c = 0; c < w; c++) {
        if (threadIdx.x == 0) {
            const double d = S[c][c];
            if (!(d > 0.0)) {
                if (*info == 0) *info = col0 + c + 1;
                S[c][c] = 1.0;  // continue with a harmless pivot; the caller reports the failure
            } else {
                S[c][c] = sqrt(d);
            }
        }
        __syncthreads();
        const double d = S[c][c];
        for (int r = c + 1 + threadIdx.x; r < w; r += blockDim.x) S[r][c] /= d;
        __syncthreads();
        // trailing update of the lower part: S[r][k] -= S[r][c] S[k][c], c < k <= r
        for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
            const int r = e / w, k = e % w;
            if (r > c && k > c && k <= r) S[r][k] = fma(-S[r][c], S[k][c], S[r][k]);
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
        const int r = e / w, k = e % w;
        T[(long long)r * ldt + k] = k <= r ? S[r][k] : 0.0;
    }
}

// perm[i] = the original row now at position i after the interchanges ipiv[0..n) in order; one thread
__global__ void perm_from_pivots_kernel(const int *__restrict__ ipiv, int n, int *__restrict__ perm) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int i = 0; i < n; i++) {
        const int p = ipiv[i];
        const int t = perm[i];
        perm[i] = perm[p];
        perm[p] = t;
    }
}

// Y[i][:] = B[perm[i]][:] (row gather), n x ncol
__global__ void gather_rows_kernel(const double *__restrict__ B, const int *__restrict__ perm, int n, int ncol,
                                   double *__restrict__ Y) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)n * ncol) return;
    const int i = (int)(e / ncol), j = (int)(e % ncol);
    Y[e] = B[(long long)perm[i] * ncol + j];
}

}  // namespace

int dgemm(sod_context *ctx, bool ta, bool tb, int M, int N, int K, double alpha, const double *A, long long lda,
          const double *B, long long ldb, double beta, double *C, long long ldc, bool lower_only) {
    if (M <= 0 || N <= 0) return SOD_OK;
    cudaStream_t st = ctx->stream;
    if (!lower_only && (M < 32 || N < 32)) {  // thin: one thread per output
        const unsigned blocks = (unsigned)(((long long)M * N + 255) / 256);
        if (!ta && !tb) dgemm_small_kernel<false, false><<<blocks, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        else if (ta && !tb) dgemm_small_kernel<true, false><<<blocks, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        else if (!ta && tb) dgemm_small_kernel<false, true><<<blocks, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        else dgemm_small_kernel<true, true><<<blocks, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        return SOD_OK;
    }
    const dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
#define SOD_GEMM_CASE(TA_, TB_, LO_)                                                                        \
    if (ta == TA_ && tb == TB_ && lower_only == LO_)                                                          \
        dgemm_kernel<TA_, TB_, LO_><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    SOD_GEMM_CASE(false, false, false)
    SOD_GEMM_CASE(true, false, false)
    SOD_GEMM_CASE(false, true, false)
    SOD_GEMM_CASE(true, true, false)
    SOD_GEMM_CASE(false, false, true)
    SOD_GEMM_CASE(true, false, true)
    SOD_GEMM_CASE(false, true, true)
    SOD_GEMM_CASE(true, true, true)
#undef SOD_GEMM_CASE
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// Triangular solves on the diagonal blocks, dispatched on the block width (8 / 16 / 32 / 64)
enum TriKind { TRI_UNIT_LOWER, TRI_UPPER, TRI_CHOL, TRI_CHOL_T, TRI_RIGHT_LT };
template <int W>
static void tri_launch(TriKind kind, const double *T, long long ldt, int w, double *X, long long ldx, int nvec,
                       cudaStream_t st) {
    const unsigned b256 = (unsigned)((nvec + 255) / 256), b128 = (unsigned)((nvec + 127) / 128);
    switch (kind) {
    case TRI_UNIT_LOWER: trsm_unit_lower_kernel<W><<<b256, 256, 0, st>>>(T, ldt, w, X, ldx, nvec); break;
    case TRI_UPPER: trsm_upper_kernel<W><<<b256, 256, 0, st>>>(T, ldt, w, X, ldx, nvec); break;
    case TRI_CHOL: trsm_chol_kernel<false, W><<<b256, 256, 0, st>>>(T, ldt, w, X, ldx, nvec); break;
    case TRI_CHOL_T: trsm_chol_kernel<true, W><<<b256, 256, 0, st>>>(T, ldt, w, X, ldx, nvec); break;
    case TRI_RIGHT_LT: trsm_right_lt_kernel<W><<<b128, 128, 0, st>>>(T, ldt, w, X, ldx, nvec); break;
    }
}
static int tri(sod_context *ctx, TriKind kind, const double *T, long long ldt, int w, double *X, long long ldx,
               int nvec) {
    if (nvec <= 0 || w <= 0) return SOD_OK;
    cudaStream_t st = ctx->stream;
    if (w <= 8) tri_launch<8>(kind, T, ldt, w, X, ldx, nvec, st);
    else if (w <= 16) tri_launch<16>(kind, T, ldt, w, X, ldx, nvec, st);
    else if (w <= 32) tri_launch<32>(kind, T, ldt, w, X, ldx, nvec, st);
    else tri_launch<64>(kind, T, ldt, w, X, ldx, nvec, st);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// columns [c0, c0 + w) of the LU, recursively (see the header)
static int lu_panel(sod_context *ctx, double *A, int n, int c0, int w, int *ipiv, int *info) {
    if (w <= LEAF) {
        lu_leaf_kernel<<<1, LEAF_THREADS, 0, ctx->stream>>>(A, n, n, c0, w, ipiv, info);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        return SOD_OK;
    }
    const int h = std::max(LEAF, (w / 2 + LEAF - 1) / LEAF * LEAF);
    SOD_TRY(lu_panel(ctx, A, n, c0, h, ipiv, info));
    double *A11 = A + (long long)c0 * n + c0;
    double *A12 = A11 + h;
    // U12 = L11^-1 A12 (h rows, w - h columns), then A22 -= L21 U12 over the rows below
    SOD_TRY(tri(ctx, TRI_UNIT_LOWER, A11, n, h, A12, n, w - h));
    if (c0 + h < n)
        SOD_TRY(dgemm(ctx, false, false, n - c0 - h, w - h, h, -1.0, A + (long long)(c0 + h) * n + c0, n, A12, n, 1.0,
                      A + (long long)(c0 + h) * n + c0 + h, n, false));
    return lu_panel(ctx, A, n, c0 + h, w - h, ipiv, info);
}

constexpr int NB = 64;

int lu_factor(sod_context *ctx, double *A, int n, int *ipiv, int *perm, int *info) {
    cudaStream_t st = ctx->stream;
    SOD_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
    for (int k = 0; k < n; k += NB) {
        const int w = std::min(NB, n - k);
        SOD_TRY(lu_panel(ctx, A, n, k, w, ipiv, info));
        if (k + w < n) {
            double *A11 = A + (long long)k * n + k;
            SOD_TRY(tri(ctx, TRI_UNIT_LOWER, A11, n, w, A11 + w, n, n - k - w));
            SOD_TRY(dgemm(ctx, false, false, n - k - w, n - k - w, w, -1.0, A + (long long)(k + w) * n + k, n, A11 + w,
                          n, 1.0, A + (long long)(k + w) * n + k + w, n, false));
        }
    }
    perm_from_pivots_kernel<<<1, 1, 0, st>>>(ipiv, n, perm);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// X = A^-1 B with P A = L U (row-major n x nrhs; X must not alias B): X = P B (row gather), then
// L Z = X (X_k = L_kk^-1 X_k, X_below -= L_below,k X_k) and U X = Z (X_k = U_kk^-1 X_k,
// X_above -= U_above,k X_k), blocked by NB rows
int lu_solve(sod_context *ctx, const double *LU, int n, const int *perm, int nrhs, const double *B, double *X) {
    cudaStream_t st = ctx->stream;
    const long long tot = (long long)n * nrhs;
    gather_rows_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(B, perm, n, nrhs, X);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    for (int k = 0; k < n; k += NB) {
        const int w = std::min(NB, n - k);
        SOD_TRY(tri(ctx, TRI_UNIT_LOWER, LU + (long long)k * n + k, n, w, X + (long long)k * nrhs, nrhs, nrhs));
        if (k + w < n)
            SOD_TRY(dgemm(ctx, false, false, n - k - w, nrhs, w, -1.0, LU + (long long)(k + w) * n + k, n,
                          X + (long long)k * nrhs, nrhs, 1.0, X + (long long)(k + w) * nrhs, nrhs, false));
    }
    for (int k = (n - 1) / NB * NB; k >= 0; k -= NB) {
        const int w = std::min(NB, n - k);
        SOD_TRY(tri(ctx, TRI_UPPER, LU + (long long)k * n + k, n, w, X + (long long)k * nrhs, nrhs, nrhs));
        if (k > 0)
            SOD_TRY(dgemm(ctx, false, false, k, nrhs, w, -1.0, LU + k, n, X + (long long)k * nrhs, nrhs, 1.0, X, nrhs,
                          false));
    }
    return SOD_OK;
}

// A = L L^T in place: the lower triangle of the row-major symmetric A is read (only it need be valid)
// and replaced by L; the diagonal blocks' strict upper parts are zeroed, the rest of the upper triangle
// is left as it was
int chol_factor(sod_context *ctx, double *A, int n, int *info) {
    cudaStream_t st = ctx->stream;
    SOD_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
    for (int k = 0; k < n; k += NB) {
        const int w = std::min(NB, n - k);
        double *A11 = A + (long long)k * n + k;
        potrf_block_kernel<<<1, 256, 0, st>>>(A11, n, w, k, info);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        if (k + w < n) {
            const int m = n - k - w;
            double *A21 = A + (long long)(k + w) * n + k;
            SOD_TRY(tri(ctx, TRI_RIGHT_LT, A11, n, w, A21, n, m));  // L21 = A21 L11^-T
            // A22 -= L21 L21^T on the lower tiles
            SOD_TRY(dgemm(ctx, false, true, m, m, w, -1.0, A21, n, A21, n, 1.0, A + (long long)(k + w) * n + k + w, n,
                          true));
        }
    }
    return SOD_OK;
}

// X = A^-1 B with A = L L^T (L from chol_factor), row-major n x nrhs; X may alias B
int chol_solve(sod_context *ctx, const double *Lf, int n, int nrhs, const double *B, double *X) {
    cudaStream_t st = ctx->stream;
    if (X != B) SOD_CHECK_CUDA(cudaMemcpyAsync(X, B, sizeof(double) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, st));
    for (int k = 0; k < n; k += NB) {  // L Z = B
        const int w = std::min(NB, n - k);
        SOD_TRY(tri(ctx, TRI_CHOL, Lf + (long long)k * n + k, n, w, X + (long long)k * nrhs, nrhs, nrhs));
        if (k + w < n)
            SOD_TRY(dgemm(ctx, false, false, n - k - w, nrhs, w, -1.0, Lf + (long long)(k + w) * n + k, n,
                          X + (long long)k * nrhs, nrhs, 1.0, X + (long long)(k + w) * nrhs, nrhs, false));
    }
    for (int k = (n - 1) / NB * NB; k >= 0; k -= NB) {  // L^T X = Z; (L^T)[i][j] = L[j][i]
        const int w = std::min(NB, n - k);
        SOD_TRY(tri(ctx, TRI_CHOL_T, Lf + (long long)k * n + k, n, w, X + (long long)k * nrhs, nrhs, nrhs));
        if (k > 0)
            SOD_TRY(dgemm(ctx, true, false, k, nrhs, w, -1.0, Lf + (long long)k * n, n, X + (long long)k * nrhs, nrhs,
                          1.0, X, nrhs, false));
    }
    return SOD_OK;
}

}  // namespace sod
