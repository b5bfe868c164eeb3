// sod_lstsq.cu -- minimum-norm least-squares solves with a tall matrix, on the device.
//
// Replaces the Eigen::CompleteOrthogonalDecomposition objects B_trans_inv / B_euler_inv of
// ElastodynamicsCQBEMMatrixCollection (include/elastodynamics_cqbem_matrix_collection.hpp:43,
// src/elastodynamics_cqbem_matrix_collection.cpp:184-191): X = B^+ Y for B = B_trans or B_euler
// (3V x 3) and Y = H_0, G', B_trans.  The results feed the rigid-frame update of
// ElastodynamicsCQBEMObject (src/elastodynamics_cqbem_object.cpp:188-195).
//
// The decomposition is the complete orthogonal decomposition:
//   - Householder QR with column pivoting, B P = Q R; the pivot is the remaining column of largest
//     norm (first on ties), norms recomputed exactly at every step;
//   - numerical rank r = number of leading |R_ii| > eps * min(m, k) * max_i |R_ii| (the default
//     threshold of Eigen's ColPivHouseholderQR);
//   - for r < k, Householder reflections from the right that zero the R12 block of [R11 R12],
//     [R11 R12] = [T 0] Z, applied in the order i = r-1 .. 0;
//   - minimum-norm solution x = P Z^T [T^-1 (Q^T y)_{1..r}; 0].
// The small factors (k <= 8) are folded into the k x m operator B^+ = P Z^T [T^-1; 0] Q_r^T once, so
// every solve is one pass over Y.  One CTA factors the matrix (k is small, m is at most a few 10^4);
// every reduction runs in a fixed order, so results are deterministic.
#include <cfloat>
#include <cmath>

#include "sod_internal.h"

using namespace sod;

namespace {

constexpr int KMAX = 8;            // columns of B
constexpr int FT = 1024;           // threads of the factorisation CTA
constexpr int APPLY_ROWS = 128;    // rows of Y per CTA of the solve
constexpr int APPLY_THREADS = 256;

// sums[c] for c in [c0, c1) over the CTA in a fixed order (xor tree in each warp, then warp 0 over
// the warp partials in order); `part` holds each thread's own partial sums.  All threads return the
// totals.  red: [FT / 32][KMAX] shared scratch; tot: [KMAX] shared.
__device__ void block_sums(double part[KMAX], int c0, int c1, double (*red)[KMAX], double *tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < KMAX; c++) {
        if (c < c0 || c >= c1) continue;
        double v = part[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < KMAX && (int)threadIdx.x >= c0 && (int)threadIdx.x < c1) {
        double v = 0.0;
        for (int w = 0; w < FT / 32; w++) v += red[w][threadIdx.x];
        tot[threadIdx.x] = v;
    }
    __syncthreads();
}

// Householder vector of x = (alpha, tail) with |tail|^2 = sigma: H x = beta e_1, H = I - tau v v^T,
// v = (1, tail * scale).  Zero tail: tau = 0 and beta = alpha.
__device__ void householder(double alpha, double sigma, double &beta, double &tau, double &scale) {
    if (sigma <= DBL_MIN) {
        beta = alpha;
        tau = 0.0;
        scale = 0.0;
        return;
    }
    beta = sqrt(alpha * alpha + sigma);
    if (alpha >= 0.0) beta = -beta;
    scale = 1.0 / (alpha - beta);
    tau = (beta - alpha) / beta;
}

// A: m x KMAX row-major scratch (B copied in, becomes R and the Householder vectors); E: m x KMAX
// scratch (Q_r); P: k x m output (B^+).  info[0] = rank.
__global__ void __launch_bounds__(FT) cod_kernel(const double *__restrict__ B, int m, int k, double *__restrict__ A,
                                                 double *__restrict__ E, double *__restrict__ P, int *info) {
    __shared__ double red[FT / 32][KMAX];
    __shared__ double tot[KMAX];
    __shared__ double tau_s[KMAX], wv[KMAX];
    __shared__ double R[KMAX][KMAX], S[KMAX][KMAX];
    __shared__ int perm[KMAX], piv_s, rank_s;
    const int tid = threadIdx.x;
    for (int r = tid; r < m; r += FT)
        for (int c = 0; c < KMAX; c++) A[(size_t)r * KMAX + c] = c < k ? B[(size_t)r * k + c] : 0.0;
    if (tid < KMAX) perm[tid] = tid;
    __syncthreads();
    double part[KMAX];
    for (int j = 0; j < k; j++) {
        // squared norms of the remaining columns over rows j..m-1
        for (int c = 0; c < KMAX; c++) part[c] = 0.0;
        for (int r = j + tid; r < m; r += FT)
            for (int c = j; c < k; c++) {
                const double v = A[(size_t)r * KMAX + c];
                part[c] = fma(v, v, part[c]);
            }
        block_sums(part, j, k, red, tot);
        if (tid == 0) {
            int p = j;
            for (int c = j + 1; c < k; c++)
                if (tot[c] > tot[p]) p = c;
            piv_s = p;
            const int t = perm[j];
            perm[j] = perm[p];
            perm[p] = t;
        }
        __syncthreads();
        const int p = piv_s;
        if (p != j)
            for (int r = tid; r < m; r += FT) {
                const double t = A[(size_t)r * KMAX + j];
                A[(size_t)r * KMAX + j] = A[(size_t)r * KMAX + p];
                A[(size_t)r * KMAX + p] = t;
            }
        __syncthreads();
        // reflector of column j over rows j..m-1
        part[0] = 0.0;
        for (int r = j + 1 + tid; r < m; r += FT) {
            const double v = A[(size_t)r * KMAX + j];
            part[0] = fma(v, v, part[0]);
        }
        block_sums(part, 0, 1, red, tot);
        if (tid == 0) {
            double beta, tau, scale;
            householder(A[(size_t)j * KMAX + j], tot[0], beta, tau, scale);
            tau_s[j] = tau;
            wv[0] = scale;
            A[(size_t)j * KMAX + j] = beta;
        }
        __syncthreads();
        const double scale = wv[0];
        for (int r = j + 1 + tid; r < m; r += FT) A[(size_t)r * KMAX + j] *= scale;
        __syncthreads();
        // apply to columns j+1..k-1: w_c = A[j][c] + sum_{r>j} v_r A[r][c]
        for (int c = 0; c < KMAX; c++) part[c] = 0.0;
        for (int r = j + 1 + tid; r < m; r += FT) {
            const double v = A[(size_t)r * KMAX + j];
            for (int c = j + 1; c < k; c++) part[c] = fma(v, A[(size_t)r * KMAX + c], part[c]);
        }
        block_sums(part, j + 1, k, red, tot);
        if (tid == 0)
            for (int c = j + 1; c < k; c++) wv[c] = tau_s[j] * (A[(size_t)j * KMAX + c] + tot[c]);
        __syncthreads();
        for (int r = j + 1 + tid; r < m; r += FT) {
            const double v = A[(size_t)r * KMAX + j];
            for (int c = j + 1; c < k; c++) A[(size_t)r * KMAX + c] -= wv[c] * v;
        }
        if (tid == 0)
            for (int c = j + 1; c < k; c++) A[(size_t)j * KMAX + c] -= wv[c];
        __syncthreads();
    }
    // small factors on one thread: rank, T^-1, Z
    if (tid == 0) {
        for (int i = 0; i < KMAX; i++)
            for (int c = 0; c < KMAX; c++) R[i][c] = (i < k && c < k && c >= i) ? A[(size_t)i * KMAX + c] : 0.0;
        double maxpiv = 0.0;
        for (int i = 0; i < k; i++) maxpiv = fmax(maxpiv, fabs(R[i][i]));
        const double thr = maxpiv * DBL_EPSILON * (double)k;
        int r = 0;
        while (r < k && fabs(R[r][r]) > thr) r++;
        rank_s = r;
        // zero R12 from the right: row i = r-1 .. 0 acts on columns {i} U {r..k-1}
        double zv[KMAX][KMAX], ztau[KMAX];
        for (int i = r - 1; i >= 0; i--) {
            double sigma = 0.0;
            for (int c = r; c < k; c++) sigma = fma(R[i][c], R[i][c], sigma);
            double beta, tau, scale;
            householder(R[i][i], sigma, beta, tau, scale);
            ztau[i] = tau;
            for (int c = r; c < k; c++) zv[i][c] = R[i][c] * scale;
            R[i][i] = beta;
            for (int c = r; c < k; c++) R[i][c] = 0.0;
            for (int l = 0; l < i; l++) {  // rows above: y <- y (I - tau v v^T)
                double w = R[l][i];
                for (int c = r; c < k; c++) w = fma(R[l][c], zv[i][c], w);
                w *= tau;
                R[l][i] -= w;
                for (int c = r; c < k; c++) R[l][c] -= w * zv[i][c];
            }
        }
        // S = Z^T [T^-1; 0] (k x r): T^-1 by back substitution, then reflections i = 0 .. r-1
        for (int a = 0; a < KMAX; a++)
            for (int b = 0; b < KMAX; b++) S[a][b] = 0.0;
        for (int b = 0; b < r; b++) {
            for (int a = b; a >= 0; a--) {
                double v = (a == b) ? 1.0 : 0.0;
                for (int c = a + 1; c <= b; c++) v -= R[a][c] * S[c][b];
                S[a][b] = v / R[a][a];
            }
        }
        if (r < k)
            for (int i = 0; i < r; i++)
                for (int b = 0; b < r; b++) {
                    double w = S[i][b];
                    for (int c = r; c < k; c++) w = fma(zv[i][c], S[c][b], w);
                    w *= ztau[i];
                    S[i][b] -= w;
                    for (int c = r; c < k; c++) S[c][b] -= w * zv[i][c];
                }
        info[0] = r;
    }
    __syncthreads();
    const int r = rank_s;
    // E = Q [I_r; 0] = H_0 ... H_{r-1} [I_r; 0]: reflectors applied last-first
    for (int i = tid; i < m; i += FT)
        for (int c = 0; c < KMAX; c++) E[(size_t)i * KMAX + c] = (i == c && c < r) ? 1.0 : 0.0;
    __syncthreads();
    for (int j = r - 1; j >= 0; j--) {
        for (int c = 0; c < KMAX; c++) part[c] = 0.0;
        for (int i = j + 1 + tid; i < m; i += FT) {
            const double v = A[(size_t)i * KMAX + j];
            for (int c = j; c < r; c++) part[c] = fma(v, E[(size_t)i * KMAX + c], part[c]);
        }
        block_sums(part, j, r, red, tot);
        if (tid == 0)
            for (int c = j; c < r; c++) wv[c] = tau_s[j] * (E[(size_t)j * KMAX + c] + tot[c]);
        __syncthreads();
        for (int i = j + 1 + tid; i < m; i += FT) {
            const double v = A[(size_t)i * KMAX + j];
            for (int c = j; c < r; c++) E[(size_t)i * KMAX + c] -= wv[c] * v;
        }
        if (tid == 0)
            for (int c = j; c < r; c++) E[(size_t)j * KMAX + c] -= wv[c];
        __syncthreads();
    }
    // B^+[perm[a]][i] = sum_b S[a][b] E[i][b]
    for (int i = tid; i < m; i += FT)
        for (int a = 0; a < k; a++) {
            double v = 0.0;
            for (int b = 0; b < r; b++) v = fma(S[a][b], E[(size_t)i * KMAX + b], v);
            P[(size_t)perm[a] * m + i] = v;
        }
}

// partial[chunk][a][j] = sum over the chunk's rows i of P[a][i] Y[i][j]
__global__ void __launch_bounds__(APPLY_THREADS) lstsq_apply_kernel(const double *__restrict__ P,
                                                                    const double *__restrict__ Y, int m, int k,
                                                                    int ncols, double *__restrict__ partial) {
    __shared__ double ps[KMAX][APPLY_ROWS];
    const int i0 = blockIdx.y * APPLY_ROWS, rows = min(APPLY_ROWS, m - i0);
    for (int t = threadIdx.x; t < k * APPLY_ROWS; t += APPLY_THREADS) {
        const int a = t / APPLY_ROWS, i = t % APPLY_ROWS;
        ps[a][i] = i < rows ? P[(size_t)a * m + i0 + i] : 0.0;
    }
    __syncthreads();
    const int j = blockIdx.x * APPLY_THREADS + threadIdx.x;
    if (j >= ncols) return;
    double acc[KMAX];
#pragma unroll
    for (int a = 0; a < KMAX; a++) acc[a] = 0.0;
    for (int i = 0; i < rows; i++) {
        const double y = __ldg(Y + (size_t)(i0 + i) * ncols + j);
#pragma unroll
        for (int a = 0; a < KMAX; a++)
            if (a < k) acc[a] = fma(ps[a][i], y, acc[a]);
    }
#pragma unroll
    for (int a = 0; a < KMAX; a++)
        if (a < k) partial[((size_t)blockIdx.y * k + a) * ncols + j] = acc[a];
}

// X[a][j] = sum over chunks in order
__global__ void lstsq_sum_kernel(const double *__restrict__ partial, int nchunk, int k, int ncols,
                                 double *__restrict__ X) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)k * ncols) return;
    double v = 0.0;
    for (int c = 0; c < nchunk; c++) v += partial[(size_t)c * k * ncols + e];
    X[e] = v;
}

}  // namespace

struct sod_lstsq {
    sod_context *ctx = nullptr;
    int m = 0, k = 0, rank = 0;
    DevBuf pinv, partial, tmp;
};

extern "C" {

int sod_lstsq_create(sod_context *ctx, int m, int k, const double *B, sod_lstsq **out) {
    SOD_REQUIRE(ctx && B && out, "null argument");
    SOD_REQUIRE(k >= 1 && k <= KMAX, "least-squares matrix needs 1 <= k <= 8 columns");
    SOD_REQUIRE(m >= k, "least-squares matrix must have at least as many rows as columns");
    *out = nullptr;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    auto s = std::make_unique<sod_lstsq>();
    s->ctx = ctx;
    s->m = m;
    s->k = k;
    DevBuf a, e, info, bin;
    SOD_TRY(a.ensure(sizeof(double) * (size_t)m * KMAX));
    SOD_TRY(e.ensure(sizeof(double) * (size_t)m * KMAX));
    SOD_TRY(info.ensure(sizeof(int)));
    SOD_TRY(s->pinv.ensure(sizeof(double) * (size_t)m * k));
    const double *db = B;
    if (!is_device_pointer(B)) {
        SOD_TRY(bin.ensure(sizeof(double) * (size_t)m * k));
        SOD_CHECK_CUDA(cudaMemcpyAsync(bin.p, B, sizeof(double) * (size_t)m * k, cudaMemcpyHostToDevice, ctx->stream));
        db = bin.as<double>();
    }
    cod_kernel<<<1, FT, 0, ctx->stream>>>(db, m, k, a.as<double>(), e.as<double>(), s->pinv.as<double>(),
                                          info.as<int>());
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    SOD_CHECK_CUDA(cudaMemcpyAsync(&s->rank, info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = s.release();
    return SOD_OK;
}

int sod_lstsq_rank(const sod_lstsq *s, int *rank) {
    SOD_REQUIRE(s && rank, "null argument");
    *rank = s->rank;
    return SOD_OK;
}

int sod_lstsq_pinv(sod_lstsq *s, double *P) {
    SOD_REQUIRE(s && P, "null argument");
    sod_context *ctx = s->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    SOD_CHECK_CUDA(cudaMemcpyAsync(P, s->pinv.p, sizeof(double) * (size_t)s->m * s->k, cudaMemcpyDefault, ctx->stream));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return SOD_OK;
}

int sod_lstsq_solve(sod_lstsq *s, int ncols, const double *Y, double *X) {
    SOD_REQUIRE(s && Y && X, "null argument");
    SOD_REQUIRE(ncols >= 1, "ncols must be >= 1");
    sod_context *ctx = s->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const int m = s->m, k = s->k;
    const size_t ybytes = sizeof(double) * (size_t)m * ncols, xbytes = sizeof(double) * (size_t)k * ncols;
    const bool hy = !is_device_pointer(Y), hx = !is_device_pointer(X);
    SOD_TRY(s->tmp.ensure((hy ? ybytes : 0) + (hx ? xbytes : 0)));
    const double *dy = Y;
    double *dx = X;
    if (hy) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(s->tmp.p, Y, ybytes, cudaMemcpyHostToDevice, ctx->stream));
        dy = s->tmp.as<double>();
    }
    if (hx) dx = s->tmp.as<double>() + (hy ? (size_t)m * ncols : 0);
    const int nchunk = (m + APPLY_ROWS - 1) / APPLY_ROWS;
    SOD_TRY(s->partial.ensure(sizeof(double) * (size_t)nchunk * k * ncols));
    const dim3 grid((ncols + APPLY_THREADS - 1) / APPLY_THREADS, nchunk);
    lstsq_apply_kernel<<<grid, APPLY_THREADS, 0, ctx->stream>>>(s->pinv.as<double>(), dy, m, k, ncols,
                                                                s->partial.as<double>());
    SOD_CHECK_CUDA(cudaGetLastError());
    const size_t ne = (size_t)k * ncols;
    lstsq_sum_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, ctx->stream>>>(s->partial.as<double>(), nchunk, k, ncols,
                                                                         dx);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count(2);
    if (hx) SOD_CHECK_CUDA(cudaMemcpyAsync(X, dx, xbytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (hy || hx) SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return SOD_OK;
}

int sod_lstsq_destroy(sod_lstsq *s) {
    if (s) {
        cudaSetDevice(s->ctx->device);
        delete s;
    }
    return SOD_OK;
}

}  // extern "C"
