// sod_static_solve.cu -- the regularised elastostatic solve for u_p, on the device.
//
// Replaces the u_p computation of ElastostaticsBEMMatrixCollection::init
// (src/elastostatics_bem_matrix_collection.cpp:58-89):
//   T   = [T_d; T_r] (6 x 3V): rigid translations and rotations weighted by the vertex areas
//         (T_d(v) += A_e / 6 I, T_r(v) += A_e / 24 [v_0 + v_1 + v_2 + v_i]_x per face e, corner i,
//          A_e the doubled face area);
//   H'  = H^T H + (tr(H) / 3V)^2 T^T T          (regularisation of [Hahn and Wojtan 2016] on H);
//   G'  = H^T G (I - A^T (A A^T)^-1 A), A = T   (tractions projected to be globally force-free);
//   u_p = H'^-1 G'                               (H' symmetric: Eigen's LDL^T in the reference).
// H' is symmetric positive definite once T spans the null space of H, so the factorisation here is
// Cholesky, the LDL^T of an SPD matrix without pivoting.  The two large products (H^T G' and the lower
// triangle of H^T H) are this library's FP64 GEMM, the Cholesky factorisation and its solves those of
// sod_dense_kernels.cu; T, the 6 x 6 projection, the rank-6 updates and the trace are kernels of this
// file.  Every reduction runs in a fixed order.  All matrices are row-major 3V x 3V.
#include <cmath>

#include "sod_dense.h"

using namespace sod;

namespace {

// T (6 x n, n = 3 nV, row-major) per vertex v: the faces of v's star in face order, each corner i
// with F[f][i] == v.  The star of v lists every face with a corner whose canonical id is v's, so
// split vertices (traction discontinuities) only take their own corners.
__global__ void rigid_modes_kernel(const double *__restrict__ V, const int *__restrict__ F, int nV,
                                   const int *__restrict__ star_off, const int *__restrict__ star_face,
                                   double *__restrict__ T) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const size_t n = 3 * (size_t)nV;
    double d = 0.0, r[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int s = star_off[v]; s < star_off[v + 1]; s++) {
        const int f = star_face[s];
        const int j[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
        double p[3][3];
        for (int c = 0; c < 3; c++)
            for (int x = 0; x < 3; x++) p[c][x] = V[3 * j[c] + x];
        const double u[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
        const double w[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        const double cx = u[1] * w[2] - u[2] * w[1], cy = u[2] * w[0] - u[0] * w[2], cz = u[0] * w[1] - u[1] * w[0];
        const double A = sqrt(cx * cx + cy * cy + cz * cz);
        for (int i = 0; i < 3; i++) {
            if (j[i] != v) continue;
            d += A / 6.0;
            const double sx = p[0][0] + p[1][0] + p[2][0] + p[i][0], sy = p[0][1] + p[1][1] + p[2][1] + p[i][1],
                         sz = p[0][2] + p[1][2] + p[2][2] + p[i][2];
            const double m[3][3] = {{0.0, -sz, sy}, {sz, 0.0, -sx}, {-sy, sx, 0.0}};
            const double a = A / 6.0 * 0.25;
            for (int q = 0; q < 3; q++)
                for (int c = 0; c < 3; c++) r[q][c] += a * m[q][c];
        }
    }
    for (int q = 0; q < 3; q++)
        for (int c = 0; c < 3; c++) {
            T[q * n + 3 * (size_t)v + c] = q == c ? d : 0.0;
            T[(3 + q) * n + 3 * (size_t)v + c] = r[q][c];
        }
}

constexpr int PT = 512;  // threads of the projection kernel

// One CTA: tr(H), A A^T (6 x 6), its LU with partial pivoting, M = (A A^T)^-1 A (6 x n) and the
// regularisation weight c2 = (tr(H) / n)^2 into scal[0].  Sums over n in a fixed order.
__global__ void __launch_bounds__(PT) projection_kernel(const double *__restrict__ H, const double *__restrict__ T,
                                                        int n, double *__restrict__ M, double *__restrict__ scal,
                                                        int *info) {
    __shared__ double red[PT / 32][22];
    __shared__ double tot[22];
    __shared__ double lu[6][6];
    __shared__ int piv[6], bad_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double part[22];
    for (int q = 0; q < 22; q++) part[q] = 0.0;
    for (int i = tid; i < n; i += PT) {
        double t[6];
        for (int a = 0; a < 6; a++) t[a] = T[(size_t)a * n + i];
        int q = 0;
        for (int a = 0; a < 6; a++)
            for (int b = a; b < 6; b++, q++) part[q] = fma(t[a], t[b], part[q]);
        part[21] += H[(size_t)i * n + i];
    }
    for (int q = 0; q < 22; q++) {
        double v = part[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (tid < 22) {
        double v = 0.0;
        for (int w = 0; w < PT / 32; w++) v += red[w][tid];
        tot[tid] = v;
    }
    __syncthreads();
    if (tid == 0) {
        int q = 0;
        for (int a = 0; a < 6; a++)
            for (int b = a; b < 6; b++, q++) lu[a][b] = lu[b][a] = tot[q];
        const double c = tot[21] / n;
        scal[0] = c * c;
        int bad = 0;
        for (int k = 0; k < 6; k++) {  // LU with partial pivoting, P (A A^T) = L U
            int p = k;
            for (int r = k + 1; r < 6; r++)
                if (fabs(lu[r][k]) > fabs(lu[p][k])) p = r;
            piv[k] = p;
            if (p != k)
                for (int c2 = 0; c2 < 6; c2++) {
                    const double t = lu[k][c2];
                    lu[k][c2] = lu[p][c2];
                    lu[p][c2] = t;
                }
            if (lu[k][k] == 0.0) {
                bad = 1;
                continue;
            }
            for (int r = k + 1; r < 6; r++) {
                const double l = lu[r][k] / lu[k][k];
                lu[r][k] = l;
                for (int c2 = k + 1; c2 < 6; c2++) lu[r][c2] -= l * lu[k][c2];
            }
        }
        info[0] = bad;
        bad_s = bad;
    }
    __syncthreads();
    if (bad_s) return;
    for (int i = tid; i < n; i += PT) {  // column i of M: solve (A A^T) x = A[:, i]
        double x[6];
        for (int a = 0; a < 6; a++) x[a] = T[(size_t)a * n + i];
        for (int k = 0; k < 6; k++) {
            const double t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
        for (int r = 1; r < 6; r++)
            for (int k = 0; k < r; k++) x[r] -= lu[r][k] * x[k];
        for (int r = 5; r >= 0; r--) {
            for (int k = r + 1; k < 6; k++) x[r] -= lu[r][k] * x[k];
            x[r] /= lu[r][r];
        }
        for (int a = 0; a < 6; a++) M[(size_t)a * n + i] = x[a];
    }
}

// GA[i][a] = sum_j G[i][j] T[a][j]: one warp per row, lanes over the columns, xor tree
__global__ void __launch_bounds__(256) g_at_kernel(const double *__restrict__ G, const double *__restrict__ T, int n,
                                                   double *__restrict__ GA) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const double *g = G + (size_t)row * n;
    for (int j = lane; j < n; j += 32) {
        const double v = __ldg(g + j);
#pragma unroll
        for (int a = 0; a < 6; a++) acc[a] = fma(v, __ldg(T + (size_t)a * n + j), acc[a]);
    }
#pragma unroll
    for (int a = 0; a < 6; a++) {
        double v = acc[a];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) GA[(size_t)row * 6 + a] = v;
    }
}

// Gp[i][j] = G[i][j] - sum_a GA[i][a] M[a][j]  (G (I - A^T (A A^T)^-1 A), row-major)
__global__ void project_kernel(const double *__restrict__ G, const double *__restrict__ GA,
                               const double *__restrict__ M, int n, double *__restrict__ Gp) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * n) return;
    const size_t i = e / n, j = e % n;
    double v = 0.0;
#pragma unroll
    for (int a = 0; a < 6; a++) v = fma(GA[i * 6 + a], M[(size_t)a * n + j], v);
    Gp[e] = G[e] - v;
}

// lower triangle (column-major, row i >= column j) of H' += c2 T^T T
__global__ void add_ttt_kernel(double *__restrict__ Hr, const double *__restrict__ T, int n,
                               const double *__restrict__ scal) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * n) return;
    const size_t i = e / n, j = e % n;  // row-major lower triangle: element (i, j), j <= i
    if (j > i) return;
    double v = 0.0;
#pragma unroll
    for (int a = 0; a < 6; a++) v = fma(T[(size_t)a * n + i], T[(size_t)a * n + j], v);
    Hr[e] = fma(scal[0], v, Hr[e]);
}

int rigid_modes_device(sod_context *ctx, const sod_mesh *m, double *T) {
    rigid_modes_kernel<<<(m->nV + 127) / 128, 128, 0, ctx->stream>>>(m->dV.as<double>(), m->dF.as<int>(), m->nV,
                                                                     m->dStarOff.as<int>(), m->dStarFace.as<int>(), T);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

}  // namespace

extern "C" {

int sod_elastostatic_rigid_modes(sod_context *ctx, const sod_mesh *m, double *T) {
    SOD_REQUIRE(ctx && m && m->ctx == ctx && T, "bad context, mesh or output");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t bytes = sizeof(double) * 6 * 3 * (size_t)m->nV;
    const bool host = !is_device_pointer(T);
    DevBuf tmp;
    double *d = T;
    if (host) {
        SOD_TRY(tmp.ensure(bytes));
        d = tmp.as<double>();
    }
    SOD_TRY(rigid_modes_device(ctx, m, d));
    if (host) SOD_CHECK_CUDA(cudaMemcpyAsync(T, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return SOD_OK;
}

int sod_elastostatic_u_p(sod_context *ctx, const sod_mesh *m, const double *H, const double *G, double *u_p) {
    SOD_REQUIRE(ctx && m && m->ctx == ctx, "bad context or mesh");
    SOD_REQUIRE(H && G && u_p, "null argument");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const int n = 3 * m->nV;
    const size_t nn = (size_t)n * n, bytes = sizeof(double) * nn;
    cudaStream_t st = ctx->stream;
    // device copies of host inputs; Gp, the right-hand side / solution and H' are scratch
    DevBuf dh, dg, gp, y, hr, small, info;
    const double *Hd = H, *Gd = G;
    if (!is_device_pointer(H)) {
        SOD_TRY(dh.ensure(bytes));
        SOD_CHECK_CUDA(cudaMemcpyAsync(dh.p, H, bytes, cudaMemcpyHostToDevice, st));
        Hd = dh.as<double>();
    }
    if (!is_device_pointer(G)) {
        SOD_TRY(dg.ensure(bytes));
        SOD_CHECK_CUDA(cudaMemcpyAsync(dg.p, G, bytes, cudaMemcpyHostToDevice, st));
        Gd = dg.as<double>();
    }
    SOD_TRY(gp.ensure(bytes));
    SOD_TRY(y.ensure(bytes));
    SOD_TRY(hr.ensure(bytes));
    // small: T (6n) | M (6n) | GA (6n) | scal (2)
    SOD_TRY(small.ensure(sizeof(double) * (18 * (size_t)n + 2)));
    SOD_TRY(info.ensure(sizeof(int)));
    double *T = small.as<double>(), *M = T + 6 * (size_t)n, *GA = M + 6 * (size_t)n, *scal = GA + 6 * (size_t)n;
    SOD_TRY(rigid_modes_device(ctx, m, T));
    projection_kernel<<<1, PT, 0, st>>>(Hd, T, n, M, scal, info.as<int>());
    SOD_CHECK_CUDA(cudaGetLastError());
    int bad = 0;
    SOD_CHECK_CUDA(cudaMemcpyAsync(&bad, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));
    if (bad) {
        set_error("rigid-mode matrix T T^T is singular");
        return SOD_ERR_INVALID_ARG;
    }
    g_at_kernel<<<(unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, st>>>(Gd, T, n, GA);
    project_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(Gd, GA, M, n, gp.as<double>());
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count(3);
    // y = H^T Gp (row-major), H' (lower triangle) = H^T H + c2 T^T T
    SOD_TRY(dgemm(ctx, true, false, n, n, n, 1.0, Hd, n, gp.as<double>(), n, 0.0, y.as<double>(), n, false));
    SOD_TRY(dgemm(ctx, true, false, n, n, n, 1.0, Hd, n, Hd, n, 0.0, hr.as<double>(), n, true));
    add_ttt_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(hr.as<double>(), T, n, scal);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    SOD_TRY(chol_factor(ctx, hr.as<double>(), n, info.as<int>()));
    int pinfo = 0;
    SOD_CHECK_CUDA(cudaMemcpyAsync(&pinfo, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));
    if (pinfo != 0) {
        set_error("regularised H^T H + c T^T T is not positive definite (leading minor " + std::to_string(pinfo) + ")");
        return SOD_ERR_INVALID_ARG;
    }
    const bool host = !is_device_pointer(u_p);
    double *dst = host ? gp.as<double>() : u_p;
    SOD_TRY(chol_solve(ctx, hr.as<double>(), n, n, y.as<double>(), dst));
    if (host) SOD_CHECK_CUDA(cudaMemcpyAsync(u_p, dst, bytes, cudaMemcpyDeviceToHost, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));
    return SOD_OK;
}

}  // extern "C"
