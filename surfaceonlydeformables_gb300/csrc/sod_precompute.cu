// sod_precompute.cu -- the time-domain CQBEM precomputation of one object.
//
// Replaces ElastodynamicsCQBEMMatrixCollection::compute_{H,G}_matrices,
// compute_B_trans_matrices, compute_B_angular_tensors and compute_B_euler_matrices
// (src/elastodynamics_cqbem_{G,H,B_trans,B_angular}.cu, src/elastodynamics_cqbem_matrix_collection.cpp:280-305):
//   1. Laplace-domain assembly of every requested kind at the L/2+1 CQ frequencies (one call);
//   2. inverse transform to the L time weights (FP64 accumulation for FP64 outputs);
//   3. H_0 += C, the free term (collocation: 3x3 blocks on the diagonal from solid angles,
//      src/elastics_bem_matrix_collection.cpp:387-445; Galerkin: mass matrix A/24, A/48, :447-467);
//   4. B_angular_n(3v+i, j, k) += B_trans_n(3v+i, j) (x_v - cm)_k (src/elastodynamics_cqbem_B_angular.cu:167-175);
//   5. B_euler_n(i, j) = B_angular_n(i, (j+2)%3, (j+1)%3) - B_angular_n(i, (j+1)%3, (j+2)%3).
// Everything after the host-side free-term geometry runs on the device; the reference writes every
// U_l to disk and re-reads all of them for every n.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sod_internal.h"

namespace sod {

// Collocation free term, 3x3 per vertex (src/elastics_bem_matrix_collection.cpp:387-445).  O(F) host
// work on the mesh's FP64 geometry.  With traction-discontinuity splitting the reference computes C
// on the original mesh (every face corner at its canonical vertex, so the split edges pair up again)
// and copies the canonical vertex's block to each split vertex (:395-400, :434-441).
static void c_matrix_collocation(const sod_mesh *m, double nu, std::vector<double> &C) {
    const int nV = m->nV, nF = m->nF;
    std::vector<int> Fc(m->F);
    if (m->has_vmap)
        for (auto &v : Fc) v = m->vmap[v];
    C.assign(9 * (size_t)nV, 0.0);
    for (int v = 0; v < nV; v++)
        for (int d = 0; d < 3; d++) C[9 * v + 4 * d] = 0.5;
    auto P = [&](int v, int d) { return m->V[3 * v + d]; };
    auto unit = [](double a[3]) {
        const double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (n > 0)
            for (int d = 0; d < 3; d++) a[d] /= n;
    };
    // undirected edges: directed edge k of face f joins F(f,(k+1)%3) -> F(f,(k+2)%3)
    struct E {
        int a, b;
        long long de;
    };
    std::vector<E> es;
    es.reserve(3 * (size_t)nF);
    for (int f = 0; f < nF; f++)
        for (int k = 0; k < 3; k++) {
            const int a = Fc[3 * f + (k + 1) % 3], b = Fc[3 * f + (k + 2) % 3];
            es.push_back({std::min(a, b), std::max(a, b), f + (long long)k * nF});
        }
    std::sort(es.begin(), es.end(), [](const E &x, const E &y) {
        return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : x.de < y.de);
    });
    for (size_t t = 0; t + 1 < es.size(); t++) {
        if (es[t].a != es[t + 1].a || es[t].b != es[t + 1].b) continue;
        const long long e1 = es[t].de, e2 = es[t + 1].de;
        const int f1 = (int)(e1 % nF), f2 = (int)(e2 % nF), k1 = (int)(e1 / nF);
        const int a = Fc[3 * f1 + (k1 + 1) % 3], b = Fc[3 * f1 + (k1 + 2) % 3];
        const double *n1 = &m->N[3 * f1], *n2 = &m->N[3 * f2];
        double r[3] = {P(a, 0) - P(b, 0), P(a, 1) - P(b, 1), P(a, 2) - P(b, 2)};
        unit(r);
        const double cx[3] = {n1[1] * n2[2] - n1[2] * n2[1], n1[2] * n2[0] - n1[0] * n2[2], n1[0] * n2[1] - n1[1] * n2[0]};
        const double sx = cx[0] * r[0] + cx[1] * r[1] + cx[2] * r[2];
        const double sg = std::abs(sx) < 1e-12 ? 0.0 : (sx > 0 ? 1.0 : -1.0);
        const double dn = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
        const double w = sg * std::atan2(std::sqrt(cx[0] * cx[0] + cx[1] * cx[1] + cx[2] * cx[2]), dn) / (4.0 * M_PI);
        for (int d = 0; d < 3; d++) {
            C[9 * a + 4 * d] += w;
            C[9 * b + 4 * d] += w;
        }
        t++;
    }
    const double coef = 1.0 / (8.0 * M_PI * (1.0 - nu));
    for (int f = 0; f < nF; f++) {
        const double *n = &m->N[3 * f];
        for (int i = 0; i < 3; i++) {
            const int vi = Fc[3 * f + i], v1 = Fc[3 * f + (i + 1) % 3], v2 = Fc[3 * f + (i + 2) % 3];
            double r1[3], r2[3];
            for (int d = 0; d < 3; d++) r1[d] = P(v1, d) - P(vi, d), r2[d] = P(v2, d) - P(vi, d);
            unit(r1);
            unit(r2);
            const double dr[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
            const double c[3] = {dr[1] * n[2] - dr[2] * n[1], dr[2] * n[0] - dr[0] * n[2], dr[0] * n[1] - dr[1] * n[0]};
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) C[9 * vi + 3 * p + q] -= coef * c[p] * n[q];
        }
    }
    if (m->has_vmap)
        for (int v = 0; v < nV; v++)
            if (m->vmap[v] != v)
                for (int t = 0; t < 9; t++) C[9 * (size_t)v + t] = C[9 * (size_t)m->vmap[v] + t];
}

// H_0 diagonal blocks += C (collocation)
template <class T> __global__ void add_block_diag_kernel(T *H0, int nV, const double *C) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 9 * nV) return;
    const int v = t / 9, p = (t / 3) % 3, q = t % 3;
    const long long ld = 3LL * nV;
    H0[(3LL * v + p) * ld + 3LL * v + q] += (T)C[t];
}

// H_0 += Galerkin mass matrix: per face f, (i, j) blocks (A/24 on i == j, A/48 otherwise) times I3.
// One thread per vertex pair entry would race; instead one thread per row vertex walks its star
// (fixed order), so every H_0 entry is updated by exactly one thread.
template <class T>
__global__ void add_mass_kernel(T *H0, int nV, const int *F, const double *A2, const int *vf_off, const int *vf) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const long long ld = 3LL * nV;
    for (int e = vf_off[v]; e < vf_off[v + 1]; e++) {
        const int f = vf[e];
        const double A = A2[f];
        for (int j = 0; j < 3; j++) {
            const int vj = F[3 * f + j];
            const double w = (vj == v) ? A / 24.0 : A / 48.0;
            for (int d = 0; d < 3; d++) H0[(3LL * v + d) * ld + 3LL * vj + d] += (T)w;
        }
    }
}

// B_angular_n(3v+i, j, k) += B_trans_n(3v+i, j) (x_v - cm)_k, then B_euler_n from B_angular_n
template <class T>
__global__ void bangular_finish_kernel(T *Ba, const T *Bt, T *Be, int nV, int L, const double *V, double cx, double cy,
                                       double cz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = 3LL * nV;
    if (t >= rows * L) return;
    const long long n = t / rows, row = t % rows;
    const int v = (int)(row / 3);
    const double d[3] = {V[3 * v] - cx, V[3 * v + 1] - cy, V[3 * v + 2] - cz};
    T *ba = Ba + (n * rows + row) * 9;
    const T *bt = Bt ? Bt + (n * rows + row) * 3 : nullptr;
    double b[9];
    for (int c = 0; c < 9; c++) {
        b[c] = (double)ba[c];
        if (bt) b[c] += (double)bt[c / 3] * d[c % 3];
        ba[c] = (T)b[c];
    }
    if (Be) {
        T *be = Be + (n * rows + row) * 3;
        for (int j = 0; j < 3; j++) be[j] = (T)(b[3 * ((j + 2) % 3) + (j + 1) % 3] - b[3 * ((j + 1) % 3) + (j + 2) % 3]);
    }
}

}  // namespace sod

using namespace sod;

extern "C" int sod_cqbem_precompute(sod_context *ctx, const sod_mesh *mesh, int method, double c1, double c2,
                                    double rho, double nu, int bdf, double dt, int N, int order, int subdiv,
                                    int sorder, int ssub, const double *cm, void *G_out, void *H_out,
                                    void *B_trans_out, void *B_angular_out, void *B_euler_out, int out_dtype) {
    SOD_REQUIRE(ctx && mesh && mesh->ctx == ctx, "bad context or mesh");
    SOD_REQUIRE(out_dtype == SOD_F64 || out_dtype == SOD_F32, "time-domain output must be float64 or float32");
    SOD_REQUIRE(nu > -1.0 && nu < 0.5, "Poisson ratio must be in (-1, 0.5)");
    SOD_REQUIRE(G_out || H_out || B_trans_out || B_angular_out || B_euler_out, "no output requested");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const int nV = mesh->nV;
    double R;
    int L;
    std::vector<double> s(2 * (N / 2 + 2));
    SOD_TRY(sod_cq_frequencies(bdf, dt, N, s.data(), &R, &L));
    const int nf = L / 2 + 1;
    const size_t per[4] = {9 * (size_t)nV * nV, 9 * (size_t)nV * nV, 9 * (size_t)nV, 27 * (size_t)nV};
    void *outs[4] = {G_out, H_out, B_trans_out, B_angular_out};
    // B_euler needs B_angular (and the shift needs B_trans): compute into internal buffers if the
    // caller did not ask for them
    const bool need_ba = B_angular_out || B_euler_out, need_bt = B_trans_out || need_ba;
    bool want[4] = {G_out != nullptr, H_out != nullptr, need_bt, need_ba};
    for (int kd = 0; kd < 4; kd++)
        if (outs[kd]) SOD_REQUIRE(is_device_pointer(outs[kd]), "precompute outputs must be device memory");
    if (B_euler_out) SOD_REQUIRE(is_device_pointer(B_euler_out), "precompute outputs must be device memory");
    const size_t osz = out_dtype == SOD_F64 ? 8 : 4;
    const int fdt = out_dtype == SOD_F64 ? SOD_C128 : SOD_C64;
    const size_t fsz = fdt == SOD_C128 ? 16 : 8;
    // frequency-domain scratch for all requested kinds + time-domain scratch for internal B parts
    size_t foff[4] = {0, 0, 0, 0}, ftot = 0, toff[4] = {0, 0, 0, 0}, ttot = 0;
    for (int kd = 0; kd < 4; kd++) {
        if (!want[kd]) continue;
        foff[kd] = ftot;
        ftot += per[kd] * nf * fsz;
        if (!outs[kd]) {
            toff[kd] = ttot;
            ttot += per[kd] * L * osz;
        }
    }
    SOD_TRY(ctx->freqbuf.ensure(ftot + ttot));
    char *fb = ctx->freqbuf.as<char>();
    void *tdom[4] = {nullptr, nullptr, nullptr, nullptr};
    void *fdom[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int kd = 0; kd < 4; kd++) {
        if (!want[kd]) continue;
        fdom[kd] = fb + foff[kd];
        tdom[kd] = outs[kd] ? outs[kd] : fb + ftot + toff[kd];
    }
    // time-domain outputs: the regular pass in compensated arithmetic unless the caller forced FP32 (the
    // transform multiplies the late weights by up to R^-N = 1e5, FP32 noise included)
    int mask = 0;
    for (int kd = 0; kd < 4; kd++)
        if (want[kd]) mask |= 1 << kd;
    SOD_TRY(assemble_kinds(ctx, mesh, mask, method, c1, c2, rho, s.data(), nf, order, subdiv, sorder, ssub,
                           SOD_PART_ALL, fdom, fdt, ctx->precision != SOD_PRECISION_FP32));
    for (int kd = 0; kd < 4; kd++)
        if (want[kd])
            SOD_TRY(launch_inverse_transform(ctx, fdom[kd], fdt, (int64_t)per[kd], nf, L, R, tdom[kd], out_dtype,
                                             ctx->stream));
    if (H_out) {
        if (method == SOD_COLLOCATION) {
            std::vector<double> C;
            c_matrix_collocation(mesh, nu, C);
            SOD_TRY(ctx->small.ensure(sizeof(double) * C.size()));
            SOD_CHECK_CUDA(cudaMemcpy(ctx->small.p, C.data(), sizeof(double) * C.size(), cudaMemcpyHostToDevice));
            const int nt = 9 * nV;
            if (out_dtype == SOD_F64)
                add_block_diag_kernel<double><<<(nt + 255) / 256, 256, 0, ctx->stream>>>((double *)H_out, nV, ctx->small.as<double>());
            else
                add_block_diag_kernel<float><<<(nt + 255) / 256, 256, 0, ctx->stream>>>((float *)H_out, nV, ctx->small.as<double>());
        } else {
            // vertex -> incident faces, double areas
            std::vector<int> off(nV + 1, 0), vf;
            for (int t = 0; t < 3 * mesh->nF; t++) off[mesh->F[t] + 1]++;
            for (int v = 0; v < nV; v++) off[v + 1] += off[v];
            vf.assign(off[nV], 0);
            std::vector<int> pos(off.begin(), off.end() - 1);
            for (int f = 0; f < mesh->nF; f++)
                for (int k = 0; k < 3; k++) vf[pos[mesh->F[3 * f + k]]++] = f;
            std::vector<double> A2(mesh->nF);
            for (int f = 0; f < mesh->nF; f++) {
                const double *a = &mesh->V[3 * mesh->F[3 * f]], *b = &mesh->V[3 * mesh->F[3 * f + 1]],
                             *c = &mesh->V[3 * mesh->F[3 * f + 2]];
                const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                const double x[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
                A2[f] = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            }
            const size_t bytes = sizeof(double) * A2.size() + sizeof(int) * (off.size() + vf.size());
            SOD_TRY(ctx->small.ensure(bytes));
            char *sb = ctx->small.as<char>();
            SOD_CHECK_CUDA(cudaMemcpy(sb, A2.data(), sizeof(double) * A2.size(), cudaMemcpyHostToDevice));
            SOD_CHECK_CUDA(cudaMemcpy(sb + sizeof(double) * A2.size(), off.data(), sizeof(int) * off.size(),
                                      cudaMemcpyHostToDevice));
            SOD_CHECK_CUDA(cudaMemcpy(sb + sizeof(double) * A2.size() + sizeof(int) * off.size(), vf.data(),
                                      sizeof(int) * vf.size(), cudaMemcpyHostToDevice));
            const double *dA = reinterpret_cast<const double *>(sb);
            const int *doff = reinterpret_cast<const int *>(sb + sizeof(double) * A2.size());
            const int *dvf = doff + off.size();
            if (out_dtype == SOD_F64)
                add_mass_kernel<double><<<(nV + 127) / 128, 128, 0, ctx->stream>>>((double *)H_out, nV, mesh->dF.as<int>(), dA, doff, dvf);
            else
                add_mass_kernel<float><<<(nV + 127) / 128, 128, 0, ctx->stream>>>((float *)H_out, nV, mesh->dF.as<int>(), dA, doff, dvf);
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    if (need_ba) {
        SOD_REQUIRE(cm != nullptr, "B_angular needs the centre of mass");
        const long long nt = 3LL * nV * L;
        const unsigned blocks = (unsigned)((nt + 255) / 256);
        if (out_dtype == SOD_F64)
            bangular_finish_kernel<double><<<blocks, 256, 0, ctx->stream>>>(
                (double *)tdom[3], (const double *)tdom[2], (double *)B_euler_out, nV, L, mesh->dV.as<double>(), cm[0], cm[1], cm[2]);
        else
            bangular_finish_kernel<float><<<blocks, 256, 0, ctx->stream>>>(
                (float *)tdom[3], (const float *)tdom[2], (float *)B_euler_out, nV, L, mesh->dV.as<double>(), cm[0], cm[1], cm[2]);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    return SOD_OK;
}
