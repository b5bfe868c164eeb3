// sod_elastostatic.cu -- elastostatic (Kelvin) BEM matrices G and H on sm_103a.
//
// Replaces ElasticsBEMMatrixCollection::compute_elastostatic_{G,H}_matrix_{collocation,galerkin}
// (src/elastics_bem_matrix_collection.cpp:43-385):
//   u*_pq = [(3 - 4 nu) d_pq + rh_p rh_q] / (16 pi (1 - nu) mu r)
//   p*_pq = C [(rh_p n_q - rh_q n_p) - (d_pq + 3 rh_p rh_q / (1 - 2 nu)) rh.n] / r^2,
//           C = (1 - 2 nu) / (8 pi (1 - nu))
// and the rigid-mode correction of H's diagonal blocks H_ii = -sum_{j != i} H_ij (:236-243).
//
// Regular faces: FP32, one CTA per field vertex with the row block in shared memory and the faces
// walked in colour order (no two faces of a colour share a vertex: conflict-free, fixed order).
// Singular faces: FP64 polar / Guiggiani rules from the mesh's geometry tables (sod_singular.cu),
// added in the epilogue.  The diagonal correction sums the finished row in FP64 in fixed order.
//
// Galerkin: the Laplace-domain kernels at s = 0 are exactly the Kelvin kernels -- with rho = 1,
// c2^2 = mu, c1^2 = lambda + 2 mu, G's alpha = 1/(16 pi mu (1 - nu) r), beta = (3 - 4 nu) alpha and
// H's a = kappa, b = -kappa, d = -3 (1 - kappa) over 4 pi r^2 (kappa = c2^2 / c1^2) -- and at
// z = 0 the psi series gives exactly -1/2 and e^-z exactly 1.  So the Galerkin path
// (sod_galerkin.cu: test-point rows, fixed-order gather, pair-shared double-float singular pairs)
// runs at s = 0 into a complex128 scratch matrix, and a finishing kernel takes the real part, adds
// the Galerkin mass matrix C (:372-373, 447-467) to H and applies H_ii = -sum_{j != i} H_ij
// (:375-382) in FP64 in fixed order.
#include <algorithm>

#include "sod_faces.cuh"
#include "sod_internal.h"

using namespace sod;

namespace {

struct StaticArgs {
    int nV, nF;
    const float4 *faces;
    const int4 *canonF;
    const int *color_off;
    int ncolors;
    const float *Vf;
    const int *canonV;
    void *out;
    int out_f32;
    const cd *S;  // singular 3x3 blocks per neighbour slot (real parts used)
    const int *nbr_off, *nbr_vert;
    float ga, gb;       // G: u = (ga rh rh^T + gb I) / r
    float ha, hb, hd;   // H: p = [ha rh n^T + hb (n rh^T + rn I) + hd rn rh rh^T] / r^2
};

__device__ __forceinline__ void put(void *out, int f32, long long idx, double v) {
    if (f32)
        static_cast<float *>(out)[idx] = (float)v;
    else
        static_cast<double *>(out)[idx] = v;
}

template <int KIND>
__global__ void __launch_bounds__(512) static_scatter_kernel(StaticArgs a, PointTable pt) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;
    extern __shared__ float acc[];  // [NC][nV]
    const int i = blockIdx.x, nV = a.nV;
    for (int t = threadIdx.x; t < NC * nV; t += blockDim.x) acc[t] = 0.f;
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    __syncthreads();
    for (int c = 0; c < a.ncolors; c++) {
        const int fend = a.color_off[c + 1];
        for (int f = a.color_off[c] + threadIdx.x; f < fend; f += blockDim.x) {
            const FaceRec fr = load_face(a.faces, f);
            bool sing;
            if (a.canonF) {
                const int4 cf = __ldg(a.canonF + f);
                sing = cf.x == ci || cf.y == ci || cf.z == ci;
            } else {
                sing = fr.j0 == i || fr.j1 == i || fr.j2 == i;
            }
            if (sing) continue;
            const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
            float part[3][NC];
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int cc = 0; cc < NC; cc++) part[k][cc] = 0.f;
            for (int q = 0; q < pt.n; q++) {
                const float4 P = pt.p[q];
                const float dx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x - x.x;
                const float dy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y - x.y;
                const float dz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z - x.z;
                const float rinv = rsqrtf(dx * dx + dy * dy + dz * dz);
                const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                float u[NC];
                if (KIND == SOD_G) {
                    const float al = a.ga * rinv, be = a.gb * rinv;
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = p; qq < 3; qq++) u[sym_index(p, qq)] = al * rh[p] * rh[qq] + (p == qq ? be : 0.f);
                } else {
                    const float r2i = rinv * rinv;
                    const float rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                    const float A = a.ha * r2i, B = a.hb * r2i, D = a.hd * r2i * rn;
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = 0; qq < 3; qq++)
                            u[3 * p + qq] = A * rh[p] * nn[qq] + B * (nn[p] * rh[qq] + (p == qq ? rn : 0.f)) +
                                            D * rh[p] * rh[qq];
                }
                const float w = P.w * fr.area;
                const float wl[3] = {w * P.x, w * P.y, w * P.z};
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) part[k][cc] = fmaf(u[cc], wl[k], part[k][cc]);
            }
            const int jj[3] = {fr.j0, fr.j1, fr.j2};
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int cc = 0; cc < NC; cc++) acc[cc * nV + jj[k]] += part[k][cc];
        }
        __syncthreads();
    }
    // singular 3x3 blocks of the neighbour slots, staged in shared memory (FP64)
    const int s0 = a.nbr_off[i], ns = a.nbr_off[i + 1] - s0;
    __shared__ double sadd[64 * 9];
    const bool fits = ns <= 64;
    if (a.S && fits)
        for (int e = threadIdx.x; e < ns * 9; e += blockDim.x) sadd[e] = a.S[(long long)s0 * 9 + e].x;
    __syncthreads();
    const long long ld = 3LL * nV, base = (long long)(3 * i) * ld;
    // H: diagonal block = -(sum over j != i of the finished blocks), FP64, fixed order
    __shared__ double dsum[16][9];
    __shared__ double diag[9];
    if (KIND == SOD_H) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        double d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = threadIdx.x; j < nV; j += blockDim.x) {
            if (j == i) continue;
#pragma unroll
            for (int c = 0; c < 9; c++) d[c] += (double)acc[c * nV + j];
        }
        if (a.S && fits)  // singular parts of the neighbour slots j != i
            for (int sl = threadIdx.x; sl < ns; sl += blockDim.x) {
                const int j = a.nbr_vert[s0 + sl];
                if (j != i)
#pragma unroll
                    for (int c = 0; c < 9; c++) d[c] += sadd[sl * 9 + c];
            }
#pragma unroll
        for (int c = 0; c < 9; c++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d[c] += __shfl_xor_sync(0xffffffffu, d[c], o);
            if (lane == 0) dsum[warp][c] = d[c];
        }
        __syncthreads();
        if (threadIdx.x < 9) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += dsum[w][threadIdx.x];
            diag[threadIdx.x] = -s;
        }
        __syncthreads();
    }
    for (int p = 0; p < 3; p++)
        for (int col = threadIdx.x; col < 3 * nV; col += blockDim.x) {
            const int j = col / 3, qq = col - 3 * j;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : 3 * p + qq;
            double v = acc[comp * nV + j];
            if (KIND == SOD_H && j == i) v = diag[3 * p + qq];
            put(a.out, a.out_f32, base + p * ld + col, v);
        }
    if (a.S && fits) {
        __syncthreads();
        for (int e = threadIdx.x; e < ns * 9; e += blockDim.x) {
            const int sl = e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
            const int j = a.nbr_vert[s0 + sl];
            if (KIND == SOD_H && j == i) continue;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : pq;
            put(a.out, a.out_f32, base + p * ld + 3 * j + qq, (double)acc[comp * nV + j] + sadd[e]);
        }
    }
}

// Galerkin finish: one warp per row r = 3 i + p of the 3V x 3V matrix.  out = Re(scratch); for H,
// the off-diagonal mass-matrix entries C[3i+p][3j+p] = sum of A_f / 48 over the faces f holding
// both i and j (A_f: twice the face area, as igl::doublearea) are added, and the diagonal block
// becomes minus the sum of the row's off-diagonal blocks (C's diagonal entries are overwritten
// there, as in the reference).
template <int KIND>
__global__ void __launch_bounds__(256) static_gal_finish_kernel(const double2 *__restrict__ scr, int nV,
                                                                const double *__restrict__ V,
                                                                const int *__restrict__ F,
                                                                const int *__restrict__ star_off,
                                                                const int *__restrict__ star_face, void *out,
                                                                int out_f32) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const long long n3 = 3LL * nV;
    if (warp >= n3) return;
    const int r = warp, i = r / 3, p = r % 3;
    const double2 *row = scr + (long long)r * n3;
    const long long base = (long long)r * n3;
    double d[3] = {0.0, 0.0, 0.0};  // sums over j != i of the row's column q = 3 j + qq entries
    for (long long c = lane; c < n3; c += 32) {
        const int j = (int)(c / 3), qq = (int)(c % 3);
        const double v = row[c].x;
        if (KIND == SOD_H && j == i) continue;
        put(out, out_f32, base + c, v);
        if (KIND == SOD_H) d[qq] += v;
    }
    if (KIND == SOD_H) {
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d[q] += __shfl_xor_sync(0xffffffffu, d[q], o);
        __syncwarp();  // the lanes' stores above come before lane 0 rewrites the mass-matrix entries
        if (lane == 0) {
            // mass matrix: the row's off-diagonal entries 3 j + p for j in a face with i
            const int s0 = star_off[i], s1 = star_off[i + 1];
            double cdiag = 0.0;
            for (int s = s0; s < s1; s++) {
                const int f = star_face[s];
                for (int c = 0; c < 3; c++) {
                    const int j = F[3 * f + c];
                    if (j == i) continue;
                    double cij = 0.0;  // all faces of i's star holding j, in star order
                    for (int t = s0; t < s1; t++) {
                        const int g = star_face[t];
                        if (F[3 * g] != j && F[3 * g + 1] != j && F[3 * g + 2] != j) continue;
                        const double *a = V + 3 * F[3 * g], *b = V + 3 * F[3 * g + 1], *e = V + 3 * F[3 * g + 2];
                        const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
                        const double w0 = e[0] - a[0], w1 = e[1] - a[1], w2 = e[2] - a[2];
                        const double x = u1 * w2 - u2 * w1, y = u2 * w0 - u0 * w2, z = u0 * w1 - u1 * w0;
                        cij += sqrt(x * x + y * y + z * z) / 48.0;
                    }
                    put(out, out_f32, base + 3LL * j + p, row[3LL * j + p].x + cij);
                }
                const double *a = V + 3 * F[3 * f], *b = V + 3 * F[3 * f + 1], *e = V + 3 * F[3 * f + 2];
                const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
                const double w0 = e[0] - a[0], w1 = e[1] - a[1], w2 = e[2] - a[2];
                const double x = u1 * w2 - u2 * w1, y = u2 * w0 - u0 * w2, z = u0 * w1 - u1 * w0;
                cdiag += 2.0 * sqrt(x * x + y * y + z * z) / 48.0;  // the two other corners of f
            }
            for (int q = 0; q < 3; q++) put(out, out_f32, base + 3LL * i + q, -(d[q] + (q == p ? cdiag : 0.0)));
        }
    }
}

}  // namespace

// Galerkin elastostatic G or H (see the file comment).
static int elastostatic_galerkin(sod_context *ctx, const sod_mesh *m, int kind, double nu, double mu, int order,
                                 int subdiv, int sorder, int ssub, void *dst, int out_dtype) {
    const int nV = m->nV;
    const long long n3 = 3LL * nV;
    SOD_TRY(ctx->freqbuf.ensure(sizeof(double2) * (size_t)(n3 * n3)));
    const double lam = 2.0 * nu * mu / (1.0 - 2.0 * nu);
    KConst<double> k0 = make_kconst(std::sqrt(lam + 2.0 * mu), std::sqrt(mu), 1.0, 0.0, 0.0);
    k0.isr = k0.isi = 0.0;  // 1/s: used by B_angular only
    CollLaunch L{};
    L.mesh = m;
    L.kind_mask = 1 << kind;
    L.nfreq = 1;
    L.kc_host = &k0;
    L.order = order, L.subdiv = subdiv, L.sorder = sorder, L.ssub = ssub;
    L.parts = SOD_PART_ALL;
    L.out[kind] = ctx->freqbuf.p;
    L.out_dtype = SOD_C128;
    for (int kd = 0; kd < 4; kd++) L.freq_stride[kd] = kd <= SOD_H ? n3 * n3 : 0;
    L.stream = ctx->stream;
    SOD_TRY(launch_galerkin(ctx, L));
    const int blocks = (int)((n3 * 32 + 255) / 256);
    if (kind == SOD_G)
        static_gal_finish_kernel<SOD_G><<<blocks, 256, 0, ctx->stream>>>(
            ctx->freqbuf.as<double2>(), nV, m->dV.as<double>(), m->dF.as<int>(), m->gal->astar_off.as<int>(),
            m->gal->astar_face.as<int>(), dst, out_dtype == SOD_F32);
    else
        static_gal_finish_kernel<SOD_H><<<blocks, 256, 0, ctx->stream>>>(
            ctx->freqbuf.as<double2>(), nV, m->dV.as<double>(), m->dF.as<int>(), m->gal->astar_off.as<int>(),
            m->gal->astar_face.as<int>(), dst, out_dtype == SOD_F32);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

extern "C" int sod_elastostatic_assemble(sod_context *ctx, const sod_mesh *m, int kind, int method, double nu,
                                         double mu, int order, int subdiv, int sorder, int ssub, void *out,
                                         int out_dtype) {
    SOD_REQUIRE(ctx && m && m->ctx == ctx, "bad context or mesh");
    SOD_REQUIRE(kind == SOD_G || kind == SOD_H, "elastostatic kind must be G or H");
    SOD_REQUIRE(out != nullptr, "null output");
    SOD_REQUIRE(out_dtype == SOD_F64 || out_dtype == SOD_F32, "output dtype must be SOD_F64 or SOD_F32");
    SOD_REQUIRE(nu > -1.0 && nu < 0.5 && mu > 0.0 && std::isfinite(mu), "need -1 < nu < 1/2 and mu > 0");
    SOD_REQUIRE(sorder >= 1 && sorder <= 5 && ssub >= 1 && ssub <= 8, "singular quadrature order must be 1..5, subdivision 1..8");
    SOD_REQUIRE(method == SOD_COLLOCATION || method == SOD_GALERKIN, "method must be collocation or Galerkin");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    if (method == SOD_GALERKIN) {
        const bool host = !is_device_pointer(out);
        const size_t esz = out_dtype == SOD_F64 ? 8 : 4, bytes = esz * 9 * (size_t)m->nV * m->nV;
        void *dst = out;
        if (host) {
            SOD_TRY(ctx->staging.ensure(bytes));
            dst = ctx->staging.p;
        }
        SOD_TRY(elastostatic_galerkin(ctx, m, kind, nu, mu, order, subdiv, sorder, ssub, dst, out_dtype));
        if (host) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, ctx->stream));
            SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        return SOD_OK;
    }
    PointTable pt;
    SOD_TRY(make_point_table(order, subdiv, pt));
    const int nV = m->nV;
    const long long nslots = m->nbr_off.back();
    for (int i = 0; i < nV; i++)
        SOD_REQUIRE(m->nbr_off[i + 1] - m->nbr_off[i] <= 64, "vertex star too large (more than 64 neighbour slots)");
    // singular blocks
    SOD_TRY(ctx->sing.ensure(sizeof(cd) * (size_t)std::max<long long>(nslots * 9, 1)));
    cd *S[4] = {nullptr, nullptr, nullptr, nullptr};
    S[kind] = ctx->sing.as<cd>();
    SOD_TRY(launch_static_singular(ctx, m, 1 << kind, sorder, ssub, nu, mu, S, ctx->stream));
    // regular pass
    const int NC = kind == SOD_G ? 6 : 9;
    const size_t smem = sizeof(float) * NC * (size_t)nV;
    SOD_REQUIRE(smem + 16 * 1024 <= ctx->smem_optin, "mesh too large for the shared-memory row accumulator");
    int T = ctx->coll_threads > 0 ? ctx->coll_threads : 256;
    T = std::max(32, std::min(512, (T / 32) * 32));
    const sod_mesh::Coloured *col = nullptr;
    SOD_TRY(const_cast<sod_mesh *>(m)->coloured_for(T, &col));
    const bool host = !is_device_pointer(out);
    const size_t esz = out_dtype == SOD_F64 ? 8 : 4, bytes = esz * 9 * (size_t)nV * nV;
    void *dst = out;
    if (host) {
        SOD_TRY(ctx->staging.ensure(bytes));
        dst = ctx->staging.p;
    }
    StaticArgs a{};
    a.nV = nV;
    a.nF = m->nF;
    a.faces = col->dFaces.as<float4>();
    a.canonF = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
    a.color_off = col->dOff.as<int>();
    a.ncolors = col->ncolors;
    a.Vf = m->dVf.as<float>();
    a.canonV = m->has_vmap ? m->dCanon.as<int>() : nullptr;
    a.out = dst;
    a.out_f32 = out_dtype == SOD_F32;
    a.S = S[kind];
    a.nbr_off = m->dNbrOff.as<int>();
    a.nbr_vert = m->dNbrVert.as<int>();
    const double gal = 1.0 / (16.0 * CUDART_PI * (1.0 - nu) * mu);
    a.ga = (float)gal;
    a.gb = (float)((3.0 - 4.0 * nu) * gal);
    const double C = (1.0 - 2.0 * nu) / (8.0 * CUDART_PI * (1.0 - nu));
    a.ha = (float)C;
    a.hb = (float)(-C);
    a.hd = (float)(-3.0 * C / (1.0 - 2.0 * nu));
    const void *fn = kind == SOD_G ? (const void *)static_scatter_kernel<SOD_G> : (const void *)static_scatter_kernel<SOD_H>;
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
    SOD_REQUIRE(smem + attr.sharedSizeBytes <= ctx->smem_optin, "mesh too large for the shared-memory row accumulator");
    SOD_CHECK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(ctx->smem_optin - attr.sharedSizeBytes)));
    if (kind == SOD_G)
        static_scatter_kernel<SOD_G><<<nV, T, smem, ctx->stream>>>(a, pt);
    else
        static_scatter_kernel<SOD_H><<<nV, T, smem, ctx->stream>>>(a, pt);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    if (host) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return SOD_OK;
}
