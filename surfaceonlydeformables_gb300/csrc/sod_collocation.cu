// sod_collocation.cu -- collocation assembly of the Laplace-domain CQBEM matrices on sm_103a.
//
// Replaces, for all field vertices and any set of Laplace frequencies at once, the reference's
// per-row kernels compute_elastodynamic_{G,H,B_trans,B_angular}_kernel_collocation
// (src/elastodynamics_cqbem_{G,H,B_trans,B_angular}_collocation.cu).
//
// Work split (one CTA per (field vertex i, frequency) in every kernel):
//   * regular (non-singular) face integrals, FP32:
//       G, H   : the CTA keeps the row block U[3i:3i+3, :] in shared memory and walks the faces in
//                colour order; faces of one colour share no vertex, so every thread adds its face's
//                three corner blocks without conflicts and the summation order is fixed ->
//                bitwise reproducible results with no atomics.  One barrier separates colours.
//       B_t,B_a: fused; per-face moments in registers, per-thread sums over faces, fixed-order
//                warp/CTA reduction in FP64.
//   * singular (x_i on the face) integrals, FP64, one warp per star face:
//       G, B_t, B_a: fused polar rule (include/integrator_collocation.hpp:19-63) -- the FP64
//                radial terms (two complex exponentials, two psi) are evaluated once for all three;
//       H       : Guiggiani-Gigante CPV rule (include/integrator_collocation.hpp:68-124).
//     Deterministic warp reductions; per-neighbour-slot sums land in small FP64 side buffers
//     that the regular kernels' epilogues add before the single store of each entry.
#include <algorithm>
#include <cstdio>

#include "sod_bmom.cuh"
#include "sod_coll_common.cuh"
#include "sod_dd.cuh"
#include "sod_faces.cuh"
#include "sod_geom.cuh"
#include "sod_internal.h"

namespace sod {

// 1-D Gauss-Legendre rules on [-1,1], orders 1..5 (include/integrator.hpp:117-133 of the reference)
__constant__ double c_glx[5][5];
__constant__ double c_glw[5][5];

// -------------------------------------------------------------------------------------------
// G / H regular scatter kernel.  With BM != 0 (G only) the same pass also integrates B_trans /
// B_angular: the radial terms are shared, each thread adds its faces' B tensors into its own column
// of a shared [NC_B][blockDim] accumulator, and the CTA sums the columns in FP64 in fixed order.
// Dynamic shared memory: NC * nV float2 (row accumulator) + NC_B * blockDim float2.
template <int KIND, int BM>
__device__ __forceinline__ void scatter_body(const CollArgs &a, const PointTable &pt, const KConst<float> k, int i,
                                             int fq, float2 *acc, ColourBar *cb, unsigned &phase) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;  // acc: [NC][nV]
    using BMo = BMom<KIND == SOD_G ? BM : 0>;
    constexpr int NCB = BMo::NC;
    const int nV = a.nV;
    float2 *accB = acc + NC * nV;  // [NCB][blockDim.x]
    for (int t = threadIdx.x; t < NC * nV; t += blockDim.x) acc[t] = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < NCB; c++) accB[c * blockDim.x + threadIdx.x] = make_float2(0.f, 0.f);
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    __syncthreads();
    if (a.do_regular) {
        for (int c = 0; c < a.ncolors; c++) {
            const int fend = a.color_off[c + 1];
            bool ready = c == 0;  // the previous colour's adds are complete
            for (int f = a.color_off[c] + threadIdx.x; f < fend; f += blockDim.x) {
                const FaceRec fr = load_face(a.faces, f);
                if (is_singular(a, i, ci, f, fr)) continue;
                const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
                // corners relative to the collocation point: y - x = sum_l P_l (y_l - x)
                const float3 d1 = make_float3(fr.y1.x - x.x, fr.y1.y - x.y, fr.y1.z - x.z),
                             d2 = make_float3(fr.y2.x - x.x, fr.y2.y - x.y, fr.y2.z - x.z),
                             d3 = make_float3(fr.y3.x - x.x, fr.y3.y - x.y, fr.y3.z - x.z);
                cf part[3][NC];
#pragma unroll
                for (int kk = 0; kk < 3; kk++)
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) part[kk][cc] = mk(0.f, 0.f);
                BMo bm;
                if (NCB) bm.zero();
                for (int q = 0; q < pt.n; q++) {
                    const float4 P = pt.p[q];
                    const float dx = P.x * d1.x + P.y * d2.x + P.z * d3.x;
                    const float dy = P.x * d1.y + P.y * d2.y + P.z * d3.y;
                    const float dz = P.x * d1.z + P.y * d2.z + P.z * d3.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    const float rinv = rsqrtf(r2);
                    const float r = r2 * rinv;
                    const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                    const RadialTerms<float, cf> t = radial<(NCB > 0)>(r, rinv, k);
                    // u without its common factor (1/(4 pi rho r) for G, 1/(4 pi r^2) for H), which
                    // goes into the weight; the tensors are built from per-row vectors, so that each
                    // entry is two packed operations:
                    //   G: u_pq = (al rh_p) rh_q + be d_pq
                    //   H: u_pq = (hd rn rh_p + hb n_p) rh_q + (ha rh_p) n_q + hb rn d_pq
                    cf u[NC];
                    float sc;
                    if (KIND == SOD_G) {
                        cf al, be;
                        g_coeffs_unit(t, k, al, be);
                        sc = k.inv4pirho * rinv;
#pragma unroll
                        for (int p = 0; p < 3; p++) {
                            const cf ar = cmulr(al, rh[p]);
#pragma unroll
                            for (int qq = p; qq < 3; qq++)
                                u[sym_index(p, qq)] = p == qq ? cfmar(ar, rh[qq], be) : cmulr(ar, rh[qq]);
                        }
                    } else {
                        cf ha, hb, hd;
                        h_coeffs_unit(t, k, ha, hb, hd);
                        sc = k.inv4pi * (rinv * rinv);
                        const float rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                        const cf hdr = cmulr(hd, rn), hbr = cmulr(hb, rn);
#pragma unroll
                        for (int p = 0; p < 3; p++) {
                            const cf dp = cfmar(hdr, rh[p], cmulr(hb, nn[p])), bp = cmulr(ha, rh[p]);
#pragma unroll
                            for (int qq = 0; qq < 3; qq++)
                                u[3 * p + qq] = cfmar(dp, rh[qq], p == qq ? cfmar(bp, nn[qq], hbr) : cmulr(bp, nn[qq]));
                        }
                    }
                    const float w = P.w * fr.area * sc;
                    const float wl[3] = {w * P.x, w * P.y, w * P.z};
#pragma unroll
                    for (int kk = 0; kk < 3; kk++)
#pragma unroll
                        for (int cc = 0; cc < NC; cc++) cfma(part[kk][cc], u[cc], wl[kk]);
                    if (NCB) bm.add(t, k, r, rh, nn, P.w);
                }
                if (NCB) {  // this thread's own column: no other thread touches it
                    float2 *col = accB + threadIdx.x;
                    bm.emit(k, nn, fr.area, [&](int cc, cf v) {
                        float2 &s = col[cc * blockDim.x];
                        s.x += v.x;
                        s.y += v.y;
                    });
                }
                if (!ready) {
                    colour_wait(cb, (phase + c - 1) & 1u, a.err);
                    ready = true;
                }
                const int jj[3] = {fr.j0, fr.j1, fr.j2};
#pragma unroll
                for (int kk = 0; kk < 3; kk++)
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) {
                        float2 &s = acc[cc * nV + jj[kk]];
                        s.x += part[kk][cc].x;
                        s.y += part[kk][cc].y;
                    }
            }
            if (c + 1 < a.ncolors) {
                if (!ready) colour_wait(cb, (phase + c - 1) & 1u, a.err);
                colour_arrive(cb);
            }
        }
        if (a.ncolors > 0) phase += (unsigned)(a.ncolors - 1);
        __syncthreads();
    }
    // epilogue: row block 3 x 3nV
    const long long ld = 3LL * nV;
    const long long base = (long long)fq * a.fstride[KIND] + (long long)(3 * i) * ld;
    const int ncol = 3 * nV;
    for (int p = 0; p < 3; p++) {
        for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
            const int j = col / 3, qq = col - 3 * j;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : 3 * p + qq;
            const float2 v = acc[comp * nV + j];
            store_out(a.out[KIND], a.out_c64, base + p * ld + col, v.x, v.y);
        }
    }
    if (a.S[KIND]) {
        __syncthreads();
        const int s0 = a.nbr_off[i], ns = a.nbr_off[i + 1] - s0;
        for (int e = threadIdx.x; e < ns * 9; e += blockDim.x) {
            const int sl = s0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
            const int j = a.nbr_vert[sl];
            const int comp = KIND == SOD_G ? sym_index(p, qq) : pq;
            const float2 v = acc[comp * nV + j];
            const cd sv = a.S[KIND][(long long)fq * a.S_fstride[KIND] + (long long)sl * 9 + pq];
            store_out(a.out[KIND], a.out_c64, base + p * ld + 3 * j + qq, (double)v.x + sv.x, (double)v.y + sv.y);
        }
    }
    if (NCB) {
        // column sums in double-float on the FP32 pipes (FP64 sums here kept GB300's small FP64
        // pipe busy for ~8% of the pass): 32 lanes per component, strided partial sums, fixed xor tree
        __shared__ cd bsum[24];
        __syncthreads();
        const int T = blockDim.x;
        for (int p = threadIdx.x; p < NCB * 32; p += T) {
            const int cc = p >> 5, l = p & 31;
            dd sx = dd{0.f, 0.f}, sy = dd{0.f, 0.f};
            for (int j = l; j < T; j += 32) {
                const float2 v = accB[cc * T + j];
                sx = sx + v.x;
                sy = sy + v.y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sx = sx + dd{__shfl_xor_sync(0xffffffffu, sx.hi, o), __shfl_xor_sync(0xffffffffu, sx.lo, o)};
                sy = sy + dd{__shfl_xor_sync(0xffffffffu, sy.hi, o), __shfl_xor_sync(0xffffffffu, sy.lo, o)};
            }
            if (l == 0) bsum[cc] = mk(dd_to(sx), dd_to(sy));
        }
        __syncthreads();
        store_b<BM>(a, bsum, i, fq);
    }
}

// Fused G + B variants are limited to 384 threads so that they may use up to 170 registers.
// CTA size bound of the scatter variants.  It also sets the register budget, 65536 / 512 = 128 per
// thread: measured on the 2562-vertex object, a 384 bound (165 registers, 12 warps per SM) made the
// G + B pass 18% slower, and a 640 bound (96 registers, with spills) made both passes ~10% slower.
constexpr int SCATTER_MAX_THREADS = 512;
template <int KIND, int BM> constexpr int scatter_max_threads() { return SCATTER_MAX_THREADS; }

template <int KIND, int BM>
__global__ void __launch_bounds__(scatter_max_threads<KIND, BM>(), 1) coll_scatter_kernel(CollArgs a, PointTable pt,
                                                               const __grid_constant__ FreqTable ft) {
    extern __shared__ float2 acc[];
    __shared__ ColourBar cb;
    colour_bar_init(&cb, a.bar_extra);
    unsigned phase = 0;
    scatter_body<KIND, BM>(a, pt, ft.kf[blockIdx.y], a.i0 + blockIdx.x, blockIdx.y, acc, &cb, phase);
}

// Row accumulator in global memory, for meshes whose row block does not fit in shared memory (for
// example H of a 3485-vertex mesh: 9 x 3485 complex FP32 = 251 KB).  A persistent grid walks the
// (vertex, frequency) items in order and each CTA reuses its own slice of the scratch, which stays
// in L2 (grid x slice is a few tens of MB).  The body is the same: colour-ordered adds separated by
// the colour phases (mbarrier release / acquire at CTA scope, which also orders the CTA's
// global-memory accesses), so the sums and their order are those of the shared-memory variant.
template <int KIND, int BM>
__global__ void __launch_bounds__(SCATTER_GLOBAL_THREADS) coll_scatter_global_kernel(CollArgs a, PointTable pt,
                                                                                   const __grid_constant__ FreqTable ft,
                                                                                   float2 *scratch, long long per_cta,
                                                                                   int nvert) {
    float2 *acc = scratch + (size_t)blockIdx.x * per_cta;
    __shared__ ColourBar cb;
    colour_bar_init(&cb, a.bar_extra);
    unsigned phase = 0;
    const int items = nvert * ft.n;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const int fq = it / nvert, i = a.i0 + it % nvert;
        scatter_body<KIND, BM>(a, pt, ft.kf[fq], i, fq, acc, &cb, phase);
        __syncthreads();  // the next item clears the accumulator
    }
}

template <int KIND, int BM>
static int launch_scatter_global(sod_context *ctx, const CollArgs &a, const PointTable &pt, const FreqTable &ft,
                                 int nvert, cudaStream_t stream) {
    const auto fn = coll_scatter_global_kernel<KIND, BM>;
    int per_sm = 0;
    SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SCATTER_GLOBAL_THREADS, 0));
    const int grid = std::max(1, std::min(ctx->num_sms * std::max(per_sm, 1), nvert * ft.n));
    const long long per_cta = (long long)scatter_smem_bytes(KIND, BM, a.nV, SCATTER_GLOBAL_THREADS) / sizeof(float2);
    SOD_TRY(ctx->gacc.ensure(sizeof(float2) * (size_t)grid * per_cta));
    fn<<<grid, SCATTER_GLOBAL_THREADS, 0, stream>>>(a, pt, ft, ctx->gacc.as<float2>(), per_cta, nvert);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// -------------------------------------------------------------------------------------------
// B_trans / B_angular regular reduction kernel (MASK subset of KM_BT | KM_BA), used when G is not
// assembled in the same call: per-thread sums over faces in FP32, fixed-order warp/CTA reduction in
// FP64.
template <int MASK>
__device__ __forceinline__ void reduce_body(const CollArgs &a, const PointTable &pt, const KConst<float> k, int i,
                                            int fq) {
    using BMo = BMom<MASK>;
    constexpr int NC = BMo::NC;
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    cf accl[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) accl[c] = mk(0.f, 0.f);
    if (a.do_regular) {
        for (int f = threadIdx.x; f < a.nF; f += blockDim.x) {
            const FaceRec fr = load_face(a.faces, f);
            if (is_singular(a, i, ci, f, fr)) continue;
            const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
            BMo bm;
            bm.zero();
            for (int q = 0; q < pt.n; q++) {
                const float4 P = pt.p[q];
                const float dx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x - x.x;
                const float dy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y - x.y;
                const float dz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z - x.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float rinv = rsqrtf(r2);
                const float r = r2 * rinv;
                const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                const RadialTerms<float, cf> t = radial<true>(r, rinv, k);
                bm.add(t, k, r, rh, nn, P.w);
            }
            bm.emit(k, nn, fr.area, [&](int c, cf v) { accl[c] = accl[c] + v; });
        }
    }
    // deterministic reduction in FP64: warp butterfly then fixed-order over warps
    __shared__ cd wsum[8][NC];
    __shared__ cd bsum[NC];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NC; c++) {
        double re = accl[c].x, im = accl[c].y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (lane == 0) wsum[warp][c] = mk(re, im);
    }
    __syncthreads();
    const int nw = blockDim.x >> 5;
    for (int c = threadIdx.x; c < NC; c += blockDim.x) {
        cd s = mk(0.0, 0.0);
        for (int w = 0; w < nw; w++) s = s + wsum[w][c];
        bsum[c] = s;
    }
    __syncthreads();
    store_b<MASK>(a, bsum, i, fq);
}

template <int MASK>
__global__ void __launch_bounds__(256) coll_reduce_kernel(CollArgs a, PointTable pt,
                                                          const __grid_constant__ FreqTable ft) {
    reduce_body<MASK>(a, pt, ft.kf[blockIdx.y], a.i0 + blockIdx.x, blockIdx.y);
}

// -------------------------------------------------------------------------------------------
// FP64 singular kernels
struct SingArgs {
    int nV;
    const double *V;  // nV x 3
    const int *F;
    const double *N;
    const int *star_off, *star_face, *star_corner, *star_slot;
    const int *nbr_off;
    int sorder, ssub;
    cd *S[4];
    long long S_fstride[4];
};

constexpr int MAX_STAR = 32;

template <int NVAL> __device__ __forceinline__ void warp_sum(cd (&v)[NVAL]) {
#pragma unroll
    for (int c = 0; c < NVAL; c++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v[c].x += __shfl_xor_sync(0xffffffffu, v[c].x, o);
            v[c].y += __shfl_xor_sync(0xffffffffu, v[c].y, o);
        }
    }
}

// (theta, r, weight) of flattened polar point pidx
__device__ __forceinline__ void polar_point(const Polar &g, int pidx, int sorder, int ssub, double &r, double3 &rh,
                                           double &w) {
    const int nq = sorder * ssub;
    const int ti = pidx / nq, ri = pidx % nq;
    const int ts = ti / sorder, tq = ti % sorder, rs = ri / sorder, rq = ri % sorder;
    const double ta = g.alpha * ts / ssub, tb = g.alpha * (ts + 1) / ssub;
    const double th = (tb - ta) * c_glx[sorder - 1][tq] / 2. + (ta + tb) / 2.;
    double st, ct;
    sincos(th, &st, &ct);
    rh = g.xh * ct + g.yh * st;
    const double rmax = g.a / cos(th - g.beta);
    const double ra = rmax * rs / ssub, rb = rmax * (rs + 1) / ssub;
    r = (rb - ra) * c_glx[sorder - 1][rq] / 2. + (ra + rb) / 2.;
    w = c_glw[sorder - 1][tq] * (tb - ta) / 2. * c_glw[sorder - 1][rq] * (rb - ra) / 2.;
}

// Sum the per-face results of the star of i into the neighbour slots of G/H (9 comps per slot)
template <int NC, int STRIDE>
__device__ __forceinline__ void scatter_slots(const SingArgs &a, int kind, int i, int fq, int s0, int ns,
                                              const cd (*fres)[STRIDE], int off, bool sym) {
    const int n0 = a.nbr_off[i], nsl = a.nbr_off[i + 1] - n0;
    cd *S = a.S[kind] + (long long)fq * a.S_fstride[kind];
    for (int e = threadIdx.x; e < nsl * 9; e += blockDim.x) {
        const int sl = n0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
        const int comp = sym ? sym_index(p, qq) : pq;
        cd s = mk(0.0, 0.0);
        for (int si = 0; si < ns; si++)
            for (int c = 0; c < 3; c++)
                if (a.star_slot[3 * (s0 + si) + c] == sl) s = s + fres[si][off + c * NC + comp];
        S[(long long)sl * 9 + pq] = s;
    }
}

// Fused polar-rule kernel for G (MASK & KM_G), B_trans, B_angular: the FP64 radial terms are
// evaluated once per point for every requested kind.
template <int MASK>
__device__ __forceinline__ void polar_body(const SingArgs &a, const KConst<double> k, int i, int fq) {
    constexpr bool DG = (MASK & KM_G) != 0, DT = (MASK & KM_BT) != 0, DA = (MASK & KM_BA) != 0;
    constexpr int NG = DG ? 18 : 0, NT = DT ? 6 : 0, NA = DA ? 18 : 0;  // per-face result sizes
    constexpr int OG = 0, OT = NG, OA = NG + NT, STRIDE = NG + NT + NA;
    __shared__ cd fres[MAX_STAR][STRIDE];
    const int s0 = a.star_off[i], ns = min(a.star_off[i + 1] - a.star_off[i], MAX_STAR);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nq = a.sorder * a.ssub;
    // accumulators: G corners x 6 sym comps, B_trans moments (Ms[3], Md), B_angular moments
    // (M1[6], M0, SB, SC)
    constexpr int NACC = (DG ? 18 : 0) + (DT ? 4 : 0) + (DA ? 9 : 0);
    constexpr int AG = 0, AT = DG ? 18 : 0, AA = AT + (DT ? 4 : 0);
    for (int si = warp; si < ns; si += nw) {
        const int f = a.star_face[s0 + si], sc = a.star_corner[s0 + si];
        const int jj[3] = {a.F[3 * f + sc], a.F[3 * f + (sc + 1) % 3], a.F[3 * f + (sc + 2) % 3]};
        const double3 y1 = ld3(a.V, jj[0]), y2 = ld3(a.V, jj[1]), y3 = ld3(a.V, jj[2]);
        const double3 n = ld3(a.N, f);
        const double nn[3] = {n.x, n.y, n.z};
        cd acc[NACC];
#pragma unroll
        for (int c = 0; c < NACC; c++) acc[c] = mk(0.0, 0.0);
        const Polar g = polar_setup(y1, y2, y3);
        for (int pidx = lane; pidx < nq * nq; pidx += 32) {
            double r, w;
            double3 rh;
            polar_point(g, pidx, a.sorder, a.ssub, r, rh, w);
            const double rr[3] = {rh.x, rh.y, rh.z};
            const RadialTerms<double, cd> t = radial<double, cd>(r, k);
            if (DG) {
                double L[3];
                bary_clamped(y1 + rh * r, y1, y2, y3, L);
                cd al, be;
                g_coeffs(t, k, 1.0, al, be);  // r * u
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int qq = p; qq < 3; qq++) {
                        cd v = al * (rr[p] * rr[qq]);
                        if (p == qq) v = v + be;
#pragma unroll
                        for (int c = 0; c < 3; c++) cfma(acc[AG + c * 6 + sym_index(p, qq)], v, w * L[c]);
                    }
            }
            if (DT) {
                cd sy, di;
                bt_coeffs(t, k, r, sy, di);  // r * b
                const cd ws = sy * w;
#pragma unroll
                for (int p = 0; p < 3; p++) cfma(acc[AT + p], ws, rr[p]);
                cfma(acc[AT + 3], di, w * dot3(rh, n));
            }
            if (DA) {
                cd A, Bq, Cq;
                ba_coeffs(t, k, r, r, A, Bq, Cq);  // r * b
                const cd wA = A * w;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int kk = p; kk < 3; kk++) cfma(acc[AA + sym_index(p, kk)], wA, rr[p] * rr[kk]);
                acc[AA + 6] = acc[AA + 6] + wA;
                cfma(acc[AA + 7], Bq, w);
                cfma(acc[AA + 8], Cq, w);
            }
        }
        warp_sum<NACC>(acc);
        if (lane == 0) {
            if (DG)
                for (int c = 0; c < 18; c++) fres[si][OG + c] = acc[AG + c];
            if (DT)
                for (int p = 0; p < 3; p++)
                    for (int qq = p; qq < 3; qq++) {
                        cd v = acc[AT + p] * nn[qq] + acc[AT + qq] * nn[p];
                        if (p == qq) v = v + acc[AT + 3];
                        fres[si][OT + sym_index(p, qq)] = v;
                    }
            if (DA) {
                const cd M0B = acc[AA + 6] + acc[AA + 7];
                for (int p = 0; p < 3; p++)
                    for (int qq = p; qq < 3; qq++)
                        for (int kk = 0; kk < 3; kk++) {
                            cd v = acc[AA + sym_index(p, kk)] * nn[qq] + acc[AA + sym_index(qq, kk)] * nn[p];
                            v = v + M0B * ((qq == kk ? nn[p] : 0.0) + (p == kk ? nn[qq] : 0.0));
                            if (p == qq) v = v + acc[AA + 8] * nn[kk];
                            fres[si][OA + 3 * sym_index(p, qq) + kk] = v;
                        }
            }
        }
    }
    __syncthreads();
    if (DG) scatter_slots<6, STRIDE>(a, SOD_G, i, fq, s0, ns, fres, OG, true);
    if (DT) {
        cd *S = a.S[SOD_B_TRANS] + (long long)fq * a.S_fstride[SOD_B_TRANS] + (long long)i * 9;
        for (int e = threadIdx.x; e < 9; e += blockDim.x) {
            cd s = mk(0.0, 0.0);
            for (int si = 0; si < ns; si++) s = s + fres[si][OT + sym_index(e / 3, e % 3)];
            S[e] = s;
        }
    }
    if (DA) {
        cd *S = a.S[SOD_B_ANGULAR] + (long long)fq * a.S_fstride[SOD_B_ANGULAR] + (long long)i * 27;
        for (int e = threadIdx.x; e < 27; e += blockDim.x) {
            const int p = e / 9, qq = (e / 3) % 3, kk = e % 3;
            cd s = mk(0.0, 0.0);
            for (int si = 0; si < ns; si++) s = s + fres[si][OA + 3 * sym_index(p, qq) + kk];
            S[e] = s;
        }
    }
}

template <int MASK>
__global__ void __launch_bounds__(256) coll_polar_kernel(SingArgs a, const __grid_constant__ FreqTable ft) {
    polar_body<MASK>(a, ft.kd[blockIdx.y], blockIdx.x, blockIdx.y);
}

// Guiggiani-Gigante rule for the strongly singular H faces (include/integrator_collocation.hpp:68-124)
__device__ __forceinline__ void guiggiani_body(const SingArgs &a, const KConst<double> k, int i, int fq) {
    constexpr int NC = 9;
    __shared__ cd fres[MAX_STAR][3 * NC];
    const int s0 = a.star_off[i], ns = min(a.star_off[i + 1] - a.star_off[i], MAX_STAR);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nq = a.sorder * a.ssub;
    for (int si = warp; si < ns; si += nw) {
        const int f = a.star_face[s0 + si], sc = a.star_corner[s0 + si];
        const int jj[3] = {a.F[3 * f + sc], a.F[3 * f + (sc + 1) % 3], a.F[3 * f + (sc + 2) % 3]};
        const double3 y1 = ld3(a.V, jj[0]), y2 = ld3(a.V, jj[1]), y3 = ld3(a.V, jj[2]);
        const double3 n = ld3(a.N, f);
        const double nn[3] = {n.x, n.y, n.z};
        cd acc[3 * NC];
#pragma unroll
        for (int c = 0; c < 3 * NC; c++) acc[c] = mk(0.0, 0.0);
        const double3 v1 = y2 - y1, v2 = y3 - y1;
        const double J = norm3(cross3(v1, v2));
        const double kc = k.inv4pi * k.kappa;
        const double tmax = CUDART_PI / 2.;
        for (int pidx = lane; pidx < nq * nq; pidx += 32) {
            const int ti = pidx / nq, ri = pidx % nq;
            const int ts = ti / a.sorder, tq = ti % a.sorder, rs = ri / a.sorder, rq = ri % a.sorder;
            const double ta = tmax * ts / a.ssub, tb = tmax * (ts + 1) / a.ssub;
            const double th = (tb - ta) * c_glx[a.sorder - 1][tq] / 2. + (ta + tb) / 2.;
            const double wt = c_glw[a.sorder - 1][tq] * (tb - ta) / 2.;
            double st, ct;
            sincos(th, &st, &ct);
            const double3 Av = v1 * ct + v2 * st;
            const double A = norm3(Av);
            const double3 Ah = nrmz(Av);
            const double ah[3] = {Ah.x, Ah.y, Ah.z};
            const double rho_bar = 1. / (cos(th - CUDART_PI / 4.) * sqrt(2.));
            const double ra = rho_bar * rs / a.ssub, rb = rho_bar * (rs + 1) / a.ssub;
            const double rho = (rb - ra) * c_glx[a.sorder - 1][rq] / 2. + (ra + rb) / 2.;
            const double w = wt * c_glw[a.sorder - 1][rq] * (rb - ra) / 2.;
            const double L[3] = {1. - rho * (ct + st), rho * ct, rho * st};
            const double3 rv = Av * rho;
            const double r = norm3(rv);
            const double3 rh = nrmz(rv);
            const double rr[3] = {rh.x, rh.y, rh.z};
            const double rn = dot3(rh, n);
            const RadialTerms<double, cd> t = radial<double, cd>(r, k);
            cd ha, hb, hd;
            h_coeffs(t, k, 1.0 / (r * r), ha, hb, hd);
            const double logt = (ri == 0) ? log(rho_bar * A) : 0.0;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int qq = 0; qq < 3; qq++) {
                    cd v = ha * (rr[p] * nn[qq]) + hb * (nn[p] * rr[qq]) + hd * (rn * rr[p] * rr[qq]);
                    if (p == qq) v = v + hb * rn;
                    const double f0 = kc * (ah[p] * nn[qq] - ah[qq] * nn[p]) / (A * A) * J;
#pragma unroll
                    for (int c = 0; c < 3; c++) cfma(acc[c * NC + 3 * p + qq], v, w * L[c] * J * rho);
                    acc[3 * p + qq].x += -w * f0 / rho + wt * f0 * logt;
                }
        }
        warp_sum<3 * NC>(acc);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3 * NC; c++) fres[si][c] = acc[c];
        }
    }
    __syncthreads();
    scatter_slots<9, 3 * NC>(a, SOD_H, i, fq, s0, ns, fres, 0, false);
}

__global__ void __launch_bounds__(256) coll_guiggiani_kernel(SingArgs a, const __grid_constant__ FreqTable ft) {
    guiggiani_body(a, ft.kd[blockIdx.y], blockIdx.x, blockIdx.y);
}

// -------------------------------------------------------------------------------------------
// Persistent batched kernels: one launch per kernel type covers many objects of uneven size.  Each
// CTA pulls (object, field vertex, frequency) items from a global counter until the list is empty;
// the lists are ordered largest object first so the tail is made of cheap items.  The per-item
// work is the same device function as in the per-object kernels, so an object's matrices are the
// same whether it is assembled alone or in a batch.
__device__ __forceinline__ int next_item(int *counter, int *s_item) {
    if (threadIdx.x == 0) *s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = *s_item;
    __syncthreads();
    return it;
}

// Kernel arguments of one batched launch, in kernel-parameter (constant bank) space: the point
// table and up to BATCH_OBJS objects' arguments, indexed by the item's object slot.
struct BatchLaunchArgs {
    PointTable pt;
    int nobj;
    int kc_off[BATCH_OBJS];  // first entry of the object in the batch's per-frequency constants
    CollArgs a[BATCH_OBJS];
};
static_assert(sizeof(BatchLaunchArgs) <= 32000, "batched launch arguments exceed the kernel parameter space");

template <int KIND, int BM>
__global__ void __launch_bounds__(scatter_max_threads<KIND, BM>(), 1) batch_scatter_kernel(const __grid_constant__ BatchLaunchArgs p,
                                                               const int4 *__restrict__ items, int nitems,
                                                               int *counter, const KConst<float> *__restrict__ kcf) {
    extern __shared__ float2 acc[];
    __shared__ int s_item;
    __shared__ ColourBar cb;
    colour_bar_init(&cb);
    unsigned phase = 0;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= nitems) break;
        const int4 w = items[it];
        scatter_body<KIND, BM>(p.a[w.x], p.pt, kcf[p.kc_off[w.x] + w.z], w.y, w.z, acc, &cb, phase);
    }
}

// The batched scatter with each CTA's row accumulator in a slice of global memory (objects whose row
// block exceeds shared memory; see coll_scatter_global_kernel).
template <int KIND, int BM>
__global__ void __launch_bounds__(256) batch_scatter_global_kernel(const __grid_constant__ BatchLaunchArgs p,
                                                                   const int4 *__restrict__ items, int nitems,
                                                                   int *counter, const KConst<float> *__restrict__ kcf,
                                                                   float2 *scratch, long long per_cta) {
    float2 *acc = scratch + (size_t)blockIdx.x * per_cta;
    __shared__ int s_item;
    __shared__ ColourBar cb;
    colour_bar_init(&cb);
    unsigned phase = 0;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= nitems) break;
        const int4 w = items[it];
        scatter_body<KIND, BM>(p.a[w.x], p.pt, kcf[p.kc_off[w.x] + w.z], w.y, w.z, acc, &cb, phase);
    }
}

template <int MASK>
__global__ void __launch_bounds__(256) batch_reduce_kernel(const __grid_constant__ BatchLaunchArgs p,
                                                           const int4 *__restrict__ items, int nitems, int *counter,
                                                           const KConst<float> *__restrict__ kcf) {
    __shared__ int s_item;
    for (;;) {
        const int it = next_item(counter, &s_item);
        if (it >= nitems) break;
        const int4 w = items[it];
        reduce_body<MASK>(p.a[w.x], p.pt, kcf[p.kc_off[w.x] + w.z], w.y, w.z);
    }
}

// -------------------------------------------------------------------------------------------
// host side

}  // namespace sod

int take_device_error(sod_context *ctx) {
    int word = 0;
    SOD_CHECK_CUDA(cudaMemcpy(&word, ctx->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (word == 0) return SOD_OK;
    SOD_CHECK_CUDA(cudaMemset(ctx->dev_err.p, 0, sizeof(int)));
    sod::set_error("a scatter kernel's bounded colour-phase wait expired; its results are not valid");
    return SOD_ERR_TIMEOUT;
}

namespace sod {
static std::atomic<bool> g_const_ready[64];  // per device; the set-up is idempotent

static int ensure_gl_constants(int device) {
    if (device >= 0 && device < 64 && g_const_ready[device]) return SOD_OK;
    double x[5][5] = {}, w[5][5] = {};
    for (int o = 1; o <= 5; o++) {
        int n;
        const double(*t)[2] = gl_rule_table(o, n);
        for (int q = 0; q < n; q++) x[o - 1][q] = t[q][0], w[o - 1][q] = t[q][1];
    }
    SOD_CHECK_CUDA(cudaMemcpyToSymbol(c_glx, x, sizeof(x)));
    SOD_CHECK_CUDA(cudaMemcpyToSymbol(c_glw, w, sizeof(w)));
    if (device >= 0 && device < 64) g_const_ready[device] = true;
    return SOD_OK;
}

// Scatter kernel variants: G or H, and for G the B kinds fused into the same pass.
static const void *scatter_fn(int kind, int bm, bool batch) {
    if (kind == SOD_H) return batch ? (const void *)batch_scatter_kernel<SOD_H, 0> : (const void *)coll_scatter_kernel<SOD_H, 0>;
    switch (bm) {
    case KM_BT: return batch ? (const void *)batch_scatter_kernel<SOD_G, KM_BT> : (const void *)coll_scatter_kernel<SOD_G, KM_BT>;
    case KM_BA: return batch ? (const void *)batch_scatter_kernel<SOD_G, KM_BA> : (const void *)coll_scatter_kernel<SOD_G, KM_BA>;
    case KM_BT | KM_BA:
        return batch ? (const void *)batch_scatter_kernel<SOD_G, KM_BT | KM_BA>
                     : (const void *)coll_scatter_kernel<SOD_G, KM_BT | KM_BA>;
    default: return batch ? (const void *)batch_scatter_kernel<SOD_G, 0> : (const void *)coll_scatter_kernel<SOD_G, 0>;
    }
}

size_t scatter_smem_bytes(int kind, int bm, int nV, int threads) {
    const int nc = kind == SOD_G ? 6 : 9;
    const int ncb = kind == SOD_G ? ((bm & KM_BT) ? 6 : 0) + ((bm & KM_BA) ? 18 : 0) : 0;
    return sizeof(float2) * ((size_t)nc * nV + (size_t)ncb * threads);
}

// Raise every scatter variant's dynamic shared-memory limit to the device maximum (once per device).
static std::atomic<bool> g_scatter_ready[64];  // per device; the set-up is idempotent
static int prepare_scatter(sod_context *ctx) {
    if (ctx->device >= 0 && ctx->device < 64 && g_scatter_ready[ctx->device]) return SOD_OK;
    const int bms[4] = {0, KM_BT, KM_BA, KM_BT | KM_BA};
    for (int batch = 0; batch < 2; batch++)
        for (int kind = 0; kind < 2; kind++)
            for (int v = 0; v < (kind == SOD_G ? 4 : 1); v++) {
                const void *fn = scatter_fn(kind, bms[v], batch != 0);
                cudaFuncAttributes attr;
                SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
                SOD_CHECK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)(ctx->smem_optin - attr.sharedSizeBytes)));
                SOD_CHECK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
            }
    if (ctx->device >= 0 && ctx->device < 64) g_scatter_ready[ctx->device] = true;
    return SOD_OK;
}

int scatter_occupancy(sod_context *ctx, int kind, int bm, bool batch, int threads, size_t smem, int *per_sm) {
    SOD_TRY(prepare_scatter(ctx));
    *per_sm = 0;
    const void *fn = scatter_fn(kind, bm, batch);
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
    if (smem + attr.sharedSizeBytes > ctx->smem_optin || threads > attr.maxThreadsPerBlock) return SOD_OK;
    SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fn, threads, smem));
    return SOD_OK;
}

// Autotuner for the scatter kernels.  A CTA walks the faces colour by colour with one barrier per
// colour, so a colour with fewer faces than threads leaves lanes idle and a CTA with few warps
// cannot hide the barrier.  For every feasible CTA size T (multiples of 32 up to the variant's
// limit) the mesh is coloured with capacity T and the cost is modelled as
//     slots(T) / occupancy(T),   slots = ncolours * T,
//     occupancy = min(1, resident warps per SM / 24)  (from the CUDA occupancy calculator with the
//     variant's registers and shared memory).
// The choice depends only on the mesh and the device, so results stay bitwise reproducible.
int autotune_scatter_threads(sod_context *ctx, sod_mesh *m, int kind, int bm, int *threads) {
    const int key = kind * 16 + bm;
    std::lock_guard<std::recursive_mutex> lock(m->sched_mu);
    auto it = m->tuned.find(key);
    if (it != m->tuned.end()) {
        *threads = it->second;
        return SOD_OK;
    }
    SOD_TRY(prepare_scatter(ctx));
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, scatter_fn(kind, bm, false)));
    double best = 1e300;
    int bestT = 0;
    for (int T = 32; T <= std::min(SCATTER_MAX_THREADS, attr.maxThreadsPerBlock); T += 32) {
        const size_t smem = scatter_smem_bytes(kind, bm, m->nV, T);
        int per_sm = 0;
        SOD_TRY(scatter_occupancy(ctx, kind, bm, false, T, smem, &per_sm));
        if (per_sm <= 0) continue;
        const sod_mesh::Coloured *col = nullptr;
        SOD_TRY(m->coloured_for(T, &col));
        const double warps = (double)per_sm * T / 32.0;
        const double occ = std::min(1.0, warps / 24.0);
        const double cost = (double)col->ncolors * T / occ;
        if (cost < best * 0.999) {
            best = cost;
            bestT = T;
        }
    }
    if (bestT == 0) {
        set_error("mesh too large for the shared-memory row accumulator (" + std::to_string(m->nV) + " vertices)");
        return SOD_ERR_UNSUPPORTED;
    }
    m->tuned[key] = bestT;
    *threads = bestT;
    return SOD_OK;
}

int launch_collocation(sod_context *ctx, const CollLaunch &L) {
    const sod_mesh *m = L.mesh;
    const int mask = L.kind_mask;
    SOD_REQUIRE(mask > 0 && mask < 16, "empty kind set");
    SOD_TRY(ensure_gl_constants(ctx->device));
    PointTable pt;
    SOD_TRY(make_point_table(L.order, L.subdiv, pt));
    SOD_REQUIRE(L.sorder >= 1 && L.sorder <= 5 && L.ssub >= 1 && L.ssub <= 8,
                "singular quadrature order must be 1..5, subdivision 1..8");
    const bool sing = (L.parts & SOD_PART_SINGULAR) != 0;
    const int chunk = std::min(L.nfreq, MAX_FREQ_PER_LAUNCH);
    // singular side buffers (per kind, one chunk of frequencies)
    const long long nslots = m->nbr_off.back();
    const long long sfs[4] = {nslots * 9, nslots * 9, (long long)m->nV * 9, (long long)m->nV * 27};
    long long soff[4] = {0, 0, 0, 0}, stot = 0;
    for (int kd = 0; kd < 4; kd++)
        if (mask & (1 << kd)) {
            soff[kd] = stot;
            stot += sfs[kd] * chunk;
        }
    cd *Sb = nullptr;
    if (sing) {
        SOD_TRY(ctx->sing.ensure(sizeof(cd) * (size_t)stot));
        Sb = ctx->sing.as<cd>();
    }
    // scatter kernel configuration; with G requested the B kinds ride along in the G pass
    const int bmG = (mask & KM_G) ? (mask & (KM_BT | KM_BA)) : 0;
    int threads[2] = {0, 0};
    const sod_mesh::Coloured *col[2] = {nullptr, nullptr};
    size_t smem[2] = {0, 0};
    bool global[2] = {false, false};  // row accumulator in global memory (row block too large for shared memory)
    for (int kd = 0; kd < 2; kd++) {
        if (!(mask & (1 << kd))) continue;
        if (L.compensated) {  // the compensated pass has its own CTA size and launcher
            SOD_TRY(comp_scatter_threads(ctx, const_cast<sod_mesh *>(m), kd, &threads[kd]));
            SOD_TRY(const_cast<sod_mesh *>(m)->coloured_for(threads[kd], &col[kd]));
            continue;
        }
        const int bm = kd == SOD_G ? bmG : 0;
        int T = ctx->coll_threads;
        int rc = SOD_OK;
        if (T <= 0) rc = autotune_scatter_threads(ctx, const_cast<sod_mesh *>(m), kd, bm, &T);
        int per_sm = 0;
        if (rc == SOD_OK) {
            cudaFuncAttributes attr;
            SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, scatter_fn(kd, bm, false)));
            T = std::max(32, std::min(std::min(SCATTER_MAX_THREADS, attr.maxThreadsPerBlock), (T / 32) * 32));
            smem[kd] = scatter_smem_bytes(kd, bm, m->nV, T);
            SOD_TRY(scatter_occupancy(ctx, kd, bm, false, T, smem[kd], &per_sm));
        } else if (rc != SOD_ERR_UNSUPPORTED) {
            return rc;
        }
        if (per_sm <= 0) {
            global[kd] = true;
            T = SCATTER_GLOBAL_THREADS;
            smem[kd] = 0;
        }
        threads[kd] = T;
        SOD_TRY(const_cast<sod_mesh *>(m)->coloured_for(T, &col[kd]));
    }
    const size_t esz = L.out_dtype == SOD_C64 ? 8 : 16;
    // host destinations: row chunks of whole waves of the scatter grid, each chunk's rows copied on
    // the copy stream while the next chunk computes
    const bool to_host = L.host[0] || L.host[1] || L.host[2] || L.host[3];
    int vchunk = m->nV;
    if (to_host) {
        int wave = ctx->num_sms;
        for (int kd = 0; kd < 2 && !L.compensated; kd++)
            if (mask & (1 << kd)) {
                int per_sm = 1;
                SOD_TRY(scatter_occupancy(ctx, kd, kd == SOD_G ? bmG : 0, false, threads[kd], smem[kd], &per_sm));
                wave = std::max(wave, ctx->num_sms * std::max(per_sm, 1));
            }
        const int target = (m->nV + 11) / 12;  // about twelve chunks: the first compute and the last copy are not overlapped
        vchunk = std::min(m->nV, std::max(wave, (target + wave - 1) / wave * wave));
        if (!ctx->copy_stream) SOD_CHECK_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        const size_t need = (size_t)((m->nV + vchunk - 1) / vchunk) + 1;
        while (ctx->chunk_events.size() < need) {
            cudaEvent_t e;
            SOD_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ctx->chunk_events.push_back(e);
        }
    }
    for (int f0 = 0; f0 < L.nfreq; f0 += chunk) {
        const int nf = std::min(chunk, L.nfreq - f0);
        FreqTable ft;
        ft.n = nf;
        for (int l = 0; l < nf; l++) {
            ft.kd[l] = L.kc_host[f0 + l];
            ft.kf[l] = to_float(ft.kd[l]);
        }
        SingArgs sa{};
        sa.nV = m->nV;
        sa.V = m->dV.as<double>();
        sa.F = m->dF.as<int>();
        sa.N = m->dN.as<double>();
        sa.star_off = m->dStarOff.as<int>();
        sa.star_face = m->dStarFace.as<int>();
        sa.star_corner = m->dStarCorner.as<int>();
        sa.star_slot = m->dStarSlot.as<int>();
        sa.nbr_off = m->dNbrOff.as<int>();
        sa.sorder = L.sorder;
        sa.ssub = L.ssub;
        for (int kd = 0; kd < 4; kd++) {
            sa.S[kd] = (sing && (mask & (1 << kd))) ? Sb + soff[kd] : nullptr;
            sa.S_fstride[kd] = sfs[kd];
        }
        if (sing) SOD_TRY(launch_singular(ctx, m, mask, L.sorder, L.ssub, ft.kd, nf, sa.S, sa.S_fstride, L.stream));
        CollArgs a{};
        a.err = ctx->dev_err.as<int>();
        a.bar_extra = ctx->wait_test ? 1 : 0;
        a.nV = m->nV;
        a.nF = m->nF;
        a.Vf = m->dVf.as<float>();
        a.canonV = m->has_vmap ? m->dCanon.as<int>() : nullptr;
        a.out_c64 = L.out_dtype == SOD_C64;
        a.do_regular = (L.parts & SOD_PART_REGULAR) != 0;
        a.nbr_off = m->dNbrOff.as<int>();
        a.nbr_vert = m->dNbrVert.as<int>();
        for (int kd = 0; kd < 4; kd++) {
            a.out[kd] = L.out[kd] ? static_cast<char *>(L.out[kd]) + (size_t)f0 * (size_t)L.freq_stride[kd] * esz : nullptr;
            a.fstride[kd] = L.freq_stride[kd];
            a.S[kd] = sa.S[kd];
            a.S_fstride[kd] = sfs[kd];
        }
        for (int v0 = 0, ci = 0; v0 < m->nV; v0 += vchunk, ci++) {
            const int v1 = std::min(m->nV, v0 + vchunk);
            const dim3 grid(v1 - v0, nf);
            a.i0 = v0;
            if (L.compensated)
                SOD_TRY(launch_regular_compensated(ctx, m, a, mask, col[SOD_G], col[SOD_H], threads, pt, ft, v1 - v0,
                                                   L.stream));
            for (int kd = 0; kd < 2 && !L.compensated; kd++) {
                if (!(mask & (1 << kd))) continue;
                a.faces = col[kd]->dFaces.as<float4>();
                a.canonF = m->has_vmap ? col[kd]->dCanonF.as<int4>() : nullptr;
                a.color_off = col[kd]->dOff.as<int>();
                a.ncolors = col[kd]->ncolors;
                if (global[kd]) {
                    const int nv = v1 - v0;
                    if (kd == SOD_H) SOD_TRY((launch_scatter_global<SOD_H, 0>(ctx, a, pt, ft, nv, L.stream)));
                    else if (bmG == KM_BT) SOD_TRY((launch_scatter_global<SOD_G, KM_BT>(ctx, a, pt, ft, nv, L.stream)));
                    else if (bmG == KM_BA) SOD_TRY((launch_scatter_global<SOD_G, KM_BA>(ctx, a, pt, ft, nv, L.stream)));
                    else if (bmG) SOD_TRY((launch_scatter_global<SOD_G, KM_BT | KM_BA>(ctx, a, pt, ft, nv, L.stream)));
                    else SOD_TRY((launch_scatter_global<SOD_G, 0>(ctx, a, pt, ft, nv, L.stream)));
                    continue;
                }
                if (kd == SOD_H)
                    coll_scatter_kernel<SOD_H, 0><<<grid, threads[kd], smem[kd], L.stream>>>(a, pt, ft);
                else if (bmG == KM_BT)
                    coll_scatter_kernel<SOD_G, KM_BT><<<grid, threads[kd], smem[kd], L.stream>>>(a, pt, ft);
                else if (bmG == KM_BA)
                    coll_scatter_kernel<SOD_G, KM_BA><<<grid, threads[kd], smem[kd], L.stream>>>(a, pt, ft);
                else if (bmG)
                    coll_scatter_kernel<SOD_G, KM_BT | KM_BA><<<grid, threads[kd], smem[kd], L.stream>>>(a, pt, ft);
                else
                    coll_scatter_kernel<SOD_G, 0><<<grid, threads[kd], smem[kd], L.stream>>>(a, pt, ft);
                SOD_CHECK_CUDA(cudaGetLastError());
                ctx->count();
            }
            const int rm = (mask & KM_G) || L.compensated ? 0 : (mask & (KM_BT | KM_BA));
            if (rm) {
                a.faces = m->dFacesNat.as<float4>();
                a.canonF = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
                if (rm == KM_BT)
                    coll_reduce_kernel<KM_BT><<<grid, 256, 0, L.stream>>>(a, pt, ft);
                else if (rm == KM_BA)
                    coll_reduce_kernel<KM_BA><<<grid, 256, 0, L.stream>>>(a, pt, ft);
                else
                    coll_reduce_kernel<KM_BT | KM_BA><<<grid, 256, 0, L.stream>>>(a, pt, ft);
                SOD_CHECK_CUDA(cudaGetLastError());
                ctx->count();
            }
            if (to_host) {  // this chunk's rows (vertices v0..v1-1) of every kind and frequency to the host
                cudaEvent_t e = ctx->chunk_events[ci];
                SOD_CHECK_CUDA(cudaEventRecord(e, L.stream));
                SOD_CHECK_CUDA(cudaStreamWaitEvent(ctx->copy_stream, e, 0));
                for (int kd = 0; kd < 4; kd++) {
                    if (!L.host[kd]) continue;
                    const size_t ncol = kd <= SOD_H ? 3 * (size_t)m->nV : (kd == SOD_B_TRANS ? 3 : 9);
                    for (int f = 0; f < nf; f++) {
                        const size_t off = ((size_t)(f0 + f) * (size_t)L.freq_stride[kd] + 3 * (size_t)v0 * ncol) * esz;
                        SOD_CHECK_CUDA(cudaMemcpyAsync(static_cast<char *>(L.host[kd]) + off,
                                                       static_cast<const char *>(L.out[kd]) + off,
                                                       3 * (size_t)(v1 - v0) * ncol * esz, cudaMemcpyDeviceToHost,
                                                       ctx->copy_stream));
                    }
                }
            }
        }
    }
    if (to_host) {  // the caller's stream sees the copies complete
        cudaEvent_t e = ctx->chunk_events.back();
        SOD_CHECK_CUDA(cudaEventRecord(e, ctx->copy_stream));
        SOD_CHECK_CUDA(cudaStreamWaitEvent(L.stream, e, 0));
    }
    return SOD_OK;
}

// -------------------------------------------------------------------------------------------
// Launcher that allocates nothing (for sod_cqbem_assemble_noalloc): the singular side buffer is
// caller-provided device memory of `scratch_elems` complex doubles, the scatter schedule must
// already exist on the mesh, the point table is built on the stack, and frequencies are chunked so
// that one chunk's side buffer fits the scratch.
static int point_table_on_stack(int order, int subdiv, PointTable &pt) {
    int nq = 0;
    const double(*rule)[4] = tri_rule_table(order, nq);
    SOD_REQUIRE(rule != nullptr, "triangle quadrature order must be 1..5 or 7 (13-point rule)");
    SOD_REQUIRE(subdiv >= 1 && subdiv <= 4, "quadrature subdivision must be 1..4");
    double tri[16][9];
    int nt = 0;
    const double h = 1.0 / subdiv;
    auto push = [&](double a0, double b0, double a1, double b1, double a2, double b2) {
        const double c[9] = {1 - a0 - b0, a0, b0, 1 - a1 - b1, a1, b1, 1 - a2 - b2, a2, b2};
        for (int t = 0; t < 9; t++) tri[nt][t] = c[t];
        nt++;
    };
    push(0, 0, h, 0, 0, h);
    for (int i = 0; i < subdiv; i++)
        for (int j = 0; j < subdiv; j++) {
            if (!(i == 0 && j == 0) && i + j < subdiv) push(i * h, j * h, (i + 1) * h, j * h, i * h, (j + 1) * h);
            if (i + j < subdiv - 1) push((i + 1) * h, (j + 1) * h, (i + 1) * h, j * h, i * h, (j + 1) * h);
        }
    SOD_REQUIRE(nt * nq <= MAX_TRI_PTS, "too many quadrature points");
    pt.n = 0;
    const double ws = 1.0 / ((double)subdiv * subdiv);
    for (int t = 0; t < nt; t++)
        for (int q = 0; q < nq; q++) {
            double l[3];
            for (int c = 0; c < 3; c++) l[c] = rule[q][0] * tri[t][c] + rule[q][1] * tri[t][3 + c] + rule[q][2] * tri[t][6 + c];
            pt.p[pt.n++] = make_float4((float)l[0], (float)l[1], (float)l[2], (float)(rule[q][3] * ws));
        }
    return SOD_OK;
}

int launch_collocation_prealloc(sod_context *ctx, const sod_mesh *m, int kind, double c1, double c2, double rho,
                                const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, void *out,
                                int out_dtype, cd *scratch, long long scratch_elems, cudaStream_t stream) {
    SOD_REQUIRE(kind >= SOD_G && kind <= SOD_B_ANGULAR, "kind must be G, H, B_trans or B_angular");
    SOD_REQUIRE(sorder >= 1 && sorder <= 5 && ssub >= 1 && ssub <= 8, "singular quadrature order must be 1..5, subdivision 1..8");
    SOD_TRY(ensure_gl_constants(ctx->device));
    PointTable pt;
    SOD_TRY(point_table_on_stack(order, subdiv, pt));
    const long long nslots = m->nbr_off.back();
    const long long sfs = kind <= SOD_H ? nslots * 9 : (long long)m->nV * (kind == SOD_B_TRANS ? 9 : 27);
    const long long fit = scratch_elems / sfs;
    if (fit < 1) {
        set_error("mesh too large for the fixed scratch of the allocation-free entry point (needs " +
                  std::to_string(sfs * (long long)sizeof(cd)) + " bytes per frequency, has " +
                  std::to_string(scratch_elems * (long long)sizeof(cd)) + ")");
        return SOD_ERR_CAPACITY;
    }
    const int chunk = (int)std::min<long long>(std::min<long long>(fit, MAX_FREQ_PER_LAUNCH), nfreq);
    int threads = 256;
    const sod_mesh::Coloured *col = nullptr;
    size_t smem = 0;
    if (kind <= SOD_H) {
        // the row block must fit in shared memory (this entry point has no global-memory accumulator):
        // H needs 72 bytes and G 48 bytes of shared memory per vertex
        if (scatter_smem_bytes(kind, 0, m->nV, 32) > ctx->smem_optin) {
            set_error("mesh too large for the allocation-free entry point: the " + std::string(kind == SOD_G ? "G" : "H") +
                      " row block of " + std::to_string(m->nV) + " vertices exceeds the " +
                      std::to_string(ctx->smem_optin) + " bytes of shared memory per CTA");
            return SOD_ERR_CAPACITY;
        }
        std::lock_guard<std::recursive_mutex> lock(m->sched_mu);
        threads = ctx->coll_threads;
        if (threads <= 0) {  // the CTA size the autotuner chose for this kind (any fused variant)
            auto tt = m->tuned.find(kind * 16);
            if (tt == m->tuned.end())
                for (auto &kv : m->tuned)
                    if (kv.first / 16 == kind) {
                        tt = m->tuned.find(kv.first);
                        break;
                    }
            threads = tt != m->tuned.end() ? tt->second : 0;
        }
        auto it = threads > 0 ? m->coloured.find(threads) : m->coloured.end();
        if (it == m->coloured.end()) {
            set_error("the mesh has no scatter schedule yet: assemble it once with sod_cqbem_assemble* during set-up");
            return SOD_ERR_INVALID_ARG;
        }
        col = it->second.get();
        smem = scatter_smem_bytes(kind, 0, m->nV, threads);
        int per_sm = 0;
        SOD_TRY(scatter_occupancy(ctx, kind, 0, false, threads, smem, &per_sm));
        if (per_sm <= 0) {
            set_error("mesh too large for the shared-memory row accumulator");
            return SOD_ERR_UNSUPPORTED;
        }
    }
    const long long per = kind <= SOD_H ? 9LL * m->nV * m->nV : (kind == SOD_B_TRANS ? 9LL : 27LL) * m->nV;
    const size_t esz = out_dtype == SOD_C64 ? 8 : 16;
    for (int f0 = 0; f0 < nfreq; f0 += chunk) {
        const int nf = std::min(chunk, nfreq - f0);
        FreqTable ft;
        ft.n = nf;
        for (int l = 0; l < nf; l++) {
            ft.kd[l] = make_kconst(c1, c2, rho, s[2 * (f0 + l)], s[2 * (f0 + l) + 1]);
            ft.kf[l] = to_float(ft.kd[l]);
        }
        const dim3 grid(m->nV, nf);
        SingArgs sa{};
        sa.nV = m->nV;
        sa.V = m->dV.as<double>();
        sa.F = m->dF.as<int>();
        sa.N = m->dN.as<double>();
        sa.star_off = m->dStarOff.as<int>();
        sa.star_face = m->dStarFace.as<int>();
        sa.star_corner = m->dStarCorner.as<int>();
        sa.star_slot = m->dStarSlot.as<int>();
        sa.nbr_off = m->dNbrOff.as<int>();
        sa.sorder = sorder;
        sa.ssub = ssub;
        sa.S[kind] = scratch;  // every slot is written by the singular pass before it is read
        sa.S_fstride[kind] = sfs;
        switch (kind) {
        case SOD_G: coll_polar_kernel<KM_G><<<grid, 256, 0, stream>>>(sa, ft); break;
        case SOD_B_TRANS: coll_polar_kernel<KM_BT><<<grid, 256, 0, stream>>>(sa, ft); break;
        case SOD_B_ANGULAR: coll_polar_kernel<KM_BA><<<grid, 256, 0, stream>>>(sa, ft); break;
        default: coll_guiggiani_kernel<<<grid, 256, 0, stream>>>(sa, ft); break;
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        CollArgs a{};
        a.err = ctx->dev_err.as<int>();
        a.bar_extra = ctx->wait_test ? 1 : 0;
        a.nV = m->nV;
        a.nF = m->nF;
        a.Vf = m->dVf.as<float>();
        a.canonV = m->has_vmap ? m->dCanon.as<int>() : nullptr;
        a.out_c64 = out_dtype == SOD_C64;
        a.do_regular = 1;
        a.nbr_off = m->dNbrOff.as<int>();
        a.nbr_vert = m->dNbrVert.as<int>();
        a.out[kind] = static_cast<char *>(out) + (size_t)f0 * (size_t)per * esz;
        a.fstride[kind] = per;
        a.S[kind] = scratch;
        a.S_fstride[kind] = sfs;
        if (kind <= SOD_H) {
            a.faces = col->dFaces.as<float4>();
            a.canonF = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
            a.color_off = col->dOff.as<int>();
            a.ncolors = col->ncolors;
            if (kind == SOD_G)
                coll_scatter_kernel<SOD_G, 0><<<grid, threads, smem, stream>>>(a, pt, ft);
            else
                coll_scatter_kernel<SOD_H, 0><<<grid, threads, smem, stream>>>(a, pt, ft);
        } else {
            a.faces = m->dFacesNat.as<float4>();
            a.canonF = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
            if (kind == SOD_B_TRANS)
                coll_reduce_kernel<KM_BT><<<grid, 256, 0, stream>>>(a, pt, ft);
            else
                coll_reduce_kernel<KM_BA><<<grid, 256, 0, stream>>>(a, pt, ft);
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    return SOD_OK;
}

// -------------------------------------------------------------------------------------------
// Batched launches (host): one BatchRegular per persistent launch holds the kernel arguments of up
// to BATCH_OBJS objects (same CTA size, point table and pass) and issues the launch on a stream,
// which may be capturing into a CUDA graph.
struct BatchRegular {
    int which, mask, threads;
    size_t smem;  // dynamic shared memory; for a global-memory launch, the accumulator slice per CTA
    bool global = false;
    int grid = 0;
    DevBuf scratch;  // global-memory accumulators, grid x slice (allocated before graph capture)
    BatchLaunchArgs args;
};

BatchRegular *batch_regular_new(int which, int mask, int threads, size_t smem, const PointTable &pt) {
    auto *r = new BatchRegular();
    r->which = which;
    r->mask = mask;
    r->threads = threads;
    r->smem = smem;
    r->args.pt = pt;
    r->args.nobj = 0;
    return r;
}

template <int KIND, int BM> static const void *batch_global_fn() { return (const void *)batch_scatter_global_kernel<KIND, BM>; }
static const void *batch_global_fn(int kind, int bm) {
    if (kind == SOD_H) return batch_global_fn<SOD_H, 0>();
    switch (bm) {
    case KM_BT: return batch_global_fn<SOD_G, KM_BT>();
    case KM_BA: return batch_global_fn<SOD_G, KM_BA>();
    case KM_BT | KM_BA: return batch_global_fn<SOD_G, KM_BT | KM_BA>();
    default: return batch_global_fn<SOD_G, 0>();
    }
}

// A scatter launch whose row accumulators live in global memory: `slice` bytes per CTA (the largest
// member's row block); the persistent grid and the scratch are sized here, before graph capture.
BatchRegular *batch_regular_new_global(sod_context *ctx, int which, int mask, size_t slice, int nitems_hint,
                                       const PointTable &pt, int *rc) {
    *rc = SOD_OK;
    auto *r = batch_regular_new(which, mask, SCATTER_GLOBAL_THREADS, slice, pt);
    r->global = true;
    const void *fn = batch_global_fn(which == 3 ? SOD_H : SOD_G, which == 3 ? 0 : (mask & (KM_BT | KM_BA)));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SCATTER_GLOBAL_THREADS, 0) != cudaSuccess ||
        per_sm <= 0) {
        set_error("batched global-memory scatter does not fit on an SM");
        *rc = SOD_ERR_CUDA;
        return r;
    }
    r->grid = std::max(1, std::min(per_sm * ctx->num_sms, std::max(nitems_hint, 1)));
    *rc = r->scratch.ensure(slice * (size_t)r->grid);
    return r;
}
void batch_regular_free(BatchRegular *r) { delete r; }

int batch_regular_add(BatchRegular *r, const sod_mesh *m, int out_dtype, void *const out[4], cd *const S[4],
                      const sod_mesh::Coloured *col, int kc_off, int *slot) {
    SOD_REQUIRE(r->args.nobj < BATCH_OBJS, "batched launch is full");
    const long long nslots = m->nbr_off.back();
    const long long sfs[4] = {nslots * 9, nslots * 9, (long long)m->nV * 9, (long long)m->nV * 27};
    const long long per[4] = {9LL * m->nV * m->nV, 9LL * m->nV * m->nV, 9LL * m->nV, 27LL * m->nV};
    CollArgs a{};
    a.err = m->ctx ? m->ctx->dev_err.as<int>() : nullptr;
    a.nV = m->nV;
    a.nF = m->nF;
    a.Vf = m->dVf.as<float>();
    a.canonV = m->has_vmap ? m->dCanon.as<int>() : nullptr;
    a.out_c64 = out_dtype == SOD_C64;
    a.do_regular = 1;
    a.nbr_off = m->dNbrOff.as<int>();
    a.nbr_vert = m->dNbrVert.as<int>();
    for (int kd = 0; kd < 4; kd++) {
        a.out[kd] = (r->mask & (1 << kd)) ? out[kd] : nullptr;
        a.fstride[kd] = per[kd];
        a.S[kd] = (r->mask & (1 << kd)) ? S[kd] : nullptr;
        a.S_fstride[kd] = sfs[kd];
    }
    if (r->which == 4) {
        a.faces = m->dFacesNat.as<float4>();
        a.canonF = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
    } else {
        SOD_REQUIRE(col != nullptr, "scatter launch needs a colouring");
        a.faces = col->dFaces.as<float4>();
        a.canonF = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
        a.color_off = col->dOff.as<int>();
        a.ncolors = col->ncolors;
    }
    const int k = r->args.nobj++;
    r->args.a[k] = a;
    r->args.kc_off[k] = kc_off;
    *slot = k;
    return SOD_OK;
}

// One persistent launch; grid = resident CTAs per SM x SMs.  `which`: 2 G scatter (with the B kinds
// of the mask fused in), 3 H scatter, 4 B reduction (when G is not assembled).
int batch_regular_issue(sod_context *ctx, const BatchRegular *r, const int4 *items, int nitems, int *counter,
                        const KConst<float> *kcf, cudaStream_t stream) {
    if (nitems <= 0) return SOD_OK;
    const int bm = r->mask & (KM_BT | KM_BA);
    const int T = r->threads;
    if (r->global) {
        SOD_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), stream));
        const BatchLaunchArgs &p = r->args;
        float2 *sc = r->scratch.as<float2>();
        const long long per_cta = (long long)(r->smem / sizeof(float2));
        if (r->which == 3)
            batch_scatter_global_kernel<SOD_H, 0><<<r->grid, T, 0, stream>>>(p, items, nitems, counter, kcf, sc, per_cta);
        else if (bm == (KM_BT | KM_BA))
            batch_scatter_global_kernel<SOD_G, KM_BT | KM_BA><<<r->grid, T, 0, stream>>>(p, items, nitems, counter, kcf, sc, per_cta);
        else if (bm == KM_BT)
            batch_scatter_global_kernel<SOD_G, KM_BT><<<r->grid, T, 0, stream>>>(p, items, nitems, counter, kcf, sc, per_cta);
        else if (bm == KM_BA)
            batch_scatter_global_kernel<SOD_G, KM_BA><<<r->grid, T, 0, stream>>>(p, items, nitems, counter, kcf, sc, per_cta);
        else
            batch_scatter_global_kernel<SOD_G, 0><<<r->grid, T, 0, stream>>>(p, items, nitems, counter, kcf, sc, per_cta);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        return SOD_OK;
    }
    const void *fn = r->which == 2   ? scatter_fn(SOD_G, bm, true)
                     : r->which == 3 ? scatter_fn(SOD_H, 0, true)
                     : bm == (KM_BT | KM_BA) ? (const void *)batch_reduce_kernel<KM_BT | KM_BA>
                     : bm == KM_BT           ? (const void *)batch_reduce_kernel<KM_BT>
                                             : (const void *)batch_reduce_kernel<KM_BA>;
    SOD_TRY(prepare_scatter(ctx));
    int per_sm = 1;
    SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, r->smem));
    SOD_REQUIRE(per_sm > 0, "batched launch does not fit on an SM");
    const int grid = std::min(nitems, per_sm * ctx->num_sms);
    SOD_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), stream));
    const BatchLaunchArgs &p = r->args;
    switch (r->which) {
    case 2:
        if (bm == (KM_BT | KM_BA))
            batch_scatter_kernel<SOD_G, KM_BT | KM_BA><<<grid, T, r->smem, stream>>>(p, items, nitems, counter, kcf);
        else if (bm == KM_BT)
            batch_scatter_kernel<SOD_G, KM_BT><<<grid, T, r->smem, stream>>>(p, items, nitems, counter, kcf);
        else if (bm == KM_BA)
            batch_scatter_kernel<SOD_G, KM_BA><<<grid, T, r->smem, stream>>>(p, items, nitems, counter, kcf);
        else
            batch_scatter_kernel<SOD_G, 0><<<grid, T, r->smem, stream>>>(p, items, nitems, counter, kcf);
        break;
    case 3: batch_scatter_kernel<SOD_H, 0><<<grid, T, r->smem, stream>>>(p, items, nitems, counter, kcf); break;
    default:
        if (bm == (KM_BT | KM_BA))
            batch_reduce_kernel<KM_BT | KM_BA><<<grid, T, 0, stream>>>(p, items, nitems, counter, kcf);
        else if (bm == KM_BT)
            batch_reduce_kernel<KM_BT><<<grid, T, 0, stream>>>(p, items, nitems, counter, kcf);
        else
            batch_reduce_kernel<KM_BA><<<grid, T, 0, stream>>>(p, items, nitems, counter, kcf);
        break;
    }
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

}  // namespace sod
