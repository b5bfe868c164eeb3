// sod_galerkin.cu -- Galerkin assembly of the Laplace-domain CQBEM matrices G and H on sm_103a.
//
// Replaces compute_elastodynamic_{G,H}_kernel_galerkin_non_singular
// (src/elastodynamics_cqbem_{G,H}_galerkin_non_singular.cu) and the singular face-pair integrals of
// src/elastodynamics_cqbem_galerkin_singular.cpp (Sauter-Schwab maps, include/integrator_galerkin.hpp:42-212):
//   U_ab = sum over face pairs (f1 containing a, f2 containing b) of
//          int_f1 int_f2 phi_a(x) phi_b(y) K(x, y) dy dx.
//
// Regular pairs (no shared vertex), FP32: one CTA per (test vertex a, frequency) owns row block a in
// shared memory.  It first stages the test quadrature points of the faces around a -- position and
// weight w_x * area * phi_a(x) -- then walks the trial faces in colour order exactly like the
// collocation scatter: each thread integrates one trial face f2 against every staged test face that
// shares no vertex with f2 and adds the three trial-corner blocks without conflicts.  A face pair is
// integrated once per test corner (three times in all) instead of scattering 9 x 9 blocks with
// atomics: the result is deterministic and the row accumulator fits in shared memory.
//
// Singular pairs (coincident, edge- and vertex-adjacent), double-float: one warp per (star entry of
// a, partner face f2, frequency); lanes share the 4-D Gauss points of the Sauter-Schwab maps and
// the warp sums in a fixed xor tree.  An FP64 combine kernel adds the partner blocks into per-
// (vertex, slot) 3 x 3 blocks over the two-ring of a, which the regular kernel's epilogue adds.
#include <algorithm>
#include <array>
#include <map>
#include <set>

#include "sod_bmom.cuh"
#include "sod_dd.cuh"
#include "sod_dd_fast.cuh"
#include "sod_faces.cuh"
#include "sod_internal.h"

using namespace sod;

namespace {

constexpr int GAL_MAXS = 32;  // faces around a vertex
constexpr int GAL_MAXQ = 13;  // points of the test rule (the 13-point rule is the largest)

__device__ __forceinline__ void store_o(void *out, int c64, long long idx, double re, double im) {
    if (c64)
        reinterpret_cast<float2 *>(out)[idx] = make_float2((float)re, (float)im);
    else
        reinterpret_cast<double2 *>(out)[idx] = make_double2(re, im);
}

struct GalArgs {
    int nV, nF;
    const float4 *faces;      // trial faces, colour ordered
    const int *color_off;
    int ncolors;
    const float4 *faces_nat;  // test faces, natural order
    const int *star_off, *star_face, *star_corner;
    void *out;
    long long fstride;
    int out_c64, do_regular;
    const cd *S;  // singular blocks per (frequency, slot)
    long long S_fstride;
    const int *slot_off, *slot_vert;
    void *outB[2];  // B_trans [3V][3], B_angular [3V][9] (null if not requested)
    long long fstrideB[2];
    const cd *SB[2];  // singular B per (frequency, vertex): 9 / 27 values
    long long SB_fstride[2];
};

// B_trans / B_angular rows of test vertex i from the CTA's component sums (FP64) + singular parts
template <int BM>
__device__ __forceinline__ void gal_store_b(const GalArgs &a, const cd *bsum, int i, int fq) {
    using M = BMom<BM>;
    if (M::BT && a.outB[0]) {
        const long long base = (long long)fq * a.fstrideB[0] + (long long)(3 * i) * 3;
        for (int e = threadIdx.x; e < 9; e += blockDim.x) {
            cd v = bsum[sym_index(e / 3, e % 3)];
            if (a.SB[0]) v = v + a.SB[0][(long long)fq * a.SB_fstride[0] + (long long)i * 9 + e];
            store_o(a.outB[0], a.out_c64, base + e, v.x, v.y);
        }
    }
    if (M::BA && a.outB[1]) {
        const long long base = (long long)fq * a.fstrideB[1] + (long long)(3 * i) * 9;
        for (int e = threadIdx.x; e < 27; e += blockDim.x) {
            const int p = e / 9, qq = (e / 3) % 3, kk = e % 3;
            cd v = bsum[M::NT + 3 * sym_index(p, qq) + kk];
            if (a.SB[1]) v = v + a.SB[1][(long long)fq * a.SB_fstride[1] + (long long)i * 27 + e];
            store_o(a.outB[1], a.out_c64, base + e, v.x, v.y);
        }
    }
}

// Regular pairs, pass 1: one CTA per (test point x, frequency).  Test point t = f1 * nq + ix is point
// ix of the test rule on test face f1.  The CTA integrates every trial face f2 that shares no vertex
// with f1 -- the collocation scatter with x as the field point -- into the unweighted row
//     R(x)[c][b] = sum_f2 int_f2 K_c(x, y) phi_b(y) dy      (c: tensor component, b: trial vertex)
// in shared memory (colour order, conflict-free, deterministic) and stores it to scratch, with the
// B_trans / B_angular sums of x when BM != 0.  Each kernel evaluation is done once per point pair.
struct GalTpArgs {
    int nV, nq, t0;            // vertices, test points per face, first test point of this launch
    const float4 *faces;       // trial faces, colour ordered
    const int *color_off;
    int ncolors;
    const float4 *faces_nat;   // test faces, natural order
    const int4 *canon_faces;   // canonical corner ids of the trial faces (colour order), NULL without splitting
    const int4 *canon_nat;     // canonical corner ids of the test faces (natural order)
    float2 *rows;              // [fq][t - t0][NC][nV]
    long long rows_fstride;
    cd *bsum;                  // [fq][t - t0][NCB] (BM != 0)
    long long b_fstride;
};

template <int KIND, int BM> constexpr int gal_max_threads() { return 512; }

// GLOBAL: the row block does not fit in shared memory, so the CTA accumulates directly in its
// output row (global memory, exclusive to the CTA; the colour barriers order its accesses) and
// keeps only the B columns in shared memory.
template <int KIND, int BM, bool GLOBAL = false>
__global__ void __launch_bounds__(gal_max_threads<KIND, BM>(), 1) gal_tp_kernel(GalTpArgs a, PointTable pt,
                                                                                const __grid_constant__ FreqTable ft) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;
    using BMo = BMom<KIND == SOD_G ? BM : 0>;
    constexpr int NCB = BMo::NC;
    extern __shared__ float2 smem_tp[];  // [NC][nV] (unless GLOBAL), then [NCB][blockDim]
    const int tl = blockIdx.x, t = a.t0 + tl, fq = blockIdx.y, nV = a.nV;
    float2 *dst = a.rows + (long long)fq * a.rows_fstride + (long long)tl * NC * nV;
    float2 *acc = GLOBAL ? dst : smem_tp;
    const KConst<float> k = ft.kf[fq];
    const int f1 = t / a.nq, ix = t - f1 * a.nq;
    const FaceRec tf = load_face(a.faces_nat, f1);
    const float4 PX = pt.p[ix];
    const float3 x = make_float3(PX.x * tf.y1.x + PX.y * tf.y2.x + PX.z * tf.y3.x,
                                 PX.x * tf.y1.y + PX.y * tf.y2.y + PX.z * tf.y3.y,
                                 PX.x * tf.y1.z + PX.y * tf.y2.z + PX.z * tf.y3.z);
    for (int e = threadIdx.x; e < NC * nV; e += blockDim.x) acc[e] = make_float2(0.f, 0.f);
    float2 *accB = GLOBAL ? smem_tp : acc + NC * nV;
#pragma unroll
    for (int c = 0; c < NCB; c++) accB[c * blockDim.x + threadIdx.x] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int c = 0; c < a.ncolors; c++) {
        const int fend = a.color_off[c + 1];
        for (int f = a.color_off[c] + threadIdx.x; f < fend; f += blockDim.x) {
            const FaceRec fr = load_face(a.faces, f);
            int p0 = fr.j0, p1 = fr.j1, p2 = fr.j2, q0 = tf.j0, q1 = tf.j1, q2 = tf.j2;
            if (a.canon_faces) {  // traction-discontinuity splitting: pairs touch through canonical ids
                const int4 cp = __ldg(a.canon_faces + f), cq = __ldg(a.canon_nat + f1);
                p0 = cp.x, p1 = cp.y, p2 = cp.z, q0 = cq.x, q1 = cq.y, q2 = cq.z;
            }
            const bool touch = p0 == q0 || p0 == q1 || p0 == q2 || p1 == q0 || p1 == q1 || p1 == q2 || p2 == q0 ||
                               p2 == q1 || p2 == q2;
            if (touch) continue;  // singular pair (coincident, edge- or vertex-adjacent)
            const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
            // corners relative to the test point: y - x = sum_l P_l (y_l - x)
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
                const RadialTerms<float, cf> rt = radial<(NCB > 0)>(r, rinv, k);
                // the collocation scatter's tensor build: per-row vectors, the common factor
                // (1/(4 pi rho r) for G, 1/(4 pi r^2) for H) in the weight
                cf u[NC];
                float sc;
                if (KIND == SOD_G) {
                    cf al, be;
                    g_coeffs_unit(rt, k, al, be);
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
                    h_coeffs_unit(rt, k, ha, hb, hd);
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
                if (NCB) bm.add(rt, k, r, rh, nn, P.w);
            }
            const int jj[3] = {fr.j0, fr.j1, fr.j2};
#pragma unroll
            for (int kk = 0; kk < 3; kk++)
#pragma unroll
                for (int cc = 0; cc < NC; cc++) {
                    float2 &sacc = acc[cc * nV + jj[kk]];
                    sacc.x += part[kk][cc].x;
                    sacc.y += part[kk][cc].y;
                }
            if (NCB) {
                float2 *col = accB + threadIdx.x;
                bm.emit(k, nn, fr.area, [&](int cc, cf v) {
                    float2 &sb = col[cc * blockDim.x];
                    sb.x += v.x;
                    sb.y += v.y;
                });
            }
        }
        __syncthreads();
    }
    // the row, unweighted, to scratch (coalesced; a GLOBAL CTA accumulated in place)
    if (!GLOBAL)
        for (int e = threadIdx.x; e < NC * nV; e += blockDim.x) dst[e] = acc[e];
    if (NCB) {
        // per-thread B columns -> double-float sums on the FP32 pipes (FP64 is ~1/64 of the FP32 rate
        // on GB300), 32 lanes per component in a fixed xor tree
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
            if (l == 0) a.bsum[(long long)fq * a.b_fstride + (long long)tl * NCB + cc] = mk(dd_to(sx), dd_to(sy));
        }
    }
}

// Regular pairs, pass 2: one CTA per (test vertex a, frequency) combines the rows of the test points
// on the faces around a, U[a] = sum_x phi_a(x) w_x area(f1) R(x), in fixed order (star face, then
// test point) with compensated FP32 sums (TwoSum, error ~ 1 ulp of the result: FP64 arithmetic runs
// at a small fraction of the FP32 rate here), and adds the singular blocks of a's two-ring slots
// (FP64) and the singular B parts.
struct Comp2 {  // compensated FP32 complex sum
    float sx = 0.f, cx = 0.f, sy = 0.f, cy = 0.f;
    __device__ __forceinline__ static void add1(float &s, float &c, float p) {
        // _rn operations: the product w v must not be contracted into the TwoSum's adds
        const float t = __fadd_rn(s, p), bp = __fsub_rn(t, s);
        c += __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
        s = t;
    }
    __device__ __forceinline__ void add(float w, float2 v) {
        add1(sx, cx, w * v.x);
        add1(sy, cy, w * v.y);
    }
    __device__ __forceinline__ cd value() const { return mk((double)sx + (double)cx, (double)sy + (double)cy); }
};
struct GalGatherArgs {
    GalArgs g;                 // outputs, singular blocks and slots
    int nq, do_regular;
    const float2 *rows;        // [fq][t][NC][nV] (all test points of the mesh)
    long long rows_fstride;
    const cd *bsum;            // [fq][t][NCB]
    long long b_fstride;
};

template <int KIND, int BM>
__global__ void __launch_bounds__(256) gal_gather_kernel(GalGatherArgs ga, PointTable pt) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;
    using BMo = BMom<KIND == SOD_G ? BM : 0>;
    constexpr int NCB = BMo::NC;
    const GalArgs &a = ga.g;
    __shared__ float wt[GAL_MAXS * GAL_MAXQ];
    __shared__ int tt[GAL_MAXS * GAL_MAXQ];
    __shared__ cd bs[24];
    const int i = blockIdx.x, fq = blockIdx.y, nV = a.nV, nq = ga.nq;
    const int s0 = a.star_off[i], ns = min(a.star_off[i + 1] - s0, GAL_MAXS);
    const int np = ns * nq;
    for (int e = threadIdx.x; e < np; e += blockDim.x) {
        const int s = e / nq, q = e - s * nq;
        const int f1 = a.star_face[s0 + s], sc = a.star_corner[s0 + s];
        const FaceRec fr = load_face(a.faces_nat, f1);
        const float4 P = pt.p[q];
        const float L = sc == 0 ? P.x : sc == 1 ? P.y : P.z;
        wt[e] = P.w * fr.area * L;
        tt[e] = f1 * nq + q;
    }
    __syncthreads();
    const float2 *R = ga.rows + (long long)fq * ga.rows_fstride;
    auto row_sum = [&](int c, int j) {
        Comp2 acc;
        if (ga.do_regular)
#pragma unroll 4
            for (int e = 0; e < np; e++) acc.add(wt[e], __ldg(R + ((long long)tt[e] * NC + c) * nV + j));
        return acc.value();
    };
    const long long ld = 3LL * nV;
    const long long base = (long long)fq * a.fstride + (long long)(3 * i) * ld;
    if (a.out) {
        // one thread per (component, trial vertex): coalesced reads of the rows
        for (int e = threadIdx.x; e < NC * nV; e += blockDim.x) {
            const int c = e / nV, j = e - c * nV;
            const cd v = row_sum(c, j);
            if (KIND == SOD_G) {
                const int p = c < 3 ? 0 : (c < 5 ? 1 : 2), qq = c < 3 ? c : (c < 5 ? c - 2 : 2);
                store_o(a.out, a.out_c64, base + p * ld + 3 * j + qq, v.x, v.y);
                if (p != qq) store_o(a.out, a.out_c64, base + qq * ld + 3 * j + p, v.x, v.y);
            } else {
                store_o(a.out, a.out_c64, base + (c / 3) * ld + 3 * j + c % 3, v.x, v.y);
            }
        }
        if (a.S) {
            __syncthreads();
            const int b0 = a.slot_off[i], nb = a.slot_off[i + 1] - b0;
            for (int e = threadIdx.x; e < nb * 9; e += blockDim.x) {
                const int sl = b0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
                const int j = a.slot_vert[sl];
                const cd v = row_sum(KIND == SOD_G ? sym_index(p, qq) : pq, j);
                const cd sv = a.S[(long long)fq * a.S_fstride + (long long)sl * 9 + pq];
                store_o(a.out, a.out_c64, base + p * ld + 3 * j + qq, v.x + sv.x, v.y + sv.y);
            }
        }
    }
    if (NCB) {
        for (int c = threadIdx.x; c < NCB; c += blockDim.x) {
            double sx = 0.0, sy = 0.0;  // FP64: 24 components per vertex, negligible
            if (ga.do_regular)
                for (int e = 0; e < np; e++) {
                    const cd v = ga.bsum[(long long)fq * ga.b_fstride + (long long)tt[e] * NCB + c];
                    sx = fma((double)wt[e], v.x, sx);
                    sy = fma((double)wt[e], v.y, sy);
                }
            bs[c] = mk(sx, sy);
        }
        __syncthreads();
        gal_store_b<BM>(a, bs, i, fq);
    }
}

// ---- singular pairs in double-float ------------------------------------------------------------
struct KDDg {
    cdd sc1, sc2, is;
    dd ic1, ic2, ic1s, ic2s, six_c2s, inv4pirho, inv4pi, k4m1, k2, k1m2, k12;
};
__device__ __forceinline__ KDDg make_kddg(const KConst<double> &k) {
    KDDg o;
    o.sc1 = cdd{dd_from(k.sc1r), dd_from(k.sc1i)};
    o.sc2 = cdd{dd_from(k.sc2r), dd_from(k.sc2i)};
    o.is = cdd{dd_from(k.isr), dd_from(k.isi)};
    o.ic1 = dd_from(k.ic1), o.ic2 = dd_from(k.ic2);
    o.ic1s = dd_from(k.ic1s), o.ic2s = dd_from(k.ic2s), o.six_c2s = dd_from(k.six_c2s);
    o.inv4pirho = dd_from(k.inv4pirho), o.inv4pi = dd_from(k.inv4pi);
    o.k4m1 = dd_from(4.0 * k.kappa - 1.0), o.k2 = dd_from(2.0 * k.kappa), o.k1m2 = dd_from(1.0 - 2.0 * k.kappa);
    o.k12 = dd_from(12.0 * k.kappa);
    return o;
}

struct DuffyRule {  // 1-D Gauss-Legendre on [0,1] after subdivision, FP64
    int n;
    double x[40], w[40];
};

struct GalSingArgs {
    int nent, npairs;
    const int4 *pairs;  // per pair: {f2, class}, {j1[3]}, {j2[3]}, {entry of test corner 0, 1, 2}
    const double *V, *N;
    double2 *R;         // [frequency][entry][3 * NCS]
    double2 *RB;        // [frequency][entry][13] B moments (G pass with B kinds)
};
constexpr int GAL_BMOM = 13;  // Ms[3], Md, M1[6], M0, SB, SC

__device__ __forceinline__ dd ddv(double x) { return dd_from(x); }

// shared-memory floats per warp of the singular kernel: kernel tensor (NCS cdd), B moment values
// (13 cdd, G pass with B kinds), the test shape functions (3 dd) and the test x trial shape-function
// products (9 dd) of 32 points
template <int KIND, int BM> constexpr int sing_warp_floats() {
    return 32 * ((KIND == SOD_G ? 6 : 9) * 4 + ((KIND == SOD_G && BM != 0) ? GAL_BMOM * 4 : 0) + 24);
}
__device__ __forceinline__ void st_cdd(float *p, const cdd &v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo);
}
__device__ __forceinline__ cdd ld_cdd(const float *p) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    return cdd{dd{q.x, q.y}, dd{q.z, q.w}};
}

// One warp per (distinct singular face pair, frequency).  The three entries of a pair (test corners
// of f1) share every kernel evaluation, so the warp integrates the pair once: in batches of 32
// Sauter-Schwab points, each lane first evaluates the kernel tensor (times the point weight) at one
// point into shared memory, then each lane adds the 32 points into the few (test corner, trial
// corner, component) sums it owns, in point order -- every sum is owned by one lane, so no cross-lane
// reduction is needed and the order is fixed.
template <int KIND, int BM>
__global__ void __launch_bounds__(128) gal_sing_kernel(GalSingArgs a, const __grid_constant__ DuffyRule g,
                                                       const __grid_constant__ FreqTable ft) {
    constexpr int NCS = KIND == SOD_G ? 6 : 9;
    constexpr bool DB = KIND == SOD_G && BM != 0;
    constexpr bool BT = (BM & (1 << SOD_B_TRANS)) != 0, BA = (BM & (1 << SOD_B_ANGULAR)) != 0;
    constexpr int NA = 9 * NCS + (DB ? 3 * GAL_BMOM : 0), PER = (NA + 31) / 32;
    constexpr int OFF_V = 32 * NCS * 4, OFF_L = OFF_V + (DB ? 32 * GAL_BMOM * 4 : 0);
    extern __shared__ float smem_sing[];
    __shared__ DdTabs tb;  // exp / sin-cos tables: the lanes' points index them differently
    dd_tabs_load(&tb);
    __syncthreads();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= a.npairs) return;
    float *sw = smem_sing + (threadIdx.x >> 5) * sing_warp_floats<KIND, BM>();
    const int fq = blockIdx.y;
    const KDDg k = make_kddg(ft.kd[fq]);
    const int4 e0 = a.pairs[4 * warp], ej1 = a.pairs[4 * warp + 1], ej2 = a.pairs[4 * warp + 2],
               ee = a.pairs[4 * warp + 3];
    const int f2 = e0.x, cls = e0.y;
    const int j1[3] = {ej1.x, ej1.y, ej1.z}, j2[3] = {ej2.x, ej2.y, ej2.z}, ent[3] = {ee.x, ee.y, ee.z};
    // parametrisation x = o + xa xh0 + xb xh1, y = o + ya yh0 + yb yh1 (FP64 set-up)
    double P1[3][3], P2[3][3];
    for (int c = 0; c < 3; c++)
        for (int d = 0; d < 3; d++) P1[c][d] = a.V[3 * j1[c] + d], P2[c][d] = a.V[3 * j2[c] + d];
    double xa[3], xb[3], ya[3], yb[3];
    for (int d = 0; d < 3; d++) {
        if (cls == 1) {
            xa[d] = ya[d] = P1[1][d] - P1[0][d];
            xb[d] = yb[d] = P1[2][d] - P1[1][d];
        } else if (cls == 2) {
            xa[d] = ya[d] = P1[1][d] - P1[0][d];
            xb[d] = P1[2][d] - P1[1][d];
            yb[d] = P2[2][d] - P1[1][d];
        } else {
            xa[d] = P1[1][d] - P1[0][d];
            xb[d] = P1[2][d] - P1[1][d];
            ya[d] = P2[1][d] - P1[0][d];
            yb[d] = P2[2][d] - P2[1][d];
        }
    }
    auto crossn = [](const double *u, const double *v) {
        const double c0 = u[1] * v[2] - u[2] * v[1], c1 = u[2] * v[0] - u[0] * v[2], c2 = u[0] * v[1] - u[1] * v[0];
        return sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    };
    const double J = crossn(xa, xb) * crossn(ya, yb);
    const dd Xa[3] = {ddv(xa[0]), ddv(xa[1]), ddv(xa[2])}, Xb[3] = {ddv(xb[0]), ddv(xb[1]), ddv(xb[2])};
    const dd Ya[3] = {ddv(ya[0]), ddv(ya[1]), ddv(ya[2])}, Yb[3] = {ddv(yb[0]), ddv(yb[1]), ddv(yb[2])};
    const dd nn[3] = {ddv(a.N[3 * f2]), ddv(a.N[3 * f2 + 1]), ddv(a.N[3 * f2 + 2])};
    cdd acc[PER];
#pragma unroll
    for (int t = 0; t < PER; t++) acc[t] = cdd{dd{0.f, 0.f}, dd{0.f, 0.f}};
    const int n = g.n, n4 = n * n * n * n;
    const int nmap = cls == 1 ? 6 : cls == 2 ? 5 : 2;
    const int total = n4 * nmap;
    const dd zero = dd{0.f, 0.f};
    for (int base = 0; base < total; base += 32) {
        // ---- phase A: this lane's point -> kernel tensor, B moment values and shape functions ----
        const int pidx = base + lane;
        cdd u[NCS];
        cdd mv[DB ? GAL_BMOM : 1];
        dd Lx[3] = {zero, zero, zero}, Ly[3] = {zero, zero, zero};
#pragma unroll
        for (int c = 0; c < NCS; c++) u[c] = cdd{zero, zero};
#pragma unroll
        for (int c = 0; c < (DB ? GAL_BMOM : 1); c++) mv[c] = cdd{zero, zero};
        if (pidx < total) {
            const int m = pidx / n4, r4 = pidx % n4;
            const int i1 = r4 / (n * n * n), i2 = (r4 / (n * n)) % n, i3 = (r4 / n) % n, i4 = r4 % n;
            const dd e1 = ddv(g.x[i1]), e2 = ddv(g.x[i2]), e3 = ddv(g.x[i3]), xi = ddv(g.x[i4]);
            const dd one = dd{1.f, 0.f};
            dd w = ddv(g.w[i1] * g.w[i2] * g.w[i3] * g.w[i4]) * (xi * xi * xi);
            dd xh0, xh1, yh0, yh1;
            const dd e12 = e1 * e2, e123 = e12 * e3;
            if (cls == 1) {  // coincident, 6 maps; jac = w xi^3 e1^2 e2
                w = w * (e1 * e1) * e2;
                switch (m) {
                case 0: xh0 = xi, xh1 = xi * (one - e1 + e12), yh0 = xi * (one - e123), yh1 = xi * (one - e1); break;
                case 1: xh0 = xi * (one - e123), xh1 = xi * (one - e1), yh0 = xi, yh1 = xi * (one - e1 + e12); break;
                case 2: xh0 = xi, xh1 = xi * e1 * (one - e2 + e2 * e3), yh0 = xi * (one - e12), yh1 = xi * e1 * (one - e2); break;
                case 3: xh0 = xi * (one - e12), xh1 = xi * e1 * (one - e2), yh0 = xi, yh1 = xi * e1 * (one - e2 + e2 * e3); break;
                case 4: xh0 = xi * (one - e123), xh1 = xi * e1 * (one - e2 * e3), yh0 = xi, yh1 = xi * e1 * (one - e2); break;
                default: xh0 = xi, xh1 = xi * e1 * (one - e2), yh0 = xi * (one - e123), yh1 = xi * e1 * (one - e2 * e3); break;
                }
            } else if (cls == 2) {  // edge adjacent, 5 maps; jac = w xi^3 e1^2 (times e2 for maps 2..5)
                w = w * (e1 * e1);
                switch (m) {
                case 0: xh0 = xi, xh1 = xi * e1 * e3, yh0 = xi * (one - e12), yh1 = xi * e1 * (one - e2); break;
                case 1: xh0 = xi, xh1 = xi * e1, yh0 = xi * (one - e123), yh1 = xi * e12 * (one - e3), w = w * e2; break;
                case 2: xh0 = xi * (one - e12), xh1 = xi * e1 * (one - e2), yh0 = xi, yh1 = xi * e123, w = w * e2; break;
                case 3: xh0 = xi * (one - e123), xh1 = xi * e12 * (one - e3), yh0 = xi, yh1 = xi * e1, w = w * e2; break;
                default: xh0 = xi * (one - e123), xh1 = xi * e1 * (one - e2 * e3), yh0 = xi, yh1 = xi * e12, w = w * e2; break;
                }
            } else {  // vertex adjacent, 2 maps; jac = w xi^3 e2
                w = w * e2;
                if (m == 0) xh0 = xi, xh1 = xi * e1, yh0 = xi * e2, yh1 = xi * e2 * e3;
                else xh0 = xi * e2, xh1 = xi * e2 * e3, yh0 = xi, yh1 = xi * e1;
            }
            // y - x = ya yh0 + yb yh1 - xa xh0 - xb xh1 (the common origin cancels exactly)
            dd rv[3];
#pragma unroll
            for (int d = 0; d < 3; d++) rv[d] = Ya[d] * yh0 + Yb[d] * yh1 - Xa[d] * xh0 - Xb[d] * xh1;
            const dd r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
            const dd r = dd_sqrt(r2);
            const dd rinv = dd_recip(r);
            const dd rh[3] = {rv[0] * rinv, rv[1] * rinv, rv[2] * rinv};
            Lx[0] = one - xh0, Lx[1] = xh0 - xh1, Lx[2] = xh1;
            Ly[0] = one - yh0, Ly[1] = yh0 - yh1, Ly[2] = yh1;
            // radial terms
            const cdd z1 = k.sc1 * r, z2 = k.sc2 * r;
            const cdd ez1 = cdd_exp_neg_tab(z1, &tb), ez2 = cdd_exp_neg_tab(z2, &tb);
            const cdd psi1 = cdd_psi(z1, ez1), psi2 = cdd_psi(z2, ez2);
            const cdd Y = psi1 * k.ic1s - psi2 * k.ic2s;
            if (KIND == SOD_G) {
                const cdd B = ez1 * k.ic1s - ez2 * k.ic2s;
                const dd sc = k.inv4pirho * rinv * w;
                const cdd al = (Y * 3.0f + B) * sc, be = (ez2 * k.ic2s - Y) * sc;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int qq = p; qq < 3; qq++) {
                        cdd v = al * (rh[p] * rh[qq]);
                        if (p == qq) v = v + be;
                        u[sym_index(p, qq)] = v;
                    }
            } else {
                const cdd Yc = Y * k.six_c2s;
                const cdd z1e1 = z1 * ez1, z2e2 = z2 * ez2;
                const dd sc = k.inv4pi * (rinv * rinv) * w;
                const cdd ca = (Yc + ez1 * k.k4m1 - ez2 * 2.0f - z1e1 * k.k1m2) * sc;
                const cdd cb = (Yc + ez1 * k.k2 - ez2 * 3.0f - z2e2) * sc;
                const cdd cdv = (Yc * (-5.0f) - ez1 * k.k12 + ez2 * 12.0f - z1e1 * k.k2 + z2e2 * 2.0f) * sc;
                const dd rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                const cdd cbr = cb * rn, cdr = cdv * rn;
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int qq = 0; qq < 3; qq++) {
                        cdd v = ca * (rh[p] * nn[qq]) + cb * (nn[p] * rh[qq]) + cdr * (rh[p] * rh[qq]);
                        if (p == qq) v = v + cbr;
                        u[3 * p + qq] = v;
                    }
            }
            if (DB) {  // B moment values with the point weight (the test corner weight comes later)
                const dd rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                if (BT) {
                    const cdd ws = Y * (k.inv4pi * 0.5f);
                    const cdd di = psi2 * (k.ic2s * k.inv4pi);
#pragma unroll
                    for (int p = 0; p < 3; p++) mv[p] = ws * (w * rh[p]);
                    mv[3] = di * (w * rn);
                }
                if (BA) {
                    const cdd A = Y * (r * k.inv4pi * 0.5f);
                    const cdd Bq = (ez2 * k.ic2 - ez1 * k.ic1) * k.is * (k.inv4pi * 0.5f);
                    const cdd Cq = ez2 * k.is * (k.ic2 * k.inv4pi);
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int q = p; q < 3; q++) mv[4 + sym_index(p, q)] = A * (w * (rh[p] * rh[q]));
                    mv[10] = A * w;
                    mv[11] = Bq * w;
                    mv[12] = Cq * w;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < NCS; c++) st_cdd(sw + (lane * NCS + c) * 4, u[c]);
        if (DB)
#pragma unroll
            for (int c = 0; c < GAL_BMOM; c++) st_cdd(sw + OFF_V + (lane * GAL_BMOM + c) * 4, mv[c]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            sw[OFF_L + lane * 24 + 2 * c] = Lx[c].hi, sw[OFF_L + lane * 24 + 2 * c + 1] = Lx[c].lo;
#pragma unroll
            for (int b = 0; b < 3; b++) {  // the weights of the 9 (test corner, trial corner) sums
                const dd wab = Lx[c] * Ly[b];
                sw[OFF_L + lane * 24 + 6 + 2 * (3 * c + b)] = wab.hi;
                sw[OFF_L + lane * 24 + 6 + 2 * (3 * c + b) + 1] = wab.lo;
            }
        }
        __syncwarp();
        // ---- phase B: the sums this lane owns, over the batch's 32 points in order ----
#pragma unroll
        for (int t = 0; t < PER; t++) {
            const int q = lane + 32 * t;
            if (q >= NA) continue;
            if (q < 9 * NCS) {
                const int ac = q / (3 * NCS), b = (q / NCS) % 3, c = q % NCS;
                for (int pt = 0; pt < 32; pt++) {
                    const float *L = sw + OFF_L + pt * 24 + 6 + 2 * (3 * ac + b);
                    cs_fma_acc(acc[t], ld_cdd(sw + (pt * NCS + c) * 4), dd{L[0], L[1]});
                }
            } else if (DB) {
                const int qm = q - 9 * NCS, ac = qm / GAL_BMOM, c = qm % GAL_BMOM;
                for (int pt = 0; pt < 32; pt++) {
                    const float *L = sw + OFF_L + pt * 24;
                    cs_fma_acc(acc[t], ld_cdd(sw + OFF_V + (pt * GAL_BMOM + c) * 4), dd{L[2 * ac], L[2 * ac + 1]});
                }
            }
        }
        __syncwarp();
    }
    // each sum belongs to one lane: scale by the map Jacobian and store per entry
#pragma unroll
    for (int t = 0; t < PER; t++) {
        const int q = lane + 32 * t;
        if (q >= NA) continue;
        const double2 v = make_double2(dd_to(acc[t].x) * J, dd_to(acc[t].y) * J);
        if (q < 9 * NCS) {
            const int ac = q / (3 * NCS), bc = q % (3 * NCS);
            a.R[((size_t)fq * a.nent + ent[ac]) * 3 * NCS + bc] = v;
        } else if (DB) {
            const int qm = q - 9 * NCS, ac = qm / GAL_BMOM, c = qm % GAL_BMOM;
            a.RB[((size_t)fq * a.nent + ent[ac]) * GAL_BMOM + c] = v;
        }
    }
}

// singular B of vertex i: sum over its partner entries of the face tensors formed from the moments
// with the partner face's normal (FP64, fixed order); one warp per (i, frequency)
template <int BM>
__global__ void __launch_bounds__(128) gal_combine_b_kernel(int nV, int nent, const int *__restrict__ ent_off,
                                                            const int4 *__restrict__ ent, const double *__restrict__ N,
                                                            const double2 *__restrict__ RB, cd *__restrict__ SBt,
                                                            cd *__restrict__ SBa, int nf) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nV * nf) return;
    const int fq = w / nV, i = w % nV;
    const int e0 = ent_off[i], e1 = ent_off[i + 1];
    const bool bt = (BM & (1 << SOD_B_TRANS)) != 0, ba = (BM & (1 << SOD_B_ANGULAR)) != 0;
    for (int el = lane; el < 36; el += 32) {
        const bool isT = el < 9;
        if ((isT && !bt) || (!isT && !ba)) continue;
        double sx = 0.0, sy = 0.0;
        for (int e = e0; e < e1; e++) {
            const int f2 = ent[4 * e].x;
            const double nv[3] = {N[3 * f2], N[3 * f2 + 1], N[3 * f2 + 2]};
            const double2 *m = RB + ((size_t)fq * nent + e) * GAL_BMOM;
            if (isT) {
                const int p = el / 3, q = el % 3;
                sx += m[p].x * nv[q] + m[q].x * nv[p] + (p == q ? m[3].x : 0.0);
                sy += m[p].y * nv[q] + m[q].y * nv[p] + (p == q ? m[3].y : 0.0);
            } else {
                const int e27 = el - 9, p = e27 / 9, q = (e27 / 3) % 3, kk = e27 % 3;
                const double2 mpk = m[4 + sym_index(p, kk)], mqk = m[4 + sym_index(q, kk)];
                const double t2 = (q == kk ? nv[p] : 0.0) + (p == kk ? nv[q] : 0.0);
                sx += mpk.x * nv[q] + mqk.x * nv[p] + (m[10].x + m[11].x) * t2 + (p == q ? m[12].x * nv[kk] : 0.0);
                sy += mpk.y * nv[q] + mqk.y * nv[p] + (m[10].y + m[11].y) * t2 + (p == q ? m[12].y * nv[kk] : 0.0);
            }
        }
        if (isT)
            SBt[(size_t)fq * nV * 9 + (size_t)i * 9 + el] = cd{sx, sy};
        else
            SBa[(size_t)fq * nV * 27 + (size_t)i * 27 + (el - 9)] = cd{sx, sy};
    }
}

// S[fq][slot][9] = sum of the partner blocks of vertex i (FP64, fixed order); one warp per (i, fq)
template <int KIND>
__global__ void __launch_bounds__(128) gal_combine_kernel(int nV, int nent, const int *__restrict__ ent_off,
                                                          const int4 *__restrict__ ent, const int *__restrict__ slot_off,
                                                          const double2 *__restrict__ R, cd *__restrict__ S,
                                                          long long S_fstride, int nf) {
    constexpr int NCS = KIND == SOD_G ? 6 : 9;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nV * nf) return;
    const int fq = w / nV, i = w % nV;
    const int b0 = slot_off[i], nb = slot_off[i + 1] - b0;
    const int e0 = ent_off[i], e1 = ent_off[i + 1];
    for (int el = lane; el < nb * 9; el += 32) {
        const int sl = b0 + el / 9, pq = el % 9, p = pq / 3, q = pq % 3;
        const int comp = KIND == SOD_G ? sym_index(p, q) : pq;
        double sx = 0.0, sy = 0.0;
        for (int e = e0; e < e1; e++) {
            const int4 s = ent[4 * e + 3];
            const int sls[3] = {s.x, s.y, s.z};
            for (int b = 0; b < 3; b++)
                if (sls[b] == sl) {
                    const double2 v = R[((size_t)fq * nent + e) * 3 * NCS + b * NCS + comp];
                    sx += v.x, sy += v.y;
                }
        }
        S[(size_t)fq * S_fstride + (size_t)sl * 9 + pq] = cd{sx, sy};
    }
}

// pair classification (the singular-pair structure of include/integrator_galerkin.hpp:262-334):
// 1 coincident, 2 edge adjacent, 3 vertex adjacent, 0 regular; permuted vertex lists j1, j2
// With traction-discontinuity splitting (vmap, may be NULL) vertices match when their canonical ids do
// (:290-291, :314); j1, j2 keep the faces' own vertex ids.
int classify(const int *F, const int *vmap, int f1, int f2, int j1[3], int j2[3]) {
    auto fv = [&](int f, int k) { return F[3 * f + k]; };
    auto cv = [&](int f, int k) { return vmap ? vmap[F[3 * f + k]] : F[3 * f + k]; };
    if (f1 == f2) {
        for (int k = 0; k < 3; k++) j1[k] = j2[k] = fv(f1, k);
        return 1;
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (cv(f1, i) == cv(f2, j) && cv(f1, (i + 1) % 3) == cv(f2, (j + 2) % 3)) {
                j1[0] = fv(f1, i), j1[1] = fv(f1, (i + 1) % 3), j1[2] = fv(f1, (i + 2) % 3);
                j2[0] = fv(f2, j), j2[1] = fv(f2, (j + 2) % 3), j2[2] = fv(f2, (j + 1) % 3);
                return 2;
            }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (cv(f1, i) == cv(f2, j)) {
                j1[0] = fv(f1, i), j1[1] = fv(f1, (i + 1) % 3), j1[2] = fv(f1, (i + 2) % 3);
                j2[0] = fv(f2, j), j2[1] = fv(f2, (j + 1) % 3), j2[2] = fv(f2, (j + 2) % 3);
                return 3;
            }
    return 0;
}

}  // namespace

// ---- per-mesh Galerkin structures (built once, kept on the mesh) ----------------------------------
static int build_gal(const sod_mesh *m, sod_mesh::GalData *g) {
    const int nV = m->nV, nF = m->nF;
    const int *vm = m->has_vmap ? m->vmap.data() : nullptr;
    auto canon = [&](int v) { return vm ? vm[v] : v; };
    std::vector<std::vector<int>> vf(nV), vfc(nV);  // faces of each vertex; of each canonical vertex
    for (int f = 0; f < nF; f++)
        for (int c = 0; c < 3; c++) {
            vf[m->F[3 * f + c]].push_back(f);
            auto &l = vfc[canon(m->F[3 * f + c])];
            if (l.empty() || l.back() != f) l.push_back(f);
        }
    // actual-vertex stars (face order; corner = first corner holding the vertex)
    {
        std::vector<int> so(nV + 1, 0), sf, sc;
        g->max_astar = 0;
        for (int v = 0; v < nV; v++) {
            for (int f : vf[v]) {
                if (!sf.empty() && so[v] < (int)sf.size() && sf.back() == f) continue;  // v twice in f
                int c = 0;
                while (m->F[3 * f + c] != v) c++;
                sf.push_back(f);
                sc.push_back(c);
            }
            so[v + 1] = (int)sf.size();
            g->max_astar = std::max(g->max_astar, so[v + 1] - so[v]);
        }
        auto up = [](DevBuf &b, const std::vector<int> &v) -> int {
            SOD_TRY(b.ensure(std::max<size_t>(sizeof(int) * v.size(), 16)));
            if (!v.empty()) SOD_CHECK_CUDA(cudaMemcpy(b.p, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice));
            return SOD_OK;
        };
        SOD_TRY(up(g->astar_off, so));
        SOD_TRY(up(g->astar_face, sf));
        SOD_TRY(up(g->astar_corner, sc));
    }
    std::vector<int4> ent;
    std::vector<int> ent_off(nV + 1, 0), slot_off(nV + 1, 0), slot_vert;
    // distinct pairs (f1, f2): the three entries of a pair (one per test corner of f1) share every
    // kernel evaluation, so the singular kernel integrates a pair once for all three
    std::map<std::pair<int, int>, int> pair_id;
    std::vector<int4> pairs;
    for (int a = 0; a < nV; a++) {
        std::vector<std::array<int, 9>> rows;  // f2, cls, ac, j1[3], j2[3]
        std::vector<int> rf1;                  // f1 of each row
        for (int f1 : vf[a]) {
            std::set<int> partners;
            for (int c = 0; c < 3; c++)
                for (int f2 : vfc[canon(m->F[3 * f1 + c])]) partners.insert(f2);
            for (int f2 : partners) {
                int j1[3], j2[3];
                const int cls = classify(m->F.data(), vm, f1, f2, j1, j2);
                int ac = 0;
                while (ac < 3 && j1[ac] != a) ac++;
                rows.push_back({f2, cls, ac, j1[0], j1[1], j1[2], j2[0], j2[1], j2[2]});
                rf1.push_back(f1);
            }
        }
        std::vector<int> sl;
        for (auto &r : rows)
            for (int b = 0; b < 3; b++) sl.push_back(r[6 + b]);
        std::sort(sl.begin(), sl.end());
        sl.erase(std::unique(sl.begin(), sl.end()), sl.end());
        const int base = (int)slot_vert.size();
        for (size_t ri = 0; ri < rows.size(); ri++) {
            auto &r = rows[ri];
            const int f1 = rf1[ri], eidx = (int)(ent.size() / 4);
            auto ins = pair_id.emplace(std::make_pair(f1, r[0]), (int)(pairs.size() / 4));
            if (ins.second) {
                pairs.push_back(make_int4(r[0], r[1], 0, 0));
                pairs.push_back(make_int4(r[3], r[4], r[5], 0));
                pairs.push_back(make_int4(r[6], r[7], r[8], 0));
                pairs.push_back(make_int4(-1, -1, -1, 0));
            }
            int4 &pe = pairs[4 * ins.first->second + 3];
            (r[2] == 0 ? pe.x : r[2] == 1 ? pe.y : pe.z) = eidx;
            int sv[3];
            for (int b = 0; b < 3; b++) sv[b] = base + (int)(std::lower_bound(sl.begin(), sl.end(), r[6 + b]) - sl.begin());
            ent.push_back(make_int4(r[0], r[1], r[2], 0));
            ent.push_back(make_int4(r[3], r[4], r[5], 0));
            ent.push_back(make_int4(r[6], r[7], r[8], 0));
            ent.push_back(make_int4(sv[0], sv[1], sv[2], 0));
        }
        slot_vert.insert(slot_vert.end(), sl.begin(), sl.end());
        ent_off[a + 1] = (int)(ent.size() / 4);
        slot_off[a + 1] = (int)slot_vert.size();
    }
    g->nent = ent_off[nV];
    g->nslots = slot_off[nV];
    g->npairs = (int)(pairs.size() / 4);
    for (int q = 0; q < g->npairs; q++) {
        const int4 pe = pairs[4 * q + 3];
        if (pe.x < 0 || pe.y < 0 || pe.z < 0) {
            set_error("Galerkin set-up: a singular face pair without all three test corners");
            return SOD_ERR_INVALID_ARG;
        }
    }
    auto up = [](DevBuf &b, const void *src, size_t bytes) -> int {
        SOD_TRY(b.ensure(std::max<size_t>(bytes, 16)));
        if (bytes) SOD_CHECK_CUDA(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice));
        return SOD_OK;
    };
    SOD_TRY(up(g->ent, ent.data(), sizeof(int4) * ent.size()));
    SOD_TRY(up(g->ent_off, ent_off.data(), sizeof(int) * ent_off.size()));
    SOD_TRY(up(g->slot_off, slot_off.data(), sizeof(int) * slot_off.size()));
    SOD_TRY(up(g->slot_vert, slot_vert.data(), sizeof(int) * slot_vert.size()));
    SOD_TRY(up(g->pairs, pairs.data(), sizeof(int4) * pairs.size()));
    return SOD_OK;
}

namespace sod {

template <bool GLOBAL> static const void *gal_tp_fn_t(int kind, int bm) {
    constexpr int BT = 1 << SOD_B_TRANS, BA = 1 << SOD_B_ANGULAR;
    if (kind == SOD_H) return (const void *)gal_tp_kernel<SOD_H, 0, GLOBAL>;
    return bm == (BT | BA) ? (const void *)gal_tp_kernel<SOD_G, BT | BA, GLOBAL>
         : bm == BT        ? (const void *)gal_tp_kernel<SOD_G, BT, GLOBAL>
         : bm == BA        ? (const void *)gal_tp_kernel<SOD_G, BA, GLOBAL>
                           : (const void *)gal_tp_kernel<SOD_G, 0, GLOBAL>;
}
static const void *gal_tp_fn(int kind, int bm, bool global = false) {
    return global ? gal_tp_fn_t<true>(kind, bm) : gal_tp_fn_t<false>(kind, bm);
}

// CTA size of the test-point kernel: the collocation scatter's cost model (colours x T / occupancy,
// occupancy from the CUDA occupancy calculator), cached on the mesh.
static int gal_tp_threads(sod_context *ctx, sod_mesh *m, int kind, int bm, const void *fn, int *threads) {
    const int key = 4096 + kind * 16 + bm;
    std::lock_guard<std::recursive_mutex> lock(m->sched_mu);
    auto it = m->tuned.find(key);
    if (it != m->tuned.end()) {
        *threads = it->second;
        return SOD_OK;
    }
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
    SOD_CHECK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(ctx->smem_optin - attr.sharedSizeBytes)));
    const int nc = kind == SOD_G ? 6 : 9;
    const int ncb = (bm & (1 << SOD_B_TRANS) ? 6 : 0) + (bm & (1 << SOD_B_ANGULAR) ? 18 : 0);
    double best = 1e300;
    int bestT = 0;
    for (int T = 32; T <= attr.maxThreadsPerBlock; T += 32) {
        const size_t smem = sizeof(float2) * ((size_t)nc * m->nV + (size_t)ncb * T);
        if (smem + attr.sharedSizeBytes > ctx->smem_optin) continue;
        int per_sm = 0;
        SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem));
        if (per_sm <= 0) continue;
        const sod_mesh::Coloured *col = nullptr;
        SOD_TRY(m->coloured_for(T, &col));
        const double occ = std::min(1.0, (double)per_sm * T / 32.0 / 24.0);
        const double cost = (double)col->ncolors * T / occ;
        if (cost < best * 0.999) best = cost, bestT = T;
    }
    if (bestT == 0) {
        set_error("mesh too large for the shared-memory row accumulator (" + std::to_string(m->nV) + " vertices)");
        return SOD_ERR_UNSUPPORTED;
    }
    m->tuned[key] = bestT;
    *threads = bestT;
    return SOD_OK;
}

// Bytes of test-point row scratch a Galerkin pass may hold at once (frequencies are chunked to fit)
constexpr size_t GAL_ROWS_BUDGET = (size_t)16 << 30;

int launch_galerkin(sod_context *ctx, const CollLaunch &L) {
    const sod_mesh *m = L.mesh;
    sod_mesh *mm = const_cast<sod_mesh *>(m);
    const int mask = L.kind_mask;
    constexpr int BT = 1 << SOD_B_TRANS, BA = 1 << SOD_B_ANGULAR;
    const int bm = mask & (BT | BA);
    PointTable pt;
    SOD_TRY(make_point_table(L.order, L.subdiv, pt));
    SOD_REQUIRE(pt.n <= GAL_MAXQ, "Galerkin test rule: at most 13 points (order <= 7, subdivision 1)");
    SOD_REQUIRE(L.sorder >= 1 && L.sorder <= 5 && L.ssub >= 1 && L.ssub * L.sorder <= 40,
                "singular rule: order 1..5, order x subdivision <= 40");
    if (!m->gal) {
        auto gd = std::make_unique<sod_mesh::GalData>();
        SOD_TRY(build_gal(m, gd.get()));
        mm->gal = std::move(gd);
    }
    sod_mesh::GalData *g = m->gal.get();
    SOD_REQUIRE(g->max_astar <= GAL_MAXS, "vertex with more than 32 faces");
    const bool sing = (L.parts & SOD_PART_SINGULAR) != 0;
    const bool reg = (L.parts & SOD_PART_REGULAR) != 0;
    const long long nslots = g->nslots;
    const int nq = pt.n;
    const long long ntp = (long long)m->nF * nq;  // test points
    DuffyRule dr{};
    {
        int n = 0;
        const double(*t)[2] = gl_rule_table(L.sorder, n);
        dr.n = 0;
        for (int s = 0; s < L.ssub; s++) {
            const double lo = (double)s / L.ssub, hi = (double)(s + 1) / L.ssub;
            for (int q = 0; q < n; q++) {
                dr.x[dr.n] = (hi - lo) * t[q][0] / 2. + (lo + hi) / 2.;
                dr.w[dr.n] = t[q][1] * (hi - lo) / 2.;
                dr.n++;
            }
        }
    }
    const size_t esz = L.out_dtype == SOD_C64 ? 8 : 16;
    // passes: G (with the B kinds of the mask; run for B even when G itself is not requested), H
    for (int kd = 0; kd < 2; kd++) {
        const bool run = kd == SOD_G ? ((mask & (1 << SOD_G)) || bm) : (mask & (1 << SOD_H)) != 0;
        if (!run) continue;
        const int pbm = kd == SOD_G ? bm : 0;
        const int NCS = kd == SOD_G ? 6 : 9;
        const int ncb = (pbm & BT ? 6 : 0) + (pbm & BA ? 18 : 0);
        const void *fn = gal_tp_fn(kd, pbm);
        int T = 0;
        bool tp_global = false;  // row block beyond shared memory: accumulate in the output row
        if (ctx->gal_threads > 0) {
            cudaFuncAttributes attr;
            SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
            T = std::max(32, std::min(attr.maxThreadsPerBlock, (ctx->gal_threads / 32) * 32));
        } else if (reg) {
            const int rc = gal_tp_threads(ctx, mm, kd, pbm, fn, &T);
            if (rc == SOD_ERR_UNSUPPORTED) {
                tp_global = true;
                T = 256;
            } else if (rc != SOD_OK) {
                return rc;
            }
        }
        const sod_mesh::Coloured *col = nullptr;
        size_t smem = 0;
        if (reg) {
            SOD_TRY(mm->coloured_for(T, &col));
            cudaFuncAttributes attr;
            smem = sizeof(float2) * ((size_t)NCS * m->nV + (size_t)ncb * T);
            SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
            if (!tp_global && smem + attr.sharedSizeBytes > ctx->smem_optin) tp_global = true;
            if (tp_global) {
                fn = gal_tp_fn(kd, pbm, true);
                SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
                smem = sizeof(float2) * (size_t)ncb * T;  // only the B columns stay in shared memory
                if (smem + attr.sharedSizeBytes > ctx->smem_optin) {
                    set_error("Galerkin B columns exceed shared memory");
                    return SOD_ERR_UNSUPPORTED;
                }
            }
            SOD_CHECK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)(ctx->smem_optin - attr.sharedSizeBytes)));
        }
        // frequency chunk: singular scratch limit and the test-point row scratch budget
        const size_t rows_per_f = (size_t)ntp * NCS * m->nV * sizeof(float2), b_per_f = (size_t)ntp * ncb * sizeof(cd);
        int chunk = std::min(L.nfreq, MAX_FREQ_PER_LAUNCH);
        if (reg) chunk = std::max(1, std::min<int>(chunk, (int)(GAL_ROWS_BUDGET / (rows_per_f + b_per_f))));
        if (reg) {
            SOD_TRY(ctx->gal_rows.ensure(rows_per_f * chunk));
            if (ncb) SOD_TRY(ctx->gal_bsum.ensure(b_per_f * chunk));
        }
        // singular scratch: slot blocks, then per-vertex B (9 + 27); results per entry, then B moments
        const long long s_slots = nslots * 9, s_bt = (long long)m->nV * 9, s_ba = (long long)m->nV * 27;
        const long long r_main = (long long)g->nent * 3 * NCS, r_b = pbm ? (long long)g->nent * GAL_BMOM : 0;
        if (sing) {
            SOD_TRY(ctx->sing.ensure(sizeof(cd) * (size_t)std::max<long long>((s_slots + s_bt + s_ba) * chunk, 1)));
            SOD_TRY(ctx->sing_res.ensure(sizeof(double2) * (size_t)std::max<long long>((r_main + r_b) * chunk, 1)));
        }
        cd *S = ctx->sing.as<cd>();
        cd *SBt = S + s_slots * chunk, *SBa = SBt + s_bt * chunk;
        double2 *R = ctx->sing_res.as<double2>(), *RB = R + r_main * chunk;
        for (int f0 = 0; f0 < L.nfreq; f0 += chunk) {
            const int nf = std::min(chunk, L.nfreq - f0);
            FreqTable ft;
            ft.n = nf;
            for (int l = 0; l < nf; l++) {
                ft.kd[l] = L.kc_host[f0 + l];
                ft.kf[l] = to_float(ft.kd[l]);
            }
            GalSingArgs sa{g->nent, g->npairs, g->pairs.as<int4>(), m->dV.as<double>(), m->dN.as<double>(), R, RB};
            GalArgs a{};
            a.nV = m->nV;
            a.nF = m->nF;
            a.faces = reg ? col->dFaces.as<float4>() : nullptr;
            a.color_off = reg ? col->dOff.as<int>() : nullptr;
            a.ncolors = reg ? col->ncolors : 0;
            a.faces_nat = m->dFacesNat.as<float4>();
            a.star_off = g->astar_off.as<int>();
            a.star_face = g->astar_face.as<int>();
            a.star_corner = g->astar_corner.as<int>();
            a.out = L.out[kd] ? static_cast<char *>(L.out[kd]) + (size_t)f0 * (size_t)L.freq_stride[kd] * esz : nullptr;
            a.fstride = L.freq_stride[kd];
            a.out_c64 = L.out_dtype == SOD_C64;
            a.do_regular = reg;
            a.S = sing ? S : nullptr;
            a.S_fstride = s_slots;
            a.slot_off = g->slot_off.as<int>();
            a.slot_vert = g->slot_vert.as<int>();
            for (int b = 0; b < 2; b++) {
                const int kb = SOD_B_TRANS + b;
                a.outB[b] = (pbm & (1 << kb)) && L.out[kb]
                                ? static_cast<char *>(L.out[kb]) + (size_t)f0 * (size_t)L.freq_stride[kb] * esz
                                : nullptr;
                a.fstrideB[b] = L.freq_stride[kb];
                a.SB[b] = (sing && (pbm & (1 << kb))) ? (b == 0 ? SBt : SBa) : nullptr;
                a.SB_fstride[b] = b == 0 ? s_bt : s_ba;
            }
            // singular pairs and their combination into slot blocks
            if (sing && g->nent > 0) {
                static std::atomic<bool> attr_done[64];  // per device: the G + B variants need more than 48 KB
                if (ctx->device < 0 || ctx->device >= 64 || !attr_done[ctx->device]) {
                    const void *fns[3] = {(const void *)gal_sing_kernel<SOD_G, BT | BA>,
                                          (const void *)gal_sing_kernel<SOD_G, BT>, (const void *)gal_sing_kernel<SOD_G, BA>};
                    for (const void *f : fns)
                        SOD_CHECK_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                            4 * 4 * sing_warp_floats<SOD_G, BT | BA>()));
                    if (ctx->device >= 0 && ctx->device < 64) attr_done[ctx->device] = true;
                }
                const dim3 grid((g->npairs * 32 + 127) / 128, nf);
                if (kd == SOD_H)
                    gal_sing_kernel<SOD_H, 0><<<grid, 128, 4 * 4 * sing_warp_floats<SOD_H, 0>(), L.stream>>>(sa, dr, ft);
                else if (pbm == (BT | BA))
                    gal_sing_kernel<SOD_G, BT | BA>
                        <<<grid, 128, 4 * 4 * sing_warp_floats<SOD_G, BT | BA>(), L.stream>>>(sa, dr, ft);
                else if (pbm == BT)
                    gal_sing_kernel<SOD_G, BT><<<grid, 128, 4 * 4 * sing_warp_floats<SOD_G, BT>(), L.stream>>>(sa, dr, ft);
                else if (pbm == BA)
                    gal_sing_kernel<SOD_G, BA><<<grid, 128, 4 * 4 * sing_warp_floats<SOD_G, BA>(), L.stream>>>(sa, dr, ft);
                else
                    gal_sing_kernel<SOD_G, 0><<<grid, 128, 4 * 4 * sing_warp_floats<SOD_G, 0>(), L.stream>>>(sa, dr, ft);
                SOD_CHECK_CUDA(cudaGetLastError());
                ctx->count();
                const int blocks = (int)(((long long)m->nV * nf * 32 + 127) / 128);
                if (kd == SOD_G)
                    gal_combine_kernel<SOD_G><<<blocks, 128, 0, L.stream>>>(
                        m->nV, g->nent, g->ent_off.as<int>(), g->ent.as<int4>(), g->slot_off.as<int>(), R, S, s_slots, nf);
                else
                    gal_combine_kernel<SOD_H><<<blocks, 128, 0, L.stream>>>(
                        m->nV, g->nent, g->ent_off.as<int>(), g->ent.as<int4>(), g->slot_off.as<int>(), R, S, s_slots, nf);
                SOD_CHECK_CUDA(cudaGetLastError());
                ctx->count();
                if (pbm) {
                    if (pbm == (BT | BA))
                        gal_combine_b_kernel<BT | BA><<<blocks, 128, 0, L.stream>>>(
                            m->nV, g->nent, g->ent_off.as<int>(), g->ent.as<int4>(), m->dN.as<double>(), RB, SBt, SBa, nf);
                    else if (pbm == BT)
                        gal_combine_b_kernel<BT><<<blocks, 128, 0, L.stream>>>(
                            m->nV, g->nent, g->ent_off.as<int>(), g->ent.as<int4>(), m->dN.as<double>(), RB, SBt, SBa, nf);
                    else
                        gal_combine_b_kernel<BA><<<blocks, 128, 0, L.stream>>>(
                            m->nV, g->nent, g->ent_off.as<int>(), g->ent.as<int4>(), m->dN.as<double>(), RB, SBt, SBa, nf);
                    SOD_CHECK_CUDA(cudaGetLastError());
                    ctx->count();
                }
            }
            // regular pairs: rows of every test point, then the per-vertex combination (which also
            // adds the singular blocks)
            GalGatherArgs ga{};
            ga.g = a;
            ga.nq = nq;
            ga.do_regular = reg;
            ga.rows_fstride = ntp * NCS * m->nV;
            ga.b_fstride = ntp * ncb;
            if (reg) {
                GalTpArgs ta{};
                ta.nV = m->nV;
                ta.nq = nq;
                ta.t0 = 0;
                ta.faces = col->dFaces.as<float4>();
                ta.color_off = col->dOff.as<int>();
                ta.ncolors = col->ncolors;
                ta.faces_nat = m->dFacesNat.as<float4>();
                ta.canon_faces = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
                ta.canon_nat = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
                ta.rows = ctx->gal_rows.as<float2>();
                ta.rows_fstride = ga.rows_fstride;
                ta.bsum = ncb ? ctx->gal_bsum.as<cd>() : nullptr;
                ta.b_fstride = ga.b_fstride;
                const dim3 grid((unsigned)ntp, nf);
                if (tp_global) {
                    if (kd == SOD_H)
                        gal_tp_kernel<SOD_H, 0, true><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                    else if (pbm == (BT | BA))
                        gal_tp_kernel<SOD_G, BT | BA, true><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                    else if (pbm == BT)
                        gal_tp_kernel<SOD_G, BT, true><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                    else if (pbm == BA)
                        gal_tp_kernel<SOD_G, BA, true><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                    else
                        gal_tp_kernel<SOD_G, 0, true><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                } else if (kd == SOD_H)
                    gal_tp_kernel<SOD_H, 0><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                else if (pbm == (BT | BA))
                    gal_tp_kernel<SOD_G, BT | BA><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                else if (pbm == BT)
                    gal_tp_kernel<SOD_G, BT><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                else if (pbm == BA)
                    gal_tp_kernel<SOD_G, BA><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                else
                    gal_tp_kernel<SOD_G, 0><<<grid, T, smem, L.stream>>>(ta, pt, ft);
                SOD_CHECK_CUDA(cudaGetLastError());
                ctx->count();
                ga.rows = ta.rows;
                ga.bsum = ta.bsum;
            }
            const dim3 grid(m->nV, nf);
            if (kd == SOD_H)
                gal_gather_kernel<SOD_H, 0><<<grid, 256, 0, L.stream>>>(ga, pt);
            else if (pbm == (BT | BA))
                gal_gather_kernel<SOD_G, BT | BA><<<grid, 256, 0, L.stream>>>(ga, pt);
            else if (pbm == BT)
                gal_gather_kernel<SOD_G, BT><<<grid, 256, 0, L.stream>>>(ga, pt);
            else if (pbm == BA)
                gal_gather_kernel<SOD_G, BA><<<grid, 256, 0, L.stream>>>(ga, pt);
            else
                gal_gather_kernel<SOD_G, 0><<<grid, 256, 0, L.stream>>>(ga, pt);
            SOD_CHECK_CUDA(cudaGetLastError());
            ctx->count();
        }
    }
    return SOD_OK;
}

}  // namespace sod
