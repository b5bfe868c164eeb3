// sod_collocation.cu -- collocation assembly of the Laplace-domain CQBEM matrices on sm_103a.
//
// Replaces, for all field vertices at once, the reference's per-row kernels
//   compute_elastodynamic_{G,H,B_trans,B_angular}_kernel_collocation
//   (src/elastodynamics_cqbem_{G,H,B_trans,B_angular}_collocation.cu).
//
// Work split
//   * regular (non-singular) face integrals, FP32:
//       G, H   : one CTA per (field vertex i, frequency).  The CTA keeps the whole row block
//                U[3i:3i+3, :] in shared memory and walks the faces in colour order: faces of
//                one colour share no vertex, so every thread adds its face's three corner blocks
//                without conflicts, and the summation order is fixed -> bitwise reproducible
//                results with no atomics.  One __syncthreads() separates colours.
//       B_t,B_a: one CTA per (i, frequency), per-thread partial sums over faces, fixed-order
//                warp/CTA reduction in FP64.
//   * singular (x_i on the face) integrals, FP64: polar rule (G, B_trans, B_angular,
//     include/integrator_collocation.hpp:19-63) or Guiggiani's CPV rule (H, :68-124), one warp
//     per (i, star face), deterministic warp reduction, summed per neighbour slot into a small
//     FP64 side buffer that the regular kernel's epilogue adds before the single store.
#include <cstdio>

#include "sod_internal.h"

namespace sod {

// 1-D Gauss-Legendre rules on [-1,1], orders 1..5 (include/integrator.hpp:117-133 of the reference)
__constant__ double c_glx[5][5];
__constant__ double c_glw[5][5];

struct FaceRec {
    float3 y1, y2, y3, n;
    float area;
    int j0, j1, j2;
};
__device__ __forceinline__ FaceRec load_face(const float4 *__restrict__ faces, int f) {
    const float4 q0 = __ldg(faces + 4 * f), q1 = __ldg(faces + 4 * f + 1), q2 = __ldg(faces + 4 * f + 2),
                 q3 = __ldg(faces + 4 * f + 3);
    FaceRec r;
    r.y1 = make_float3(q0.x, q0.y, q0.z);
    r.area = q0.w;
    r.y2 = make_float3(q1.x, q1.y, q1.z);
    r.y3 = make_float3(q2.x, q2.y, q2.z);
    r.n = make_float3(q1.w, q2.w, q3.x);
    r.j0 = __float_as_int(q3.y);
    r.j1 = __float_as_int(q3.z);
    r.j2 = __float_as_int(q3.w);
    return r;
}

struct CollArgs {
    int nV, nF;
    const float4 *faces;       // coloured (scatter kernels) or natural (reduce kernels) order
    const int4 *canonF;        // canonical corner ids per face record, or null
    const int *color_off;      // ncolors+1 (scatter kernels)
    int ncolors;
    const float *Vf;           // nV x 3
    const int *canonV;         // canonical id per vertex, or null
    void *out;
    int out_c64;               // 1: complex64 output, 0: complex128
    long long ld;              // row stride of out (elements)
    long long fstride;         // frequency stride of out (elements)
    int do_regular;
    const cd *S;               // singular corrections (null if none)
    const int *nbr_off;        // G/H: per vertex slot ranges
    const int *nbr_vert;
    long long S_fstride;       // elements (cd) between frequencies in S
};

__device__ __forceinline__ bool is_singular(const CollArgs &a, int i, int ci, int f, const FaceRec &fr) {
    if (a.canonF) {
        const int4 c = __ldg(a.canonF + f);
        return c.x == ci || c.y == ci || c.z == ci;
    }
    return fr.j0 == i || fr.j1 == i || fr.j2 == i;
}

__device__ __forceinline__ void store_out(void *out, int c64, long long idx, double re, double im) {
    if (c64)
        reinterpret_cast<float2 *>(out)[idx] = make_float2((float)re, (float)im);
    else
        reinterpret_cast<double2 *>(out)[idx] = make_double2(re, im);
}

// -------------------------------------------------------------------------------------------
// G / H regular scatter kernel
template <int KIND>
__global__ void __launch_bounds__(512, 1) coll_scatter_kernel(CollArgs a, PointTable pt,
                                                               const __grid_constant__ FreqTable ft) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;
    extern __shared__ float2 acc[];  // [NC][nV]
    const int i = blockIdx.x, fq = blockIdx.y;
    const int nV = a.nV;
    for (int t = threadIdx.x; t < NC * nV; t += blockDim.x) acc[t] = make_float2(0.f, 0.f);
    const KConst<float> k = ft.kf[fq];
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    __syncthreads();
    if (a.do_regular) {
        for (int c = 0; c < a.ncolors; c++) {
            const int f = a.color_off[c] + threadIdx.x;
            if (f < a.color_off[c + 1]) {
                const FaceRec fr = load_face(a.faces, f);
                if (!is_singular(a, i, ci, f, fr)) {
                    cf part[3][NC];
#pragma unroll
                    for (int kk = 0; kk < 3; kk++)
#pragma unroll
                        for (int cc = 0; cc < NC; cc++) part[kk][cc] = mk(0.f, 0.f);
                    for (int q = 0; q < pt.n; q++) {
                        const float4 P = pt.p[q];
                        const float yx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x;
                        const float yy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y;
                        const float yz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z;
                        const float dx = yx - x.x, dy = yy - x.y, dz = yz - x.z;
                        const float r2 = dx * dx + dy * dy + dz * dz;
                        const float rinv = rsqrtf(r2);
                        const float r = r2 * rinv;
                        const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                        const RadialTerms<float, cf> t = radial<float, cf>(r, k);
                        cf u[NC];
                        if (KIND == SOD_G) {
                            cf al, be;
                            g_coeffs(t, k, rinv, al, be);
#pragma unroll
                            for (int p = 0; p < 3; p++)
#pragma unroll
                                for (int qq = p; qq < 3; qq++) {
                                    cf v = al * (rh[p] * rh[qq]);
                                    if (p == qq) v = v + be;
                                    u[sym_index(p, qq)] = v;
                                }
                        } else {
                            cf ha, hb, hd;
                            h_coeffs(t, k, rinv * rinv, ha, hb, hd);
                            const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
                            const float rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                            const cf hdr = hd * rn, hbr = hb * rn;
#pragma unroll
                            for (int p = 0; p < 3; p++)
#pragma unroll
                                for (int qq = 0; qq < 3; qq++) {
                                    cf v = ha * (rh[p] * nn[qq]) + hb * (nn[p] * rh[qq]) + hdr * (rh[p] * rh[qq]);
                                    if (p == qq) v = v + hbr;
                                    u[3 * p + qq] = v;
                                }
                        }
                        const float w = P.w * fr.area;
                        const float wl[3] = {w * P.x, w * P.y, w * P.z};
#pragma unroll
                        for (int kk = 0; kk < 3; kk++)
#pragma unroll
                            for (int cc = 0; cc < NC; cc++) cfma(part[kk][cc], u[cc], wl[kk]);
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
            }
            __syncthreads();
        }
    }
    // epilogue: row block 3 x 3nV
    const long long base = (long long)fq * a.fstride + (long long)(3 * i) * a.ld;
    const int ncol = 3 * nV;
    for (int p = 0; p < 3; p++) {
        for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
            const int j = col / 3, qq = col - 3 * j;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : 3 * p + qq;
            const float2 v = acc[comp * nV + j];
            store_out(a.out, a.out_c64, base + p * a.ld + col, v.x, v.y);
        }
    }
    if (a.S) {
        __syncthreads();
        const int s0 = a.nbr_off[i], ns = a.nbr_off[i + 1] - s0;
        for (int e = threadIdx.x; e < ns * 9; e += blockDim.x) {
            const int sl = s0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
            const int j = a.nbr_vert[sl];
            const int comp = KIND == SOD_G ? sym_index(p, qq) : pq;
            const float2 v = acc[comp * nV + j];
            const cd sv = a.S[(long long)fq * a.S_fstride + (long long)sl * 9 + pq];
            store_out(a.out, a.out_c64, base + p * a.ld + 3 * j + qq, (double)v.x + sv.x, (double)v.y + sv.y);
        }
    }
}

// -------------------------------------------------------------------------------------------
// B_trans / B_angular regular reduction kernel
template <int KIND>
__global__ void __launch_bounds__(256) coll_reduce_kernel(CollArgs a, PointTable pt,
                                                          const __grid_constant__ FreqTable ft) {
    constexpr int NC = KIND == SOD_B_TRANS ? 6 : 18;  // Ba: (pq sym) x k
    const int i = blockIdx.x, fq = blockIdx.y;
    const KConst<float> k = ft.kf[fq];
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
            cf part[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) part[c] = mk(0.f, 0.f);
            for (int q = 0; q < pt.n; q++) {
                const float4 P = pt.p[q];
                const float dx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x - x.x;
                const float dy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y - x.y;
                const float dz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z - x.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float rinv = rsqrtf(r2);
                const float r = r2 * rinv;
                const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                const float rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                const RadialTerms<float, cf> t = radial<float, cf>(r, k);
                const float w = P.w;
                if (KIND == SOD_B_TRANS) {
                    cf sy, di;
                    bt_coeffs(t, k, 1.0f, sy, di);
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = p; qq < 3; qq++) {
                            cf v = sy * (rh[p] * nn[qq] + rh[qq] * nn[p]);
                            if (p == qq) v = v + di * rn;
                            cfma(part[sym_index(p, qq)], v, w);
                        }
                } else {
                    cf A, Bq, Cq;
                    ba_coeffs(t, k, r, 1.0f, A, Bq, Cq);
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = p; qq < 3; qq++)
#pragma unroll
                            for (int kk = 0; kk < 3; kk++) {
                                const float T1 = rh[p] * rh[kk] * nn[qq] + rh[qq] * rh[kk] * nn[p] +
                                                 (qq == kk ? nn[p] : 0.f) + (p == kk ? nn[qq] : 0.f);
                                const float T2 = (qq == kk ? nn[p] : 0.f) + (p == kk ? nn[qq] : 0.f);
                                const float T3 = p == qq ? nn[kk] : 0.f;
                                cf v = A * T1 + Bq * T2 + Cq * T3;
                                cfma(part[3 * sym_index(p, qq) + kk], v, w);
                            }
                }
            }
#pragma unroll
            for (int c = 0; c < NC; c++) cfma(accl[c], part[c], fr.area);
        }
    }
    // deterministic reduction in FP64: warp butterfly then fixed-order over warps
    __shared__ cd wsum[8][NC];
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
    const long long base = (long long)fq * a.fstride + (long long)(3 * i) * a.ld;
    if (KIND == SOD_B_TRANS) {
        for (int e = threadIdx.x; e < 9; e += blockDim.x) {
            const int p = e / 3, qq = e % 3;
            cd s = mk(0.0, 0.0);
            for (int w = 0; w < nw; w++) s = s + wsum[w][sym_index(p, qq)];
            if (a.S) s = s + a.S[(long long)fq * a.S_fstride + (long long)i * 9 + e];
            store_out(a.out, a.out_c64, base + p * a.ld + qq, s.x, s.y);
        }
    } else {
        for (int e = threadIdx.x; e < 27; e += blockDim.x) {
            const int p = e / 9, qq = (e / 3) % 3, kk = e % 3;
            cd s = mk(0.0, 0.0);
            for (int w = 0; w < nw; w++) s = s + wsum[w][3 * sym_index(p, qq) + kk];
            if (a.S) s = s + a.S[(long long)fq * a.S_fstride + (long long)i * 27 + e];
            store_out(a.out, a.out_c64, base + p * a.ld + 3 * qq + kk, s.x, s.y);
        }
    }
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
    cd *S;
    long long S_fstride;
};

constexpr int MAX_STAR = 32;

__device__ __forceinline__ double3 ld3(const double *p, int i) { return make_double3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ double3 operator-(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 operator+(double3 a, double3 b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 operator*(double3 a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double norm3(double3 a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ double3 nrmz(double3 a) {
    const double n = norm3(a);
    return n > 0.0 ? a * (1.0 / n) : a;
}
__device__ __forceinline__ double comp3(double3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// barycentrics of P in (A,B,C), clamped (include/barycentric_coordinates.cuh:14-38)
__device__ __forceinline__ void bary_clamped(double3 P, double3 A, double3 B, double3 C, double L[3]) {
    const double3 v0 = B - A, v1 = C - A, v2 = P - A;
    const double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1), d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    const double den = d00 * d11 - d01 * d01;
    L[1] = (d11 * d20 - d01 * d21) / den;
    L[2] = (d00 * d21 - d01 * d20) / den;
    L[0] = 1.0 - (L[1] + L[2]);
    for (int c = 0; c < 3; c++) L[c] = fmin(1.0, fmax(0.0, L[c]));
}

template <int NVAL>
__device__ __forceinline__ void warp_sum(cd (&v)[NVAL]) {
#pragma unroll
    for (int c = 0; c < NVAL; c++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v[c].x += __shfl_xor_sync(0xffffffffu, v[c].x, o);
            v[c].y += __shfl_xor_sync(0xffffffffu, v[c].y, o);
        }
    }
}

// Polar-rule geometry about the singular vertex (include/integrator_collocation.hpp:28-36)
struct Polar {
    double3 y1, y2, y3, xh, yh;
    double a, alpha, beta;
};
__device__ __forceinline__ Polar polar_setup(double3 y1, double3 y2, double3 y3) {
    Polar g;
    g.y1 = y1, g.y2 = y2, g.y3 = y3;
    const double3 v1 = y2 - y1, v2 = y3 - y1;
    const double3 v1n = nrmz(v1), v2n = nrmz(v2);
    g.xh = v1n;
    g.yh = nrmz(cross3(cross3(g.xh, v2n), g.xh));
    const double3 v12 = v1 + nrmz(v2 - v1) * dot3(v1, nrmz(v1 - v2));
    g.a = norm3(v12);
    g.alpha = acos(dot3(v1n, v2n));
    g.beta = acos(fmin(1.0, fmax(-1.0, dot3(nrmz(v12), v1n))));
    return g;
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

template <int KIND>
__global__ void __launch_bounds__(256) coll_singular_kernel(SingArgs a, const __grid_constant__ FreqTable ft) {
    constexpr int NC = KIND == SOD_G ? 6 : (KIND == SOD_H ? 9 : (KIND == SOD_B_TRANS ? 6 : 18));
    constexpr int NCORN = (KIND == SOD_G || KIND == SOD_H) ? 3 : 1;
    __shared__ cd fres[MAX_STAR][NCORN * NC];
    const int i = blockIdx.x, fq = blockIdx.y;
    const KConst<double> k = ft.kd[fq];
    const int s0 = a.star_off[i], ns = min(a.star_off[i + 1] - a.star_off[i], MAX_STAR);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nq = a.sorder * a.ssub;
    for (int si = warp; si < ns; si += nw) {
        const int f = a.star_face[s0 + si], sc = a.star_corner[s0 + si];
        const int jj[3] = {a.F[3 * f + sc], a.F[3 * f + (sc + 1) % 3], a.F[3 * f + (sc + 2) % 3]};
        const double3 y1 = ld3(a.V, jj[0]), y2 = ld3(a.V, jj[1]), y3 = ld3(a.V, jj[2]);
        const double3 n = ld3(a.N, f);
        const double nn[3] = {n.x, n.y, n.z};
        cd acc[NCORN * NC];
#pragma unroll
        for (int c = 0; c < NCORN * NC; c++) acc[c] = mk(0.0, 0.0);
        if (KIND != SOD_H) {
            const Polar g = polar_setup(y1, y2, y3);
            for (int pidx = lane; pidx < nq * nq; pidx += 32) {
                double r, w;
                double3 rh;
                polar_point(g, pidx, a.sorder, a.ssub, r, rh, w);
                const double rr[3] = {rh.x, rh.y, rh.z};
                const RadialTerms<double, cd> t = radial<double, cd>(r, k);
                if (KIND == SOD_G) {
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
                            for (int c = 0; c < 3; c++) cfma(acc[c * NC + sym_index(p, qq)], v, w * L[c]);
                        }
                } else if (KIND == SOD_B_TRANS) {
                    const double rn = dot3(rh, n);
                    cd sy, di;
                    bt_coeffs(t, k, r, sy, di);  // r * b
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = p; qq < 3; qq++) {
                            cd v = sy * (rr[p] * nn[qq] + rr[qq] * nn[p]);
                            if (p == qq) v = v + di * rn;
                            cfma(acc[sym_index(p, qq)], v, w);
                        }
                } else {
                    cd A, Bq, Cq;
                    ba_coeffs(t, k, r, r, A, Bq, Cq);  // r * b
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int qq = p; qq < 3; qq++)
#pragma unroll
                            for (int kk = 0; kk < 3; kk++) {
                                const double T1 = rr[p] * rr[kk] * nn[qq] + rr[qq] * rr[kk] * nn[p] +
                                                  (qq == kk ? nn[p] : 0.0) + (p == kk ? nn[qq] : 0.0);
                                const double T2 = (qq == kk ? nn[p] : 0.0) + (p == kk ? nn[qq] : 0.0);
                                const double T3 = p == qq ? nn[kk] : 0.0;
                                cd v = A * T1 + Bq * T2 + Cq * T3;
                                cfma(acc[3 * sym_index(p, qq) + kk], v, w);
                            }
                }
            }
        } else {
            // Guiggiani-Gigante rule (include/integrator_collocation.hpp:68-124)
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
        }
        warp_sum<NCORN * NC>(acc);
        if (lane == 0 && si < MAX_STAR) {
#pragma unroll
            for (int c = 0; c < NCORN * NC; c++) fres[si][c] = acc[c];
        }
    }
    __syncthreads();
    const long long sb = (long long)fq * a.S_fstride;
    if (KIND == SOD_G || KIND == SOD_H) {
        const int n0 = a.nbr_off[i], nsl = a.nbr_off[i + 1] - n0;
        for (int e = threadIdx.x; e < nsl * 9; e += blockDim.x) {
            const int sl = n0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : pq;
            cd s = mk(0.0, 0.0);
            for (int si = 0; si < ns; si++)
                for (int c = 0; c < 3; c++)
                    if (a.star_slot[3 * (s0 + si) + c] == sl) s = s + fres[si][c * NC + comp];
            a.S[sb + (long long)sl * 9 + pq] = s;
        }
    } else if (KIND == SOD_B_TRANS) {
        for (int e = threadIdx.x; e < 9; e += blockDim.x) {
            cd s = mk(0.0, 0.0);
            for (int si = 0; si < ns; si++) s = s + fres[si][sym_index(e / 3, e % 3)];
            a.S[sb + (long long)i * 9 + e] = s;
        }
    } else {
        for (int e = threadIdx.x; e < 27; e += blockDim.x) {
            const int p = e / 9, qq = (e / 3) % 3, kk = e % 3;
            cd s = mk(0.0, 0.0);
            for (int si = 0; si < ns; si++) s = s + fres[si][3 * sym_index(p, qq) + kk];
            a.S[sb + (long long)i * 27 + e] = s;
        }
    }
}

// -------------------------------------------------------------------------------------------
// host launcher
static bool g_const_ready[64] = {};

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

int launch_collocation(sod_context *ctx, const CollLaunch &L) {
    const sod_mesh *m = L.mesh;
    SOD_TRY(ensure_gl_constants(ctx->device));
    PointTable pt;
    SOD_TRY(make_point_table(L.order, L.subdiv, pt));
    SOD_REQUIRE(L.sorder >= 1 && L.sorder <= 5 && L.ssub >= 1 && L.ssub <= 8,
                "singular quadrature order must be 1..5, subdivision 1..8");
    const bool sing = (L.parts & SOD_PART_SINGULAR) != 0;
    const bool gh = L.kind == SOD_G || L.kind == SOD_H;
    const int ncomp_s = L.kind == SOD_B_ANGULAR ? 27 : 9;
    const long long s_fstride = gh ? (long long)m->nbr_off.back() * 9 : (long long)m->nV * ncomp_s;
    const int chunk = std::min(L.nfreq, MAX_FREQ_PER_LAUNCH);
    cd *S = nullptr;
    if (sing) {
        SOD_TRY(ctx->sing.ensure(sizeof(cd) * (size_t)s_fstride * chunk));
        S = ctx->sing.as<cd>();
    }
    int threads = 256;
    const sod_mesh::Coloured *col = nullptr;
    size_t smem = 0;
    if (gh) {
        threads = ctx->coll_threads;
        if (threads <= 0) threads = m->nF >= 4096 ? 512 : (m->nF >= 1024 ? 256 : 128);
        threads = std::max(32, std::min(512, (threads / 32) * 32));
        SOD_TRY(const_cast<sod_mesh *>(m)->coloured_for(threads, &col));
        smem = sizeof(float2) * (L.kind == SOD_G ? 6 : 9) * (size_t)m->nV;
        if (smem > ctx->smem_optin) {
            set_error("mesh too large for the shared-memory row accumulator (" + std::to_string(m->nV) + " vertices)");
            return SOD_ERR_UNSUPPORTED;
        }
        if (L.kind == SOD_G)
            SOD_CHECK_CUDA(cudaFuncSetAttribute(coll_scatter_kernel<SOD_G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        else
            SOD_CHECK_CUDA(cudaFuncSetAttribute(coll_scatter_kernel<SOD_H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    for (int f0 = 0; f0 < L.nfreq; f0 += chunk) {
        const int nf = std::min(chunk, L.nfreq - f0);
        FreqTable ft;
        ft.n = nf;
        for (int l = 0; l < nf; l++) {
            ft.kd[l] = L.kc_host[f0 + l];
            ft.kf[l] = to_float(ft.kd[l]);
        }
        const dim3 grid(m->nV, nf);
        if (sing) {
            SingArgs sa;
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
            sa.S = S;
            sa.S_fstride = s_fstride;
            switch (L.kind) {
            case SOD_G: coll_singular_kernel<SOD_G><<<grid, 256, 0, L.stream>>>(sa, ft); break;
            case SOD_H: coll_singular_kernel<SOD_H><<<grid, 256, 0, L.stream>>>(sa, ft); break;
            case SOD_B_TRANS: coll_singular_kernel<SOD_B_TRANS><<<grid, 256, 0, L.stream>>>(sa, ft); break;
            default: coll_singular_kernel<SOD_B_ANGULAR><<<grid, 256, 0, L.stream>>>(sa, ft); break;
            }
            SOD_CHECK_CUDA(cudaGetLastError());
            ctx->count();
        }
        CollArgs a{};
        a.nV = m->nV;
        a.nF = m->nF;
        a.Vf = m->dVf.as<float>();
        a.canonV = m->has_vmap ? m->dCanon.as<int>() : nullptr;
        const size_t esz = L.out_dtype == SOD_C64 ? 8 : 16;
        a.out = static_cast<char *>(L.out) + (size_t)f0 * (size_t)L.freq_stride * esz;
        a.out_c64 = L.out_dtype == SOD_C64;
        a.fstride = L.freq_stride;
        a.do_regular = (L.parts & SOD_PART_REGULAR) != 0;
        a.S = S;
        a.nbr_off = m->dNbrOff.as<int>();
        a.nbr_vert = m->dNbrVert.as<int>();
        a.S_fstride = s_fstride;
        if (gh) {
            a.faces = col->dFaces.as<float4>();
            a.canonF = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
            a.color_off = col->dOff.as<int>();
            a.ncolors = col->ncolors;
            a.ld = 3LL * m->nV;
            if (L.kind == SOD_G)
                coll_scatter_kernel<SOD_G><<<grid, threads, smem, L.stream>>>(a, pt, ft);
            else
                coll_scatter_kernel<SOD_H><<<grid, threads, smem, L.stream>>>(a, pt, ft);
        } else {
            a.faces = m->dFacesNat.as<float4>();
            a.canonF = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
            a.ld = L.kind == SOD_B_TRANS ? 3 : 9;
            if (L.kind == SOD_B_TRANS)
                coll_reduce_kernel<SOD_B_TRANS><<<grid, 256, 0, L.stream>>>(a, pt, ft);
            else
                coll_reduce_kernel<SOD_B_ANGULAR><<<grid, 256, 0, L.stream>>>(a, pt, ft);
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    return SOD_OK;
}

}  // namespace sod
