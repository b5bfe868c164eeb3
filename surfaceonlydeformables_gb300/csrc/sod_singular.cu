// sod_singular.cu -- singular collocation quadrature in double-float on the FP32 pipes.
//
// For field vertex x_i and a face f of its star (x_i is corner `sc` of f) the reference integrates
//   G, B_trans, B_angular : the polar rule about x_i (include/integrator_collocation.hpp:19-63),
//   H                     : the Guiggiani-Gigante CPV rule (include/integrator_collocation.hpp:68-124)
// in FP64.  GB300 runs FP64 at 1/64 of its FP32 rate, so here:
//   1. sing_geom_kernel (FP64, once per mesh and rule) tabulates the frequency-independent part of
//      every quadrature point of every star entry -- r, r-hat, r-hat.n, the polar weights times the
//      barycentric shape functions -- as float pairs, plus the frequency-independent CPV
//      subtraction term of H;
//   2. polar_dd / guig_dd (one thread per star entry and frequency) evaluate the radial terms
//      (two complex exponentials, two psi) and the kernel tensors in double-float (48-bit
//      significand; sod_dd.cuh) and write per-star-entry moments in FP64;
//   3. combine_kernel (FP64, one warp per field vertex and frequency) sums the star entries into
//      the per-neighbour-slot blocks (G, H) or per-vertex tensors (B_trans, B_angular) of the side
//      buffers S that the regular kernels' epilogues add.
// Every sum runs in a fixed order: results are bitwise reproducible.
#include <algorithm>

#include "sod_dd.cuh"
#include "sod_dd_fast.cuh"
#include "sod_geom.cuh"
#include "sod_internal.h"

namespace sod {
namespace {

constexpr int KM_G = 1 << SOD_G, KM_H = 1 << SOD_H, KM_BT = 1 << SOD_B_TRANS, KM_BA = 1 << SOD_B_ANGULAR;
constexpr int POLAR_FIELDS = 9, GUIG_FIELDS = 8, GUIG_COMPS = 27;
constexpr int SING_THREADS = 128;

// 1-D Gauss-Legendre nodes and weights on [-1, 1] of the singular rule's order
struct GLRule {
    double x[5], w[5];
};

// ---- 1. frequency-independent geometry (FP64) ---------------------------------------------------
struct GeomArgs {
    int nstar, sorder, ssub;
    const double *V, *N;
    const int *F, *star_face, *star_corner;
    float2 *polar, *guig;
    double *guig_sub;
};

__device__ __forceinline__ void put(float2 *tab, int nfield, int nstar, int p, int field, int e, double v) {
    const dd d = dd_from(v);
    tab[((size_t)p * nfield + field) * nstar + e] = make_float2(d.hi, d.lo);
}

__global__ void __launch_bounds__(128) sing_geom_kernel(GeomArgs a, const __grid_constant__ GLRule gl) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.nstar) return;
    const int f = a.star_face[e], sc = a.star_corner[e];
    const int j0 = a.F[3 * f + sc], j1 = a.F[3 * f + (sc + 1) % 3], j2 = a.F[3 * f + (sc + 2) % 3];
    const double3 y1 = ld3(a.V, j0), y2 = ld3(a.V, j1), y3 = ld3(a.V, j2);
    const double3 n = ld3(a.N, f);
    const double nn[3] = {n.x, n.y, n.z};
    const int nq = a.sorder * a.ssub;
    // polar rule about y1 (theta in [0, alpha], r in [0, a / cos(theta - beta)])
    const Polar g = polar_setup(y1, y2, y3);
    for (int pidx = 0; pidx < nq * nq; pidx++) {
        const int ti = pidx / nq, ri = pidx % nq;
        const int ts = ti / a.sorder, tq = ti % a.sorder, rs = ri / a.sorder, rq = ri % a.sorder;
        const double ta = g.alpha * ts / a.ssub, tb = g.alpha * (ts + 1) / a.ssub;
        const double th = (tb - ta) * gl.x[tq] / 2. + (ta + tb) / 2.;
        double st, ct;
        sincos(th, &st, &ct);
        const double3 rh = g.xh * ct + g.yh * st;
        const double rmax = g.a / cos(th - g.beta);
        const double ra = rmax * rs / a.ssub, rb = rmax * (rs + 1) / a.ssub;
        const double r = (rb - ra) * gl.x[rq] / 2. + (ra + rb) / 2.;
        const double w = gl.w[tq] * (tb - ta) / 2. * gl.w[rq] * (rb - ra) / 2.;
        double L[3];
        bary_clamped(y1 + rh * r, y1, y2, y3, L);
        const double v[POLAR_FIELDS] = {r, rh.x, rh.y, rh.z, dot3(rh, n), w, w * L[0], w * L[1], w * L[2]};
        for (int k = 0; k < POLAR_FIELDS; k++) put(a.polar, POLAR_FIELDS, a.nstar, pidx, k, e, v[k]);
    }
    // Guiggiani rule on the unit right triangle mapped to (y1, y2, y3)
    const double3 v1 = y2 - y1, v2 = y3 - y1;
    const double J = norm3(cross3(v1, v2));
    const double tmax = CUDART_PI / 2.;
    double sub[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int pidx = 0; pidx < nq * nq; pidx++) {
        const int ti = pidx / nq, ri = pidx % nq;
        const int ts = ti / a.sorder, tq = ti % a.sorder, rs = ri / a.sorder, rq = ri % a.sorder;
        const double ta = tmax * ts / a.ssub, tb = tmax * (ts + 1) / a.ssub;
        const double th = (tb - ta) * gl.x[tq] / 2. + (ta + tb) / 2.;
        const double wt = gl.w[tq] * (tb - ta) / 2.;
        double st, ct;
        sincos(th, &st, &ct);
        const double3 Av = v1 * ct + v2 * st;
        const double A = norm3(Av);
        const double3 Ah = nrmz(Av);
        const double ah[3] = {Ah.x, Ah.y, Ah.z};
        const double rho_bar = 1. / (cos(th - CUDART_PI / 4.) * sqrt(2.));
        const double ra = rho_bar * rs / a.ssub, rb = rho_bar * (rs + 1) / a.ssub;
        const double rho = (rb - ra) * gl.x[rq] / 2. + (ra + rb) / 2.;
        const double w = wt * gl.w[rq] * (rb - ra) / 2.;
        const double L[3] = {1. - rho * (ct + st), rho * ct, rho * st};
        const double3 rv = Av * rho;
        const double r = norm3(rv);
        const double3 rh = nrmz(rv);
        const double wr = w * J * rho / (r * r);
        const double v[GUIG_FIELDS] = {r, rh.x, rh.y, rh.z, dot3(rh, n), wr * L[0], wr * L[1], wr * L[2]};
        for (int k = 0; k < GUIG_FIELDS; k++) put(a.guig, GUIG_FIELDS, a.nstar, pidx, k, e, v[k]);
        // subtracted 1/rho singularity and its log-term (corner 0, real part), times kappa / 4 pi later
        const double coef = -w / rho + (ri == 0 ? wt * log(rho_bar * A) : 0.0);
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) sub[3 * p + q] += coef * (ah[p] * nn[q] - ah[q] * nn[p]) / (A * A) * J;
    }
    for (int k = 0; k < 9; k++) a.guig_sub[(size_t)k * a.nstar + e] = sub[k];
}

// ---- 2. per-frequency evaluation in double-float ------------------------------------------------
struct KDD {
    cdd sc1, sc2, is;  // s / c1, s / c2, 1 / s
    dd ic1, ic2, ic1s, ic2s, six_c2s, inv4pirho, inv4pi, k4m1, k2, k1m2, k12;
};
__device__ __forceinline__ KDD make_kdd(const KConst<double> &k) {
    KDD o;
    o.sc1 = cdd{dd_from(k.sr * k.ic1), dd_from(k.si * k.ic1)};
    o.sc2 = cdd{dd_from(k.sr * k.ic2), dd_from(k.si * k.ic2)};
    o.is = cdd{dd_from(k.isr), dd_from(k.isi)};
    o.ic1 = dd_from(k.ic1), o.ic2 = dd_from(k.ic2), o.ic1s = dd_from(k.ic1s), o.ic2s = dd_from(k.ic2s);
    o.six_c2s = dd_from(k.six_c2s), o.inv4pirho = dd_from(k.inv4pirho), o.inv4pi = dd_from(k.inv4pi);
    o.k4m1 = dd_from(4.0 * k.kappa - 1.0), o.k2 = dd_from(2.0 * k.kappa), o.k1m2 = dd_from(1.0 - 2.0 * k.kappa);
    o.k12 = dd_from(12.0 * k.kappa);
    return o;
}

struct RadialDD {
    cdd z1, z2, e1, e2, psi2, Y;
};
// e^-z with the exponential and sine / cosine tables in shared memory (sod_dd_fast.cuh): the
// constant-memory tables are read with lane-varying indices, which the constant cache serialises
__device__ __forceinline__ RadialDD radial_dd(dd r, const KDD &k, const DdTabs *tb) {
    RadialDD t;
    t.z1 = k.sc1 * r;
    t.z2 = k.sc2 * r;
    t.e1 = cdd_exp_neg_tab(t.z1, tb);
    t.e2 = cdd_exp_neg_tab(t.z2, tb);
    const cdd psi1 = cdd_psi(t.z1, t.e1);
    t.psi2 = cdd_psi(t.z2, t.e2);
    t.Y = psi1 * k.ic1s - t.psi2 * k.ic2s;
    return t;
}

__device__ __forceinline__ dd ldd(const float2 *p) {
    const float2 v = __ldg(p);
    return dd{v.x, v.y};
}
__device__ __forceinline__ cdd cdd_zero() { return cdd{dd{0.f, 0.f}, dd{0.f, 0.f}}; }

template <int MASK> struct PolarLayout {
    static constexpr bool DG = (MASK & KM_G) != 0, DT = (MASK & KM_BT) != 0, DA = (MASK & KM_BA) != 0;
    static constexpr int NG = DG ? 18 : 0, NT = DT ? 4 : 0, NA = DA ? 9 : 0;
    static constexpr int OT = NG, OA = NG + NT, N = NG + NT + NA;
};

// G: 3 corners x 6 symmetric components of r u; B_trans moments (sum w sym rh_p, sum w dia rh.n);
// B_angular moments (sum w A rh_p rh_k, sum w A, sum w Bq, sum w Cq) -- all times the face's
// polar weights, as in the reference's polar rule with the FP64 kernels of sod_device.cuh.
template <int MASK>
__device__ __forceinline__ void polar_dd_body(const float2 *__restrict__ tab, int nstar, int nq2, int e,
                                              const KDD &k, double2 *__restrict__ R, const DdTabs *tb) {
    using Ly = PolarLayout<MASK>;
    cdd acc[Ly::N];
#pragma unroll
    for (int c = 0; c < Ly::N; c++) acc[c] = cdd_zero();
    for (int p = 0; p < nq2; p++) {
        const float2 *t = tab + (size_t)p * POLAR_FIELDS * nstar + e;
        const dd r = ldd(t), rh[3] = {ldd(t + nstar), ldd(t + 2 * nstar), ldd(t + 3 * nstar)};
        const dd rn = ldd(t + 4 * (size_t)nstar), w = ldd(t + 5 * (size_t)nstar);
        const RadialDD T = radial_dd(r, k, tb);
        if (Ly::DG) {
            const dd wl[3] = {ldd(t + 6 * (size_t)nstar), ldd(t + 7 * (size_t)nstar), ldd(t + 8 * (size_t)nstar)};
            const cdd B = T.e1 * k.ic1s - T.e2 * k.ic2s;
            const cdd al = (T.Y * 3.0f + B) * k.inv4pirho;
            const cdd be = (T.e2 * k.ic2s - T.Y) * k.inv4pirho;
#pragma unroll
            for (int p2 = 0; p2 < 3; p2++)
#pragma unroll
                for (int q2 = p2; q2 < 3; q2++) {
                    cdd v = al * (rh[p2] * rh[q2]);
                    if (p2 == q2) v = v + be;
#pragma unroll
                    for (int c = 0; c < 3; c++) cs_fma_acc(acc[c * 6 + sym_index(p2, q2)], v, wl[c]);
                }
        }
        if (Ly::DT || Ly::DA) {
            const dd pr = k.inv4pi * r;
            if (Ly::DT) {
                const cdd ws = T.Y * (pr * 0.5f) * w;
                const cdd di = T.psi2 * (k.ic2s * pr);
#pragma unroll
                for (int p2 = 0; p2 < 3; p2++) cs_fma_acc(acc[Ly::OT + p2], ws, rh[p2]);
                cs_fma_acc(acc[Ly::OT + 3], di, w * rn);
            }
            if (Ly::DA) {
                const cdd wA = T.Y * (r * pr * 0.5f) * w;
                const cdd Bq = (T.e2 * k.ic2 - T.e1 * k.ic1) * k.is * (pr * 0.5f);
                const cdd Cq = T.e2 * k.is * (k.ic2 * pr);
#pragma unroll
                for (int p2 = 0; p2 < 3; p2++)
#pragma unroll
                    for (int q2 = p2; q2 < 3; q2++) cs_fma_acc(acc[Ly::OA + sym_index(p2, q2)], wA, rh[p2] * rh[q2]);
                sd_acc(acc[Ly::OA + 6].x, wA.x);
                sd_acc(acc[Ly::OA + 6].y, wA.y);
                cs_fma_acc(acc[Ly::OA + 7], Bq, w);
                cs_fma_acc(acc[Ly::OA + 8], Cq, w);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < Ly::N; c++) R[(size_t)c * nstar + e] = make_double2(dd_to(acc[c].x), dd_to(acc[c].y));
}

// H: 3 corners x 9 components of the traction kernel times the Guiggiani weights (the CPV
// subtraction is frequency-independent and added by the combine kernel).  Scaled by 1/(4 pi) there.
__device__ __forceinline__ void guig_dd_body(const float2 *__restrict__ tab, int nstar, int nq2, int e,
                                             const double *__restrict__ N, int f, const KDD &k,
                                             double2 *__restrict__ R, const DdTabs *tb) {
    cdd acc[GUIG_COMPS];
#pragma unroll
    for (int c = 0; c < GUIG_COMPS; c++) acc[c] = cdd_zero();
    const dd nn[3] = {dd_from(N[3 * f]), dd_from(N[3 * f + 1]), dd_from(N[3 * f + 2])};
    for (int p = 0; p < nq2; p++) {
        const float2 *t = tab + (size_t)p * GUIG_FIELDS * nstar + e;
        const dd r = ldd(t), rh[3] = {ldd(t + nstar), ldd(t + 2 * nstar), ldd(t + 3 * nstar)};
        const dd rn = ldd(t + 4 * (size_t)nstar);
        const dd wc[3] = {ldd(t + 5 * (size_t)nstar), ldd(t + 6 * (size_t)nstar), ldd(t + 7 * (size_t)nstar)};
        const RadialDD T = radial_dd(r, k, tb);
        const cdd Yc = T.Y * k.six_c2s;
        const cdd z1e1 = T.z1 * T.e1, z2e2 = T.z2 * T.e2;
        const cdd ca = Yc + T.e1 * k.k4m1 - T.e2 * 2.0f - z1e1 * k.k1m2;
        const cdd cb = Yc + T.e1 * k.k2 - T.e2 * 3.0f - z2e2;
        const cdd cdv = Yc * (-5.0f) - T.e1 * k.k12 + T.e2 * 12.0f - z1e1 * k.k2 + z2e2 * 2.0f;
        const cdd cbr = cb * rn, cdr = cdv * rn;
#pragma unroll
        for (int p2 = 0; p2 < 3; p2++)
#pragma unroll
            for (int q2 = 0; q2 < 3; q2++) {
                cdd v = ca * (rh[p2] * nn[q2]) + cb * (nn[p2] * rh[q2]) + cdr * (rh[p2] * rh[q2]);
                if (p2 == q2) v = v + cbr;
#pragma unroll
                for (int c = 0; c < 3; c++) cs_fma_acc(acc[c * 9 + 3 * p2 + q2], v, wc[c]);
            }
    }
#pragma unroll
    for (int c = 0; c < GUIG_COMPS; c++) R[(size_t)c * nstar + e] = make_double2(dd_to(acc[c].x), dd_to(acc[c].y));
}

// ---- 3. per-vertex combination (FP64) -----------------------------------------------------------
struct CombineObj {
    int nV, nstar;
    const int *star_off, *star_face, *star_slot, *nbr_off;
    const double *N;
    const double2 *Rp, *Rg;  // this frequency's results: [comp][nstar]
    const double *guig_sub;  // [9][nstar]
    double kc;               // kappa / (4 pi)
    double inv4pi;
    cd *S[4];                // this frequency's side buffers
};
// CombineObj of frequency fq from frequency 0's pointers
__device__ __forceinline__ CombineObj at_frequency(const CombineObj &a, int fq, long long rp_fstride,
                                                   long long rg_fstride, const long long *s_fstride,
                                                   const KConst<double> &k) {
    CombineObj b = a;
    if (a.Rp) b.Rp = a.Rp + (size_t)fq * rp_fstride;
    if (a.Rg) b.Rg = a.Rg + (size_t)fq * rg_fstride;
    for (int kd = 0; kd < 4; kd++)
        if (a.S[kd]) b.S[kd] = a.S[kd] + (size_t)fq * s_fstride[kd];
    b.kc = k.inv4pi * k.kappa;
    b.inv4pi = k.inv4pi;
    return b;
}

template <int MASK>
__device__ __forceinline__ void combine_body(const CombineObj &a, int i, int lane) {
    using Ly = PolarLayout<MASK & (KM_G | KM_BT | KM_BA)>;
    const int s0 = a.star_off[i], s1 = a.star_off[i + 1];
    const int n0 = a.nbr_off[i], nsl = a.nbr_off[i + 1] - n0;
    if (MASK & (KM_G | KM_H)) {
        for (int el = lane; el < nsl * 9; el += 32) {
            const int sl = n0 + el / 9, pq = el % 9, p = pq / 3, q = pq % 3;
            double2 sg = make_double2(0., 0.), sh = make_double2(0., 0.);
            for (int e = s0; e < s1; e++)
                for (int c = 0; c < 3; c++) {
                    if (a.star_slot[3 * e + c] != sl) continue;
                    if (MASK & KM_G) {
                        const double2 v = a.Rp[(size_t)(c * 6 + sym_index(p, q)) * a.nstar + e];
                        sg.x += v.x, sg.y += v.y;
                    }
                    if (MASK & KM_H) {
                        const double2 v = a.Rg[(size_t)(c * 9 + pq) * a.nstar + e];
                        sh.x += v.x * a.inv4pi, sh.y += v.y * a.inv4pi;
                        if (c == 0) sh.x += a.kc * a.guig_sub[(size_t)pq * a.nstar + e];
                    }
                }
            if (MASK & KM_G) a.S[SOD_G][(size_t)sl * 9 + pq] = cd{sg.x, sg.y};
            if (MASK & KM_H) a.S[SOD_H][(size_t)sl * 9 + pq] = cd{sh.x, sh.y};
        }
    }
    if (MASK & KM_BT) {
        for (int el = lane; el < 9; el += 32) {
            const int p = el / 3, q = el % 3;
            double2 s = make_double2(0., 0.);
            for (int e = s0; e < s1; e++) {
                const int f = a.star_face[e];
                const double np = a.N[3 * f + p], nq = a.N[3 * f + q];
                const double2 mp = a.Rp[(size_t)(Ly::OT + p) * a.nstar + e];
                const double2 mq = a.Rp[(size_t)(Ly::OT + q) * a.nstar + e];
                s.x += mp.x * nq + mq.x * np;
                s.y += mp.y * nq + mq.y * np;
                if (p == q) {
                    const double2 md = a.Rp[(size_t)(Ly::OT + 3) * a.nstar + e];
                    s.x += md.x, s.y += md.y;
                }
            }
            a.S[SOD_B_TRANS][(size_t)i * 9 + el] = cd{s.x, s.y};
        }
    }
    if (MASK & KM_BA) {
        for (int el = lane; el < 27; el += 32) {
            const int p = el / 9, q = (el / 3) % 3, kk = el % 3;
            double2 s = make_double2(0., 0.);
            for (int e = s0; e < s1; e++) {
                const int f = a.star_face[e];
                const double nv[3] = {a.N[3 * f], a.N[3 * f + 1], a.N[3 * f + 2]};
                const double2 m_pk = a.Rp[(size_t)(Ly::OA + sym_index(p, kk)) * a.nstar + e];
                const double2 m_qk = a.Rp[(size_t)(Ly::OA + sym_index(q, kk)) * a.nstar + e];
                const double2 m0 = a.Rp[(size_t)(Ly::OA + 6) * a.nstar + e];
                const double2 mb = a.Rp[(size_t)(Ly::OA + 7) * a.nstar + e];
                const double2 mc = a.Rp[(size_t)(Ly::OA + 8) * a.nstar + e];
                const double t2 = (q == kk ? nv[p] : 0.0) + (p == kk ? nv[q] : 0.0);
                s.x += m_pk.x * nv[q] + m_qk.x * nv[p] + (m0.x + mb.x) * t2;
                s.y += m_pk.y * nv[q] + m_qk.y * nv[p] + (m0.y + mb.y) * t2;
                if (p == q) s.x += mc.x * nv[kk], s.y += mc.y * nv[kk];
            }
            a.S[SOD_B_ANGULAR][(size_t)i * 27 + el] = cd{s.x, s.y};
        }
    }
}

// ---- per-object kernels ---------------------------------------------------------------------------
struct FreqD {
    int n;
    KConst<double> k[MAX_FREQ_PER_LAUNCH];
};

template <int MASK>
__global__ void __launch_bounds__(SING_THREADS) polar_dd_kernel(const float2 *__restrict__ tab, int nstar, int nq2,
                                                                double2 *__restrict__ R,
                                                                const __grid_constant__ FreqD fd) {
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nstar) return;
    const KDD k = make_kdd(fd.k[blockIdx.y]);
    polar_dd_body<MASK>(tab, nstar, nq2, e, k, R + (size_t)blockIdx.y * PolarLayout<MASK>::N * nstar, &tb);
}

__global__ void __launch_bounds__(SING_THREADS) guig_dd_kernel(const float2 *__restrict__ tab, int nstar, int nq2,
                                                               const int *__restrict__ star_face,
                                                               const double *__restrict__ N, double2 *__restrict__ R,
                                                               const __grid_constant__ FreqD fd) {
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nstar) return;
    const KDD k = make_kdd(fd.k[blockIdx.y]);
    guig_dd_body(tab, nstar, nq2, e, N, star_face[e], k, R + (size_t)blockIdx.y * GUIG_COMPS * nstar, &tb);
}

// one warp per (vertex, frequency); `a` holds frequency 0's pointers
struct CombineStrides {
    long long rp, rg, s[4];
};
template <int MASK>
__global__ void __launch_bounds__(128) combine_kernel(CombineObj a, CombineStrides st, int nf,
                                                      const __grid_constant__ FreqD fd) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= a.nV * nf) return;
    const int fq = w / a.nV, i = w % a.nV;
    combine_body<MASK>(at_frequency(a, fq, st.rp, st.rg, st.s, fd.k[fq]), i, lane);
}

// ---- batched kernels: one CTA per work item --------------------------------------------------------
//   polar / Guiggiani items (object, frequency, first star entry), SING_THREADS star entries each;
//   combine items (object, frequency, first vertex), 4 vertices (one per warp) each.
template <int PM>
__global__ void __launch_bounds__(SING_THREADS) batch_polar_dd_kernel(const SingBatchObj *__restrict__ objs,
                                                                      const int4 *__restrict__ items,
                                                                      const KConst<double> *__restrict__ kcd) {
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    __syncthreads();
    const int4 w = items[blockIdx.x];
    const SingBatchObj &o = objs[w.x];
    const int e = w.z + threadIdx.x;
    if (e >= o.nstar) return;
    const KDD k = make_kdd(kcd[o.kc_off + w.y]);
    polar_dd_body<PM>(o.polar, o.nstar, o.nq2, e, k, o.Rp + (size_t)w.y * PolarLayout<PM>::N * o.nstar, &tb);
}

__global__ void __launch_bounds__(SING_THREADS) batch_guig_dd_kernel(const SingBatchObj *__restrict__ objs,
                                                                     const int4 *__restrict__ items,
                                                                     const KConst<double> *__restrict__ kcd) {
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    __syncthreads();
    const int4 w = items[blockIdx.x];
    const SingBatchObj &o = objs[w.x];
    const int e = w.z + threadIdx.x;
    if (e >= o.nstar) return;
    const KDD k = make_kdd(kcd[o.kc_off + w.y]);
    guig_dd_body(o.guig, o.nstar, o.nq2, e, o.N, o.star_face[e], k, o.Rg + (size_t)w.y * GUIG_COMPS * o.nstar, &tb);
}

template <int MASK>
__global__ void __launch_bounds__(128) batch_combine_kernel(const SingBatchObj *__restrict__ objs,
                                                            const int4 *__restrict__ items,
                                                            const KConst<double> *__restrict__ kcd) {
    const int4 w = items[blockIdx.x];
    const SingBatchObj &o = objs[w.x];
    const int i = w.z + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= o.nV) return;
    CombineObj a{};
    a.nV = o.nV;
    a.nstar = o.nstar;
    a.star_off = o.star_off;
    a.star_face = o.star_face;
    a.star_slot = o.star_slot;
    a.nbr_off = o.nbr_off;
    a.N = o.N;
    a.Rp = o.Rp;
    a.Rg = o.Rg;
    a.guig_sub = o.guig_sub;
    for (int kd = 0; kd < 4; kd++) a.S[kd] = (MASK & (1 << kd)) ? o.S[kd] : nullptr;
    // MASK's polar kinds are the batch's full polar kind set, so the result layout matches the producer
    const long long rpf = (long long)PolarLayout<MASK & (KM_G | KM_BT | KM_BA)>::N * o.nstar;
    combine_body<MASK>(at_frequency(a, w.y, rpf, (long long)GUIG_COMPS * o.nstar, o.S_fstride, kcd[o.kc_off + w.y]),
                       i, lane);
}

// ---- elastostatic (Kelvin) singular integrals, FP64 from the same geometry tables ---------------
//   G: r u* = a_g ((3 - 4 nu) d_pq + rh_p rh_q) / a_g'..., i.e. alpha rh_p rh_q + beta d_pq (polar rule);
//   H: p* in the traction-kernel structure with constant coefficients (Guiggiani rule), the 1/(4 pi)
//      and the CPV subtraction (times kappa / 4 pi = (1 - 2 nu) / (8 pi (1 - nu))) added by the combine.
struct StaticSing {
    double g_alpha, g_beta;  // G (r u form)
    double ha, hb, hd;       // H (times 1 / (4 pi r^2) from the weights and the combine)
};
__device__ __forceinline__ double dlo(const float2 *p) {
    const float2 v = __ldg(p);
    return (double)v.x + (double)v.y;
}
__global__ void __launch_bounds__(128) static_sing_kernel(const float2 *__restrict__ polar,
                                                          const float2 *__restrict__ guig, int nstar, int nq2,
                                                          const int *__restrict__ star_face,
                                                          const double *__restrict__ N, int do_g, int do_h,
                                                          StaticSing c, double2 *__restrict__ Rp,
                                                          double2 *__restrict__ Rg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nstar) return;
    if (do_g) {
        double acc[18] = {};
        for (int p = 0; p < nq2; p++) {
            const float2 *t = polar + (size_t)p * POLAR_FIELDS * nstar + e;
            const double rh[3] = {dlo(t + nstar), dlo(t + 2 * (size_t)nstar), dlo(t + 3 * (size_t)nstar)};
            const double wl[3] = {dlo(t + 6 * (size_t)nstar), dlo(t + 7 * (size_t)nstar), dlo(t + 8 * (size_t)nstar)};
            for (int p2 = 0; p2 < 3; p2++)
                for (int q2 = p2; q2 < 3; q2++) {
                    const double v = c.g_alpha * rh[p2] * rh[q2] + (p2 == q2 ? c.g_beta : 0.0);
                    for (int k = 0; k < 3; k++) acc[k * 6 + sym_index(p2, q2)] += v * wl[k];
                }
        }
        for (int k = 0; k < 18; k++) Rp[(size_t)k * nstar + e] = make_double2(acc[k], 0.0);
    }
    if (do_h) {
        const int f = star_face[e];
        const double nn[3] = {N[3 * f], N[3 * f + 1], N[3 * f + 2]};
        double acc[27] = {};
        for (int p = 0; p < nq2; p++) {
            const float2 *t = guig + (size_t)p * GUIG_FIELDS * nstar + e;
            const double rh[3] = {dlo(t + nstar), dlo(t + 2 * (size_t)nstar), dlo(t + 3 * (size_t)nstar)};
            const double rn = dlo(t + 4 * (size_t)nstar);
            const double wc[3] = {dlo(t + 5 * (size_t)nstar), dlo(t + 6 * (size_t)nstar), dlo(t + 7 * (size_t)nstar)};
            for (int p2 = 0; p2 < 3; p2++)
                for (int q2 = 0; q2 < 3; q2++) {
                    double v = c.ha * rh[p2] * nn[q2] + c.hb * nn[p2] * rh[q2] + c.hd * rn * rh[p2] * rh[q2];
                    if (p2 == q2) v += c.hb * rn;
                    for (int k = 0; k < 3; k++) acc[k * 9 + 3 * p2 + q2] += v * wc[k];
                }
        }
        for (int k = 0; k < 27; k++) Rg[(size_t)k * nstar + e] = make_double2(acc[k], 0.0);
    }
}

}  // namespace

// ---- mesh cache of the geometry tables -------------------------------------------------------
}  // namespace sod

int sod_mesh::sing_geom_for(int sorder, int ssub, cudaStream_t stream, const SingGeom **out) {
    using namespace sod;
    auto key = std::make_pair(sorder, ssub);
    auto it = sing_geom.find(key);
    if (it != sing_geom.end()) {
        *out = it->second.get();
        return SOD_OK;
    }
    SOD_REQUIRE(sorder >= 1 && sorder <= 5 && ssub >= 1 && ssub <= 8,
                "singular quadrature order must be 1..5, subdivision 1..8");
    auto g = std::make_unique<SingGeom>();
    const int nstar = star_off.back();
    const int nq = sorder * ssub;
    g->nq2 = nq * nq;
    SOD_TRY(g->polar.ensure(sizeof(float2) * (size_t)g->nq2 * POLAR_FIELDS * std::max(nstar, 1)));
    SOD_TRY(g->guig.ensure(sizeof(float2) * (size_t)g->nq2 * GUIG_FIELDS * std::max(nstar, 1)));
    SOD_TRY(g->guig_sub.ensure(sizeof(double) * 9 * (size_t)std::max(nstar, 1)));
    GLRule gl{};
    int n = 0;
    const double(*t)[2] = gl_rule_table(sorder, n);
    for (int q = 0; q < n; q++) gl.x[q] = t[q][0], gl.w[q] = t[q][1];
    GeomArgs a;
    a.nstar = nstar;
    a.sorder = sorder;
    a.ssub = ssub;
    a.V = dV.as<double>();
    a.N = dN.as<double>();
    a.F = dF.as<int>();
    a.star_face = dStarFace.as<int>();
    a.star_corner = dStarCorner.as<int>();
    a.polar = g->polar.as<float2>();
    a.guig = g->guig.as<float2>();
    a.guig_sub = g->guig_sub.as<double>();
    if (nstar > 0) {
        sing_geom_kernel<<<(nstar + 127) / 128, 128, 0, stream>>>(a, gl);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    *out = g.get();
    sing_geom.emplace(key, std::move(g));
    return SOD_OK;
}

namespace sod {

size_t sing_result_elems(int mask, int nstar, int nf, bool guiggiani) {
    if (guiggiani) return (mask & KM_H) ? (size_t)GUIG_COMPS * nstar * nf : 0;
    int n = 0;
    if (mask & KM_G) n += 18;
    if (mask & KM_BT) n += 4;
    if (mask & KM_BA) n += 9;
    return (size_t)n * nstar * nf;
}

template <int PM>
static void launch_polar(const float2 *tab, int nstar, int nq2, double2 *R, const FreqD &fd, cudaStream_t st) {
    const dim3 grid((nstar + SING_THREADS - 1) / SING_THREADS, fd.n);
    polar_dd_kernel<PM><<<grid, SING_THREADS, 0, st>>>(tab, nstar, nq2, R, fd);
}

template <int M>
static void launch_combine(const CombineObj &a, const CombineStrides &st, int nf, const FreqD &fd, cudaStream_t stream) {
    const long long warps = (long long)a.nV * nf;
    const int blocks = (int)((warps * 32 + 127) / 128);
    combine_kernel<M><<<blocks, 128, 0, stream>>>(a, st, nf, fd);
}

#define SOD_MASK_SWITCH(M, CALL)                 \
    switch (M) {                                 \
    case 1: CALL(1); break;                      \
    case 2: CALL(2); break;                      \
    case 3: CALL(3); break;                      \
    case 4: CALL(4); break;                      \
    case 5: CALL(5); break;                      \
    case 6: CALL(6); break;                      \
    case 7: CALL(7); break;                      \
    case 8: CALL(8); break;                      \
    case 9: CALL(9); break;                      \
    case 10: CALL(10); break;                    \
    case 11: CALL(11); break;                    \
    case 12: CALL(12); break;                    \
    case 13: CALL(13); break;                    \
    case 14: CALL(14); break;                    \
    case 15: CALL(15); break;                    \
    default: break;                              \
    }

#define SOD_POLAR_SWITCH(M, CALL) \
    switch (M) {                  \
    case 1: CALL(1); break;       \
    case 4: CALL(4); break;       \
    case 5: CALL(5); break;       \
    case 8: CALL(8); break;       \
    case 9: CALL(9); break;       \
    case 12: CALL(12); break;     \
    case 13: CALL(13); break;     \
    default: break;               \
    }

int launch_singular(sod_context *ctx, const sod_mesh *m, int mask, int sorder, int ssub, const KConst<double> *kc,
                    int nf, cd *const S[4], const long long S_fstride[4], cudaStream_t stream) {
    SOD_REQUIRE(nf >= 1 && nf <= MAX_FREQ_PER_LAUNCH, "singular pass: bad frequency chunk");
    const sod_mesh::SingGeom *g = nullptr;
    SOD_TRY(const_cast<sod_mesh *>(m)->sing_geom_for(sorder, ssub, stream, &g));
    const int nstar = m->star_off.back();
    if (nstar == 0) return SOD_OK;
    const int pm = mask & (KM_G | KM_BT | KM_BA);
    const size_t np = sing_result_elems(mask, nstar, nf, false), ng = sing_result_elems(mask, nstar, nf, true);
    SOD_TRY(ctx->sing_res.ensure(sizeof(double2) * (np + ng)));
    double2 *Rp = np ? ctx->sing_res.as<double2>() : nullptr;
    double2 *Rg = ng ? ctx->sing_res.as<double2>() + np : nullptr;
    FreqD fd;
    fd.n = nf;
    for (int l = 0; l < nf; l++) fd.k[l] = kc[l];
    if (pm) {
#define SOD_LP(PM) launch_polar<PM>(g->polar.as<float2>(), nstar, g->nq2, Rp, fd, stream)
        SOD_POLAR_SWITCH(pm, SOD_LP)
#undef SOD_LP
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    if (mask & KM_H) {
        const dim3 grid((nstar + SING_THREADS - 1) / SING_THREADS, nf);
        guig_dd_kernel<<<grid, SING_THREADS, 0, stream>>>(g->guig.as<float2>(), nstar, g->nq2, m->dStarFace.as<int>(),
                                                          m->dN.as<double>(), Rg, fd);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    CombineObj a{};
    a.nV = m->nV;
    a.nstar = nstar;
    a.star_off = m->dStarOff.as<int>();
    a.star_face = m->dStarFace.as<int>();
    a.star_slot = m->dStarSlot.as<int>();
    a.nbr_off = m->dNbrOff.as<int>();
    a.N = m->dN.as<double>();
    a.Rp = Rp;
    a.Rg = Rg;
    a.guig_sub = g->guig_sub.as<double>();
    for (int kd = 0; kd < 4; kd++) a.S[kd] = (mask & (1 << kd)) ? S[kd] : nullptr;
    CombineStrides st;
    st.rp = (long long)(np / nf);
    st.rg = (long long)(ng / nf);
    for (int kd = 0; kd < 4; kd++) st.s[kd] = S_fstride[kd];
#define SOD_LC(M) launch_combine<M>(a, st, nf, fd, stream)
    SOD_MASK_SWITCH(mask, SOD_LC)
#undef SOD_LC
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

int sing_batch_launch(sod_context *ctx, int which, int mask, const SingBatchObj *objs, const int4 *items, int nitems,
                      const KConst<double> *kcd, cudaStream_t stream) {
    if (nitems <= 0) return SOD_OK;
    const int pm = mask & (KM_G | KM_BT | KM_BA);
    switch (which) {
    case 0:
#define SOD_BP(PM) batch_polar_dd_kernel<PM><<<nitems, SING_THREADS, 0, stream>>>(objs, items, kcd)
        SOD_POLAR_SWITCH(pm, SOD_BP)
#undef SOD_BP
        break;
    case 1: batch_guig_dd_kernel<<<nitems, SING_THREADS, 0, stream>>>(objs, items, kcd); break;
    default:
#define SOD_BC(M) batch_combine_kernel<M><<<nitems, 128, 0, stream>>>(objs, items, kcd)
        SOD_MASK_SWITCH(mask, SOD_BC)
#undef SOD_BC
        break;
    }
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// Singular blocks of the elastostatic Kelvin kernels into S[SOD_G] / S[SOD_H] (per-slot 3x3 blocks,
// complex layout with zero imaginary parts), FP64.
int launch_static_singular(sod_context *ctx, const sod_mesh *m, int mask, int sorder, int ssub, double nu, double mu,
                           cd *const S[4], cudaStream_t stream) {
    const sod_mesh::SingGeom *g = nullptr;
    SOD_TRY(const_cast<sod_mesh *>(m)->sing_geom_for(sorder, ssub, stream, &g));
    const int nstar = m->star_off.back();
    if (nstar == 0) return SOD_OK;
    const bool dg = (mask & KM_G) != 0, dh = (mask & KM_H) != 0;
    const size_t np = dg ? (size_t)18 * nstar : 0, ng = dh ? (size_t)GUIG_COMPS * nstar : 0;
    SOD_TRY(ctx->sing_res.ensure(sizeof(double2) * std::max<size_t>(np + ng, 1)));
    double2 *Rp = dg ? ctx->sing_res.as<double2>() : nullptr;
    double2 *Rg = dh ? ctx->sing_res.as<double2>() + np : nullptr;
    StaticSing c;
    c.g_alpha = 1.0 / (16.0 * CUDART_PI * (1.0 - nu) * mu);
    c.g_beta = (3.0 - 4.0 * nu) * c.g_alpha;
    const double C = (1.0 - 2.0 * nu) / (8.0 * CUDART_PI * (1.0 - nu));
    c.ha = 4.0 * CUDART_PI * C;
    c.hb = -4.0 * CUDART_PI * C;
    c.hd = -12.0 * CUDART_PI * C / (1.0 - 2.0 * nu);
    static_sing_kernel<<<(nstar + 127) / 128, 128, 0, stream>>>(g->polar.as<float2>(), g->guig.as<float2>(), nstar,
                                                               g->nq2, m->dStarFace.as<int>(), m->dN.as<double>(),
                                                               dg, dh, c, Rp, Rg);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    CombineObj a{};
    a.nV = m->nV;
    a.nstar = nstar;
    a.star_off = m->dStarOff.as<int>();
    a.star_face = m->dStarFace.as<int>();
    a.star_slot = m->dStarSlot.as<int>();
    a.nbr_off = m->dNbrOff.as<int>();
    a.N = m->dN.as<double>();
    a.Rp = Rp;
    a.Rg = Rg;
    a.guig_sub = g->guig_sub.as<double>();
    for (int kd = 0; kd < 4; kd++) a.S[kd] = (mask & (1 << kd)) ? S[kd] : nullptr;
    FreqD fd;
    fd.n = 1;
    fd.k[0] = KConst<double>{};
    fd.k[0].inv4pi = 1.0 / (4.0 * CUDART_PI);
    fd.k[0].kappa = (1.0 - 2.0 * nu) / (2.0 * (1.0 - nu));  // kappa / (4 pi) = C
    CombineStrides st{};
    st.rp = (long long)np;
    st.rg = (long long)ng;
    const int sm = mask & (KM_G | KM_H);
    if (sm == KM_G)
        launch_combine<KM_G>(a, st, 1, fd, stream);
    else if (sm == KM_H)
        launch_combine<KM_H>(a, st, 1, fd, stream);
    else
        launch_combine<KM_G | KM_H>(a, st, 1, fd, stream);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

}  // namespace sod
