// sod_device.cuh -- device math shared by the CQBEM kernels (sm_103a).
//
// Kernel functions are evaluated in an algebraically exact rearrangement of the reference's
// formulas (src/elastodynamics_cqbem_{G,H,B_trans,B_angular}_collocation.cu) that removes the
// catastrophic cancellation at small |s| r / c:
//   psi(z) = ((1 + z) e^-z - 1) / z^2          (series below |z| = tau, closed form above)
//   Y      = psi(z1)/c1^2 - psi(z2)/c2^2,     z_a = s r / c_a,  e_a = e^-z_a,  kappa = c2^2/c1^2
//   G : u_pq  = alpha rh_p rh_q + beta d_pq,   alpha = (3Y + e1/c1^2 - e2/c2^2)/(4 pi rho r),
//                                              beta  = (e2/c2^2 - Y)/(4 pi rho r)
//   H : p_pq  = [a rh_p n_q + b (n_p rh_q + rn d_pq) + d rn rh_p rh_q] / (4 pi r^2), rn = rh.n
//       a = 6 c2^2 Y + (4 kappa - 1) e1 - 2 e2 - (1 - 2 kappa) z1 e1
//       b = 6 c2^2 Y + 2 kappa e1 - 3 e2 - z2 e2
//       d = -30 c2^2 Y - 12 kappa e1 + 12 e2 - 2 kappa z1 e1 + 2 z2 e2
//   B_trans  : b_pq  = [ (Y/2)(rh_p n_q + rh_q n_p) + psi(z2)/c2^2 rn d_pq ] / (4 pi)
//   B_angular: b_pqk = [ (r Y/2)(rh_p rh_k n_q + rh_q rh_k n_p + d_qk n_p + d_pk n_q)
//                        + (d_qk n_p + d_pk n_q)(e2/c2 - e1/c1)/(2 s) + d_pq n_k e2/(c2 s) ] / (4 pi)
// Each identity was checked against the literal formulas to 1e-36 (40-digit arithmetic).
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

namespace sod {

// ------------------------------------------------------------------------------------------
// small complex types
struct cf {
    float x, y;
};
struct cd {
    double x, y;
};
__device__ __forceinline__ cf mk(float a, float b) { return {a, b}; }
__device__ __forceinline__ cd mk(double a, double b) { return {a, b}; }
__device__ __forceinline__ cf operator+(cf a, cf b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cf operator-(cf a, cf b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cf operator*(cf a, cf b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cf operator*(cf a, float s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ cf operator*(float s, cf a) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ cd operator+(cd a, cd b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd operator-(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cd operator*(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd operator*(cd a, double s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ cd operator*(double s, cd a) { return {a.x * s, a.y * s}; }
template <class C, class R> __device__ __forceinline__ void cfma(C &acc, C a, R s) {
    acc.x = fma(a.x, s, acc.x);
    acc.y = fma(a.y, s, acc.y);
}
// FP32 complex times real, accumulated: one packed two-lane FMA (sm_100+), each lane an ordinary
// round-to-nearest fma, so the results are those of the two scalar fmas above
__device__ __forceinline__ void cfma(cf &acc, cf a, float s) {
    const float2 r = __ffma2_rn(make_float2(a.x, a.y), make_float2(s, s), make_float2(acc.x, acc.y));
    acc = {r.x, r.y};
}
// a * s and a * s + b for FP32 complex a, b and real s, as single packed instructions
__device__ __forceinline__ cf cmulr(cf a, float s) {
    const float2 r = __fmul2_rn(make_float2(a.x, a.y), make_float2(s, s));
    return {r.x, r.y};
}
__device__ __forceinline__ cf cfmar(cf a, float s, cf b) {
    const float2 r = __ffma2_rn(make_float2(a.x, a.y), make_float2(s, s), make_float2(b.x, b.y));
    return {r.x, r.y};
}
__device__ __forceinline__ cd crecip(cd a) {
    const double d = 1.0 / fma(a.x, a.x, a.y * a.y);
    return {a.x * d, -a.y * d};
}

// e^-z for complex z in FP32 on the SFU: Cody-Waite reduction of the phase to [-pi, pi] and of the
// exponent to [-1/2, 1/2] (three-term splits of 2 pi and log2 e), then MUFU sin/cos/ex2.  Phase
// error < 4e-7 rad, magnitude error < 3e-7 relative (checked against the FP64 oracle in the tests).
// The reduction integers come from the 1.5 * 2^23 rounding constant (an add on the FMA pipe instead
// of a round and a float-to-int conversion on the SFU pipe), and 2^n is added into the exponent
// field of 2^f; results below 2^-125 flush to zero.
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kRound23 = 12582912.0f;  // 1.5 * 2^23: x + kRound23 - kRound23 = round(x), |x| < 2^22
__device__ __forceinline__ cf cexp_neg(cf z) {
    // phase: y - k 2pi with 2pi = P1 + P2
    const float k = fmaf(z.y, 0.15915494309189535f, kRound23) - kRound23;
    float ph = fmaf(-k, 6.28318548202514648f, z.y);
    ph = fmaf(-k, -1.74845553e-7f, ph);
    float sn, cs;
    __sincosf(ph, &sn, &cs);
    // magnitude: e^-x = 2^(-x log2 e) = 2^n 2^f (n <= 0 here: Re z >= 0)
    const float nr = fmaf(-z.x, 1.44269504088896341f, kRound23);
    const int ni = __float_as_int(nr) - __float_as_int(kRound23);
    const float n = nr - kRound23;
    float f = fmaf(-z.x, 1.44269502162933350f, -n);
    f = fmaf(-z.x, 1.92596299e-8f, f);
    const float m = ni > -125 ? __int_as_float(__float_as_int(ex2_approx(f)) + ni * (1 << 23)) : 0.f;
    return {m * cs, -m * sn};
}
__device__ __forceinline__ cd cexp_neg(cd z) {
    double sn, cs;
    sincos(z.y, &sn, &cs);
    const double m = exp(-z.x);
    return {m * cs, -m * sn};
}

// psi(z) = ((1+z) e^-z - 1) / z^2 = -sum_{m>=0} (-1)^m (m+1) z^m / (m+2)!
// FP32: below |z| = 1 the 11-term series (truncation < 4e-9 relative) in Estrin's scheme (dependency
// depth 4 complex multiply-adds instead of Horner's 10); above it the FP32 radial terms below need no
// psi of their own.
__device__ __forceinline__ cf cfmac(cf a, cf b, cf c) {  // a b + c
    return {fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y))};
}
__device__ __forceinline__ cf psi_series(cf z) {
    // c_m = -(-1)^m (m+1)/(m+2)!, m = 0..10, paired as c_2j + c_2j+1 z
    const float c0 = -1.0f / 2.0f, c1 = 1.0f / 3.0f, c2 = -1.0f / 8.0f, c3 = 1.0f / 30.0f, c4 = -1.0f / 144.0f,
                c5 = 1.0f / 840.0f, c6 = -1.0f / 5760.0f, c7 = 1.0f / 45360.0f, c8 = -9.0f / 3628800.0f,
                c9 = 10.0f / 39916800.0f, c10 = -11.0f / 479001600.0f;
    const cf z2 = z * z, z4 = z2 * z2, z8 = z4 * z4;
    const cf p01 = {fmaf(c1, z.x, c0), c1 * z.y}, p23 = {fmaf(c3, z.x, c2), c3 * z.y};
    const cf p45 = {fmaf(c5, z.x, c4), c5 * z.y}, p67 = {fmaf(c7, z.x, c6), c7 * z.y};
    const cf p89 = {fmaf(c9, z.x, c8), c9 * z.y};
    const cf q0 = cfmac(z2, p23, p01), q1 = cfmac(z2, p67, p45);
    const cf q2 = {fmaf(c10, z2.x, p89.x), fmaf(c10, z2.y, p89.y)};
    return cfmac(z8, q2, cfmac(z4, q1, q0));
}
// FP64: the closed form loses about 2 eps / |z|^2, i.e. <= 2e-12 relative for |z| >= 0.01; below
// that a 7-term series (truncation < 1e-17 relative) is used.
__device__ __forceinline__ cd psi(cd z, cd ez) {
    const double az2 = z.x * z.x + z.y * z.y;
    if (az2 < 1e-4) {
        const double c[7] = {-1.0 / 2.0, 1.0 / 3.0, -1.0 / 8.0, 1.0 / 30.0, -1.0 / 144.0, 1.0 / 840.0, -1.0 / 5760.0};
        cd acc = {c[6], 0.0};
#pragma unroll
        for (int m = 5; m >= 0; m--) acc = acc * z + mk(c[m], 0.0);
        return acc;
    }
    const cd num = (mk(1.0, 0.0) + z) * ez - mk(1.0, 0.0);
    return num * crecip(z * z);
}

// ------------------------------------------------------------------------------------------
// per-frequency material constants
template <class R> struct KConst {
    R ic1, ic2;          // 1/c1, 1/c2
    R ic1s, ic2s;        // 1/c1^2, 1/c2^2
    R kappa;             // c2^2/c1^2
    R six_c2s;           // 6 c2^2
    R inv4pirho;         // 1/(4 pi rho)
    R inv4pi;            // 1/(4 pi)
    R sr, si;            // s
    R isr, isi;          // 1/s
    R sc1r, sc1i;        // s/c1
    R sc2r, sc2i;        // s/c2
    R is2r, is2i;        // 1/s^2
    R c2sq;              // c2^2
};

template <class R, class C> struct RadialTerms {
    C z1, z2, e1, e2, psi1, psi2, Y;
};

template <class R, class C>
__device__ __forceinline__ RadialTerms<R, C> radial(R r, const KConst<R> &k) {
    RadialTerms<R, C> t;
    t.z1 = mk(r * k.sc1r, r * k.sc1i);
    t.z2 = mk(r * k.sc2r, r * k.sc2i);
    t.e1 = cexp_neg(t.z1);
    t.e2 = cexp_neg(t.z2);
    t.psi1 = psi(t.z1, t.e1);
    t.psi2 = psi(t.z2, t.e2);
    t.Y = t.psi1 * k.ic1s - t.psi2 * k.ic2s;
    return t;
}

// G: u = alpha rh rh^T + beta I, times r (the "r u" form used by the polar rule when mul_r)
template <class R, class C>
__device__ __forceinline__ void g_coeffs(const RadialTerms<R, C> &t, const KConst<R> &k, R scale, C &alpha,
                                         C &beta) {
    const C B = t.e1 * k.ic1s - t.e2 * k.ic2s;
    const C Cc = t.e2 * k.ic2s;
    const R p = k.inv4pirho * scale;
    alpha = (t.Y * (R)3 + B) * p;
    beta = (Cc - t.Y) * p;
}

// H: p = [a rh n^T + b (n rh^T + rn I) + d rn rh rh^T] * scale / (4 pi)
template <class R, class C>
__device__ __forceinline__ void h_coeffs(const RadialTerms<R, C> &t, const KConst<R> &k, R scale, C &a, C &b,
                                         C &d) {
    const C Yc = t.Y * k.six_c2s;
    const C z1e1 = t.z1 * t.e1, z2e2 = t.z2 * t.e2;
    const R kp = k.kappa;
    a = Yc + t.e1 * ((R)4 * kp - (R)1) - t.e2 * (R)2 - z1e1 * ((R)1 - (R)2 * kp);
    b = Yc + t.e1 * ((R)2 * kp) - t.e2 * (R)3 - z2e2;
    d = Yc * (R)(-5) - t.e1 * ((R)12 * kp) + t.e2 * (R)12 - z1e1 * ((R)2 * kp) + z2e2 * (R)2;
    const R p = k.inv4pi * scale;
    a = a * p;
    b = b * p;
    d = d * p;
}

// FP32 overloads of the above with packed two-lane FMA / multiply chains (same algebra; each
// complex-times-real multiply-add is one instruction).  Since c1^2 z1^2 = c2^2 z2^2 = s^2 r^2,
//     Y = psi(z1)/c1^2 - psi(z2)/c2^2 = ((1 + z1) e1 - (1 + z2) e2) / (s^2 r^2)
// (the -1 of both psi cancel exactly), so above |z2| = 1 (|z1| >= |z2| c2/c1) Y takes no reciprocal
// and no psi at all; below, both psi come from the series.  psi2 itself (the B kinds, PSI2) is
// ((1 + z2) e2 - 1) c2^2 / (s^2 r^2) there.  rinv is the caller's 1/r: a relative error of it scales
// Y uniformly over the frequencies.
template <bool PSI2>
__device__ __forceinline__ RadialTerms<float, cf> radial(float r, float rinv, const KConst<float> &k) {
    RadialTerms<float, cf> t;
    t.z1 = mk(r * k.sc1r, r * k.sc1i);
    t.z2 = mk(r * k.sc2r, r * k.sc2i);
    t.e1 = cexp_neg(t.z1);
    t.e2 = cexp_neg(t.z2);
    if (t.z2.x * t.z2.x + t.z2.y * t.z2.y < 1.0f) {
        const cf psi1 = psi_series(t.z1);
        t.psi2 = psi_series(t.z2);
        t.Y = cfmar(t.psi2, -k.ic2s, cmulr(psi1, k.ic1s));
    } else {
        const float ri2 = rinv * rinv;
        const cf W = mk(k.is2r * ri2, k.is2i * ri2);
        const cf a1 = cfmac(t.z1, t.e1, t.e1), a2 = cfmac(t.z2, t.e2, t.e2);  // (1 + z) e
        t.Y = (a1 - a2) * W;
        if (PSI2) t.psi2 = cmulr((a2 - mk(1.0f, 0.0f)) * W, k.c2sq);
    }
    return t;
}
// The _unit forms leave out the common factor (1/(4 pi rho) for G, 1/(4 pi) for H, times `scale`),
// for callers that fold it into their quadrature weight.
__device__ __forceinline__ void g_coeffs_unit(const RadialTerms<float, cf> &t, const KConst<float> &k, cf &alpha,
                                              cf &beta) {
    const cf Cc = cmulr(t.e2, k.ic2s);
    const cf B = cfmar(t.e1, k.ic1s, cmulr(Cc, -1.0f));
    alpha = cfmar(t.Y, 3.0f, B);
    beta = cfmar(t.Y, -1.0f, Cc);
}
__device__ __forceinline__ void g_coeffs(const RadialTerms<float, cf> &t, const KConst<float> &k, float scale,
                                         cf &alpha, cf &beta) {
    g_coeffs_unit(t, k, alpha, beta);
    const float p = k.inv4pirho * scale;
    alpha = cmulr(alpha, p);
    beta = cmulr(beta, p);
}
__device__ __forceinline__ void h_coeffs_unit(const RadialTerms<float, cf> &t, const KConst<float> &k, cf &a, cf &b,
                                              cf &d) {
    const cf Yc = cmulr(t.Y, k.six_c2s);
    const cf z1e1 = t.z1 * t.e1, z2e2 = t.z2 * t.e2;
    const float kp = k.kappa;
    a = cfmar(z1e1, -(1.0f - 2.0f * kp), cfmar(t.e2, -2.0f, cfmar(t.e1, 4.0f * kp - 1.0f, Yc)));
    b = cfmar(z2e2, -1.0f, cfmar(t.e2, -3.0f, cfmar(t.e1, 2.0f * kp, Yc)));
    d = cfmar(z2e2, 2.0f, cfmar(z1e1, -2.0f * kp, cfmar(t.e2, 12.0f, cfmar(t.e1, -12.0f * kp, cmulr(Yc, -5.0f)))));
}
__device__ __forceinline__ void h_coeffs(const RadialTerms<float, cf> &t, const KConst<float> &k, float scale,
                                         cf &a, cf &b, cf &d) {
    h_coeffs_unit(t, k, a, b, d);
    const float p = k.inv4pi * scale;
    a = cmulr(a, p);
    b = cmulr(b, p);
    d = cmulr(d, p);
}

// B_trans: b = [(Y/2)(rh n^T + n rh^T) + psi2/c2^2 rn I] * scale/(4 pi)
template <class R, class C>
__device__ __forceinline__ void bt_coeffs(const RadialTerms<R, C> &t, const KConst<R> &k, R scale, C &sym, C &dia) {
    const R p = k.inv4pi * scale;
    sym = t.Y * ((R)0.5 * p);
    dia = t.psi2 * (k.ic2s * p);
}

// B_angular: b_pqk = [A T1 + Bq T2 + Cq T3] * scale/(4 pi) with
//   T1 = rh_p rh_k n_q + rh_q rh_k n_p + d_qk n_p + d_pk n_q,  A = r Y / 2
//   T2 = d_qk n_p + d_pk n_q,                                  Bq = (e2/c2 - e1/c1)/(2 s)
//   T3 = d_pq n_k,                                             Cq = e2/(c2 s)
template <class R, class C>
__device__ __forceinline__ void ba_coeffs(const RadialTerms<R, C> &t, const KConst<R> &k, R r, R scale, C &A, C &Bq,
                                          C &Cq) {
    const R p = k.inv4pi * scale;
    const C is = mk(k.isr, k.isi);
    A = t.Y * ((R)0.5 * r * p);
    Bq = (t.e2 * k.ic2 - t.e1 * k.ic1) * is * ((R)0.5 * p);
    Cq = t.e2 * is * (k.ic2 * p);
}

// symmetric 3x3 component order used for G and B_trans: 00 01 02 11 12 22
__host__ __device__ constexpr int sym_index(int p, int q) {
    return p <= q ? (p == 0 ? q : (p == 1 ? 2 + q : 5)) : (q == 0 ? p : (q == 1 ? 2 + p : 5));
}

}  // namespace sod
