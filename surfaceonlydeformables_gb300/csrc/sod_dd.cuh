// sod_dd.cuh -- double-float ("dd") arithmetic for the singular quadrature on the FP32 pipes.
//
// GB300 runs FP64 at 1/64 of its FP32 rate.  The singular passes need about 1e-13 relative accuracy
// (they are checked against the FP64 oracle to 1e-10), which a pair of floats (hi + lo, 48-bit
// significand, |lo| <= ulp(hi)/2) delivers at a fraction of the FP64 cost.
//
// Algorithms (restated, not taken from any library source):
//   * error-free transformations: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971),
//     the FMA product error a*b - fl(a*b);
//   * double-word addition and multiplication as in Dekker (1971) and Hida, Li & Bailey,
//     "Algorithms for quad-double precision floating point arithmetic" (2001), on float pairs;
//   * reciprocal: one Newton step from the float reciprocal (doubles the correct bits);
//   * exp: Tang's table-driven method (ACM TOMS 15(2), 1989): a = (64k + j) ln2/64 + r,
//     e^a = 2^k 2^(j/64) e^r, |r| <= ln2/128, Taylor series of e^r - 1;
//   * sin/cos: reduction by pi/32 with a three-part Cody-Waite constant, Taylor series on
//     |u| <= pi/64 and the angle-addition formulas with a 64-entry table of sin/cos(j pi/32).
// Tables and split constants come from gen_dd_tables.py (mpmath, 60 digits).
//
// The header compiles for the host as well (plain C++ with -ffp-contract=off) so that the CPU
// tests can check every function against high-precision references.
#pragma once
#include <cmath>

// The error-free transformations below need every operation rounded on its own.  nvcc contracts a
// multiply into a later add or subtract (-fmad=true, also across statements and when the product
// has other uses), which would make TwoSum / TwoProduct compute their error term from an unrounded
// product, i.e. return the rounding error of a different sum: the pair then loses the low word's
// accuracy (~1e-7 relative instead of ~1e-14).  The _rn intrinsics are never contracted.
#if defined(__CUDA_ARCH__)
#define SOD_ADD_RN(a, b) __fadd_rn((a), (b))
#define SOD_SUB_RN(a, b) __fsub_rn((a), (b))
#define SOD_MUL_RN(a, b) __fmul_rn((a), (b))
#else
#define SOD_ADD_RN(a, b) ((a) + (b))
#define SOD_SUB_RN(a, b) ((a) - (b))
#define SOD_MUL_RN(a, b) ((a) * (b))
#endif

#ifdef __CUDACC__
#define SOD_HD __device__ __forceinline__
#define SOD_DD_TABLE static __device__ __constant__ const
#else
#define SOD_HD inline
#define SOD_DD_TABLE static const
#endif

#include "sod_dd_tables.h"

namespace sod {

struct dd {
    float hi, lo;
};

SOD_HD dd dd_make(float hi, float lo) { return dd{hi, lo}; }
SOD_HD dd dd_from(double x) {
    const float h = (float)x;
    return dd{h, (float)(x - (double)h)};
}
SOD_HD double dd_to(dd a) { return (double)a.hi + (double)a.lo; }

// ---- error-free transformations ----
SOD_HD dd two_sum(float a, float b) {
    const float s = SOD_ADD_RN(a, b);
    const float bb = SOD_SUB_RN(s, a);
    const float e = SOD_ADD_RN(SOD_SUB_RN(a, SOD_SUB_RN(s, bb)), SOD_SUB_RN(b, bb));
    return dd{s, e};
}
SOD_HD dd fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = SOD_ADD_RN(a, b);
    return dd{s, SOD_SUB_RN(b, SOD_SUB_RN(s, a))};
}
SOD_HD dd two_prod(float a, float b) {
    const float p = SOD_MUL_RN(a, b);
    return dd{p, fmaf(a, b, -p)};
}

// ---- arithmetic ----
SOD_HD dd operator-(dd a) { return dd{-a.hi, -a.lo}; }
SOD_HD dd operator+(dd a, dd b) {  // accurate addition (both error terms kept)
    dd s = two_sum(a.hi, b.hi);
    const dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
SOD_HD dd operator-(dd a, dd b) { return a + (-b); }
SOD_HD dd operator+(dd a, float b) {
    dd s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
SOD_HD dd operator*(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
SOD_HD dd operator*(dd a, float b) {
    dd p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
SOD_HD dd operator*(float b, dd a) { return a * b; }
// exact scaling by a power of two
SOD_HD dd dd_ldexp(dd a, int k) { return dd{ldexpf(a.hi, k), ldexpf(a.lo, k)}; }
// accumulation of many terms of similar size: one TwoSum, the low parts added in float
SOD_HD void dd_acc(dd &acc, dd x) {
    dd s = two_sum(acc.hi, x.hi);
    s.lo += acc.lo + x.lo;
    acc = fast_two_sum(s.hi, s.lo);
}
SOD_HD dd dd_recip(dd b) {
    const float y = 1.0f / b.hi;
    const dd e = dd{1.0f, 0.0f} - b * y;  // 1 - b y, exact to dd precision
    return dd{y, 0.0f} + e * y;
}
SOD_HD dd operator/(dd a, dd b) { return a * dd_recip(b); }
// square root: correctly rounded float root, then one Newton correction of the residual in dd
SOD_HD dd dd_sqrt(dd a) {
    if (!(a.hi > 0.0f)) return dd{0.0f, 0.0f};
    const float s = sqrtf(a.hi);
    const dd e = a - two_prod(s, s);
    return fast_two_sum(s, e.hi * (0.5f / s));
}

// ---- exp ----
// e^a for a.hi in [-87, 88]: 2^-47 relative accuracy down to a = -69; below that the low word
// falls into FP32 subnormals and loses bits, and below -87 the result is flushed to zero.
// (the table of 2^(j/64) is read through `tab(j)`: the constant table here, a shared-memory copy in
// kernels whose lanes index it differently)
template <class Tab> SOD_HD dd dd_exp_t(dd a, const Tab &tab) {
    if (a.hi < -87.0f) return dd{0.0f, 0.0f};
    const float m = rintf(a.hi * kDd64oLn2);
    // r = a - m ln2/64 (m ln2/64 with a three-part constant; m * c1 is exact for |m| < 2^13)
    dd r = two_sum(fmaf(-m, kDdLn2o64_1, a.hi), a.lo);
    r = r - two_prod(m, kDdLn2o64_2);
    r = r + (-m * kDdLn2o64_3);
    // e^r - 1 = r + r^2/2 + r^3/6 + r^4/24 + ..., |r| <= 0.0055: r^4/24 onwards in float
    const dd r2 = r * r;
    const dd r3 = r2 * r;
    const float h = r.hi;
    const float tail = h * h * h * h * (1.0f / 24.0f + h * (1.0f / 120.0f + h * (1.0f / 720.0f)));
    dd em1 = r + dd{0.5f * r2.hi, 0.5f * r2.lo};
    em1 = em1 + r3 * dd{kDdSixth_hi, kDdSixth_lo};
    em1 = em1 + tail;
    const int mi = (int)m;
    const int j = mi & 63;
    const int k = (mi - j) / 64;
    const dd t = tab(j);
    return dd_ldexp(t + t * em1, k);
}

SOD_HD dd dd_exp(dd a) {
    return dd_exp_t(a, [](int j) { return dd{c_dd_exp2_tab[j][0], c_dd_exp2_tab[j][1]}; });
}

// ---- sin / cos ----
// |y.hi| < 400 (|m| < 2^12 keeps m * c1 exact); larger arguments fall back to FP64.
template <class Tab> SOD_HD void dd_sincos_t(dd y, dd &s, dd &c, const Tab &tab) {
    if (!(fabsf(y.hi) < 400.0f)) {
        const double v = dd_to(y);
        s = dd_from(sin(v));
        c = dd_from(cos(v));
        return;
    }
    const float m = rintf(y.hi * kDd32oPi);
    dd u = two_sum(fmaf(-m, kDdPio32_1, y.hi), y.lo);
    u = u - two_prod(m, kDdPio32_2);
    u = u + (-m * kDdPio32_3);
    const dd u2 = u * u;
    const float h = u2.hi;
    // sin u = u (1 + P), P = -u^2/6 + u^4/120 - u^6/5040 (|u| <= pi/64)
    dd P = -(u2 * dd{kDdSixth_hi, kDdSixth_lo});
    P = P + h * h * (1.0f / 120.0f - h * (1.0f / 5040.0f));
    const dd su = u + u * P;
    // cos u = 1 + Q, Q = -u^2/2 + u^4/24 - u^6/720 + u^8/40320
    dd Q = dd{-0.5f * u2.hi, -0.5f * u2.lo};
    Q = Q + (u2 * u2) * dd{kDdTwentyFourth_hi, kDdTwentyFourth_lo};
    Q = Q + h * h * h * (-1.0f / 720.0f + h * (1.0f / 40320.0f));
    const int j = ((int)m) & 63;
    dd S, C;
    tab(j, S, C);
    s = S + (S * Q + C * su);
    c = C + (C * Q - S * su);
}

SOD_HD void dd_sincos(dd y, dd &s, dd &c) {
    dd_sincos_t(y, s, c, [](int j, dd &S, dd &C) {
        S = dd{c_dd_sincos_tab[j][0], c_dd_sincos_tab[j][1]};
        C = dd{c_dd_sincos_tab[j][2], c_dd_sincos_tab[j][3]};
    });
}

// ---- complex double-float ----
struct cdd {
    dd x, y;
};
SOD_HD cdd cdd_make(dd x, dd y) { return cdd{x, y}; }
SOD_HD cdd operator+(cdd a, cdd b) { return cdd{a.x + b.x, a.y + b.y}; }
SOD_HD cdd operator-(cdd a, cdd b) { return cdd{a.x - b.x, a.y - b.y}; }
SOD_HD cdd operator*(cdd a, cdd b) { return cdd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
SOD_HD cdd operator*(cdd a, dd s) { return cdd{a.x * s, a.y * s}; }
SOD_HD cdd operator*(cdd a, float s) { return cdd{a.x * s, a.y * s}; }
SOD_HD cdd cdd_recip(cdd a) {
    const dd inv = dd_recip(a.x * a.x + a.y * a.y);
    return cdd{a.x * inv, -(a.y * inv)};
}
SOD_HD void cdd_acc(cdd &acc, cdd v, dd w) {
    dd_acc(acc.x, v.x * w);
    dd_acc(acc.y, v.y * w);
}
// e^-z
SOD_HD cdd cdd_exp_neg(cdd z) {
    const dd m = dd_exp(-z.x);
    dd s, c;
    dd_sincos(z.y, s, c);
    return cdd{m * c, -(m * s)};
}

// psi(z) = ((1 + z) e^-z - 1) / z^2.  The closed form loses about 2 eps / |z|^2 (eps = 2^-48), so
// below |z| = 0.1 the Taylor series -sum (-1)^m (m+1) z^m / (m+2)! is used instead: terms m <= 4
// in double-float, m = 5..8 in float (truncation < 1e-15 relative).
SOD_HD cdd cdd_psi(cdd z, cdd ez) {
    const float az2 = z.x.hi * z.x.hi + z.y.hi * z.y.hi;
    if (az2 < 0.01f) {
        // float tail T = c5 + z (c6 + z (c7 + z c8))
        const float zr = z.x.hi, zi = z.y.hi;
        const float c8 = -9.0f / 3628800.0f, c7 = 8.0f / 362880.0f, c6 = -7.0f / 40320.0f, c5 = 6.0f / 5040.0f;
        float tr = c8, ti = 0.0f;
        float nr = tr * zr - ti * zi + c7, ni = tr * zi + ti * zr;
        tr = nr, ti = ni;
        nr = tr * zr - ti * zi + c6, ni = tr * zi + ti * zr;
        tr = nr, ti = ni;
        nr = tr * zr - ti * zi + c5, ni = tr * zi + ti * zr;
        cdd acc = cdd{dd{nr, 0.0f}, dd{ni, 0.0f}};
        // c4 = -5/720 = -1/144, c3 = 4/120 = 1/30, c2 = -3/24 = -1/8, c1 = 2/6 = 1/3, c0 = -1/2
        acc = acc * z;
        acc.x = acc.x + dd{kDdM144th_hi, kDdM144th_lo};
        acc = acc * z;
        acc.x = acc.x + dd{kDdThirtieth_hi, kDdThirtieth_lo};
        acc = acc * z;
        acc.x = acc.x + (-0.125f);
        acc = acc * z;
        acc.x = acc.x + dd{kDdThird_hi, kDdThird_lo};
        acc = acc * z;
        acc.x = acc.x + (-0.5f);
        return acc;
    }
    cdd num = (cdd{z.x + 1.0f, z.y}) * ez;
    num.x = num.x + (-1.0f);
    return num * cdd_recip(z * z);
}

}  // namespace sod
