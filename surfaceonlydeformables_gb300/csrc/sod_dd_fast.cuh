// sod_dd_fast.cuh -- double-float arithmetic without renormalisation, and e^-z with its tables in
// shared memory, for the device passes that need ~1e-10 per evaluation rather than the ~1e-14 of
// the renormalised operations of sod_dd.cuh: the compensated regular collocation pass and the
// singular passes.
#pragma once
#include "sod_dd.cuh"
#include "sod_device.cuh"

namespace sod {

// ---- double-float arithmetic without renormalisation ----------------------------------------------
// The pass needs ~1e-10 relative per evaluation, not the 1e-14 of renormalised double-float, so the
// radial terms use products and sums that keep the rounding error of the high words exactly (TwoProd
// by FMA, TwoSum) and add the low words in plain float, without the renormalising steps: the low word
// then carries a few ulps of the high word, which is harmless at this accuracy.  Sums that cancel
// (the psi numerator, Y, the kernel coefficients) are followed by one FastTwoSum.
// (high words through the non-contractible _rn operations, see sod_dd.cuh)
__device__ __forceinline__ dd sd_mul(dd a, dd b) {
    const float p = SOD_MUL_RN(a.hi, b.hi);
    return dd{p, fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, fmaf(a.hi, b.hi, -p)))};
}
__device__ __forceinline__ dd sd_mulf(dd a, float b) {
    const float p = SOD_MUL_RN(a.hi, b);
    return dd{p, fmaf(a.lo, b, fmaf(a.hi, b, -p))};
}
__device__ __forceinline__ dd sd_add(dd a, dd b) {
    const float s = SOD_ADD_RN(a.hi, b.hi), bb = SOD_SUB_RN(s, a.hi);
    return dd{s, SOD_ADD_RN(SOD_SUB_RN(a.hi, SOD_SUB_RN(s, bb)), SOD_SUB_RN(b.hi, bb)) + (a.lo + b.lo)};
}
__device__ __forceinline__ dd sd_neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd sd_sub(dd a, dd b) { return sd_add(a, sd_neg(b)); }
// renormalisation by TwoSum: after a cancelling sum the low word can exceed the high word
__device__ __forceinline__ dd sd_norm(dd a) { return two_sum(a.hi, a.lo); }
__device__ __forceinline__ cdd cs_mul(const cdd &a, const cdd &b) {
    return cdd{sd_sub(sd_mul(a.x, b.x), sd_mul(a.y, b.y)), sd_add(sd_mul(a.x, b.y), sd_mul(a.y, b.x))};
}
__device__ __forceinline__ cdd cs_add(const cdd &a, const cdd &b) { return cdd{sd_add(a.x, b.x), sd_add(a.y, b.y)}; }
__device__ __forceinline__ cdd cs_sub(const cdd &a, const cdd &b) { return cdd{sd_sub(a.x, b.x), sd_sub(a.y, b.y)}; }
__device__ __forceinline__ cdd cs_scale(const cdd &a, dd s) { return cdd{sd_mul(a.x, s), sd_mul(a.y, s)}; }
__device__ __forceinline__ cdd cs_scalef(const cdd &a, float s) { return cdd{sd_mulf(a.x, s), sd_mulf(a.y, s)}; }
__device__ __forceinline__ cdd cs_norm(const cdd &a) { return cdd{sd_norm(a.x), sd_norm(a.y)}; }

// Tables of the exponential and sine / cosine reductions (2^(j/64) and sin, cos (j pi / 32), double-float)
// copied to shared memory at kernel start: their indices differ from lane to lane, which the constant
// cache would serialise.
struct DdTabs {
    float2 e[64];
    float4 sc[64];
};
__device__ __forceinline__ void dd_tabs_load(DdTabs *t) {
    for (int j = threadIdx.x; j < 64; j += blockDim.x) {
        t->e[j] = make_float2(c_dd_exp2_tab[j][0], c_dd_exp2_tab[j][1]);
        t->sc[j] = make_float4(c_dd_sincos_tab[j][0], c_dd_sincos_tab[j][1], c_dd_sincos_tab[j][2], c_dd_sincos_tab[j][3]);
    }
}

// e^-z for z = x + iy with x >= 0: Tang's reduction of the exponent (-x = (64k + j) ln2/64 + r,
// |r| <= ln2/128) and a reduction of the phase by pi/32 (|u| <= pi/64), short Taylor series with only
// the leading terms in double-float (the rest is below 1e-12 of the result in float), table values
// combined by the angle addition.  About 1e-13 relative; results below 2^-124 flush to zero.  Phases
// beyond |y| = 400 (outside the exact range of the reduction) take FP64 sin/cos.
__device__ __forceinline__ cdd cs_exp_neg(const cdd &z, const DdTabs *tb) {
    dd mag;
    {
        const float ah = -z.x.hi;
        if (ah < -86.0f) return cdd{dd{0.f, 0.f}, dd{0.f, 0.f}};
        const float m = fmaf(ah, kDd64oLn2, kRound23) - kRound23;
        const float rh0 = fmaf(-m, kDdLn2o64_1, ah);  // exact: m kDdLn2o64_1 has few bits
        const dd p2 = two_prod(m, kDdLn2o64_2);
        const dd r0 = two_sum(rh0, -p2.hi);
        // renormalised: the low word of x (up to half an ulp of x, ~4e-6 at x = 80) is far above an ulp
        // of r, and the series below drops the cross terms of the low word beyond the first order
        const dd r = two_sum(r0.hi, r0.lo + (-z.x.lo - p2.lo - m * kDdLn2o64_3));
        const float rl = r.lo;
        // e^r = 1 + r + r^2/2 + r^3/6 + r^4/24 (|r| <= 0.0055: the r^2 terms and beyond in float)
        const float h = r.hi;
        const float q = h * h * fmaf(h, fmaf(h, 1.0f / 24.0f, 1.0f / 6.0f), 0.5f);
        const dd one_r = fast_two_sum(1.0f, h);
        const dd em = dd{one_r.hi, one_r.lo + fmaf(h, rl, rl + q)};
        const int mi = (int)m, j = mi & 63, k = (mi - j) / 64;
        const float2 t = tb->e[j];
        const dd v = sd_mul(dd{t.x, t.y}, em);
        const float sc = __int_as_float((k + 127) * (1 << 23));  // 2^k, k >= -124 here
        mag = dd{v.hi * sc, v.lo * sc};
    }
    dd sn, cs;
    {
        const float yh = z.y.hi;
        if (!(fabsf(yh) < 400.0f)) {
            double sv, cv;
            sincos(dd_to(z.y), &sv, &cv);
            sn = dd_from(sv), cs = dd_from(cv);
        } else {
            const float m = fmaf(yh, kDd32oPi, kRound23) - kRound23;
            const float uh0 = fmaf(-m, kDdPio32_1, yh);  // exact
            const dd p2 = two_prod(m, kDdPio32_2);
            const dd u0 = two_sum(uh0, -p2.hi);
            // renormalised for the same reason (the low word of y reaches ~8e-6 at |y| = 150)
            const dd u = two_sum(u0.hi, u0.lo + (z.y.lo - p2.lo - m * kDdPio32_3));
            const float ul = u.lo;
            const float h = u.hi, h2 = h * h;
            // sin u = u - u^3/6 + u^5/120; cos u = 1 - u^2/2 + u^4/24 - u^6/720
            const dd su = dd{h, fmaf(h * h2, fmaf(h2, 1.0f / 120.0f, -1.0f / 6.0f), ul)};
            const dd sq = two_prod(h, h);  // u^2 high part, exactly
            const dd c1 = fast_two_sum(1.0f, -0.5f * sq.hi);
            const dd cu = dd{c1.hi, c1.lo + (fmaf(-h, ul, -0.5f * sq.lo) + h2 * h2 * fmaf(h2, -1.0f / 720.0f, 1.0f / 24.0f))};
            const float4 t = tb->sc[((int)m) & 63];
            const dd S = dd{t.x, t.y}, C = dd{t.z, t.w};
            sn = sd_norm(sd_add(sd_mul(S, cu), sd_mul(C, su)));  // cancel near the zeros of sin / cos
            cs = sd_norm(sd_sub(sd_mul(C, cu), sd_mul(S, su)));
        }
    }
    return cdd{sd_mul(mag, cs), sd_neg(sd_mul(mag, sn))};
}

// acc += x * w for double-float x and w: one TwoSum on the high words, the product's error and the
// cross terms summed in float into an unnormalised low word (a few dozen terms per accumulator; the
// caller reads hi + lo at the end).
__device__ __forceinline__ void sd_fma_acc(dd &acc, dd x, dd w) {
    const float p = SOD_MUL_RN(x.hi, w.hi);
    const float e = fmaf(x.hi, w.hi, -p);
    const dd s = two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo += s.lo + fmaf(x.lo, w.hi, fmaf(x.hi, w.lo, e));
}
__device__ __forceinline__ void cs_fma_acc(cdd &acc, const cdd &x, dd w) {
    sd_fma_acc(acc.x, x.x, w);
    sd_fma_acc(acc.y, x.y, w);
}
__device__ __forceinline__ void sd_acc(dd &acc, dd x) {
    const dd s = two_sum(acc.hi, x.hi);
    acc.hi = s.hi;
    acc.lo += s.lo + x.lo;
}

// e^-z with the renormalised double-float arithmetic of sod_dd.cuh (2^-47 relative) and the tables in
// shared memory: for the singular passes, whose cancelling traction kernel needs the full accuracy
__device__ __forceinline__ cdd cdd_exp_neg_tab(const cdd &z, const DdTabs *tb) {
    const dd m = dd_exp_t(-z.x, [tb](int j) { return dd{tb->e[j].x, tb->e[j].y}; });
    dd s, c;
    dd_sincos_t(z.y, s, c, [tb](int j, dd &S, dd &C) {
        const float4 t = tb->sc[j];
        S = dd{t.x, t.y};
        C = dd{t.z, t.w};
    });
    return cdd{m * c, -(m * s)};
}

}  // namespace sod
