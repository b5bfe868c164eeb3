// sod_bmom.cuh -- B_trans / B_angular face moments shared by the collocation and Galerkin passes.
#pragma once
#include "../../include/sod_gb300.h"
#include "sod_device.cuh"

namespace sod {

// B_trans / B_angular moments of one face (BM subset of KM_BT | KM_BA).  The tensor structure
// depends only on the face normal, so the quadrature accumulates scalar moments and the face
// tensor is formed once per face:
//     B_trans   b_pq  = Ms_p n_q + Ms_q n_p + d_pq Md
//     B_angular b_pqk = M1_pk n_q + M1_qk n_p + (M0 + SB)(d_qk n_p + d_pk n_q) + SC d_pq n_k
// Component order of the face tensor: B_trans sym(p,q) (6), then B_angular 3 sym(p,q) + k (18).
// The per-point sums carry only the radial factors (Y, psi2, e1, e2) times the geometric weights;
// the frequency constants common to a moment (1/(4 pi), 1/c2^2, 1/s, 1/c2) multiply it once, when
// the face tensor is formed.
template <int BM> struct BMom {
    static constexpr bool BT = (BM & (1 << SOD_B_TRANS)) != 0, BA = (BM & (1 << SOD_B_ANGULAR)) != 0;
    static constexpr int NT = BT ? 6 : 0, NA = BA ? 18 : 0, NC = NT + NA;
    cf Ms[3], Md, M1[6], M0, SE, SC;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int c = 0; c < 3; c++) Ms[c] = mk(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 6; c++) M1[c] = mk(0.f, 0.f);
        Md = M0 = SE = SC = mk(0.f, 0.f);
    }
    // Ms_p += Y w rh_p, Md += psi2 w rn;  M1_pk += Y r w rh_p rh_k, M0 += Y r w,
    // SE += e1 w, SC += e2 w (the sum of (e2/c2 - e1/c1) w is SC/c2 - SE/c1, formed at the emit)
    __device__ __forceinline__ void add(const RadialTerms<float, cf> &t, const KConst<float> &k, float r,
                                        const float rh[3], const float nn[3], float w) {
        if (BT) {
            const cf ws = cmulr(t.Y, w);
#pragma unroll
            for (int p = 0; p < 3; p++) cfma(Ms[p], ws, rh[p]);
            cfma(Md, t.psi2, w * (rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2]));
        }
        if (BA) {
            const cf wA = cmulr(t.Y, r * w);
#pragma unroll
            for (int p = 0; p < 3; p++) {
                const cf wp = cmulr(wA, rh[p]);
#pragma unroll
                for (int kk = p; kk < 3; kk++) cfma(M1[sym_index(p, kk)], wp, rh[kk]);
            }
            M0 = M0 + wA;
            cfma(SE, t.e1, w);
            cfma(SC, t.e2, w);
        }
    }
    // face tensor times `ar`, component by component: sink(c, value).  Scales the moments by their
    // frequency constants first: Ms, M1, M0 by 1/(8 pi); Md by 1/(4 pi c2^2); SB by 1/(8 pi s);
    // SC by 1/(4 pi c2 s).
    template <class Sink>
    __device__ __forceinline__ void emit(const KConst<float> &k, const float nn[3], float ar, Sink &&sink) {
        const float half = 0.5f * k.inv4pi * ar;
        if (BT) {
#pragma unroll
            for (int p = 0; p < 3; p++) Ms[p] = cmulr(Ms[p], half);
            Md = cmulr(Md, k.ic2s * k.inv4pi * ar);
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int qq = p; qq < 3; qq++) {
                    cf v = cfmar(Ms[p], nn[qq], cmulr(Ms[qq], nn[p]));
                    if (p == qq) v = v + Md;
                    sink(sym_index(p, qq), v);
                }
        }
        if (BA) {
            const cf is = mk(k.isr, k.isi);
#pragma unroll
            for (int c = 0; c < 6; c++) M1[c] = cmulr(M1[c], half);
            const cf SB = cfmar(SE, -k.ic1, cmulr(SC, k.ic2));
            const cf M0B = cmulr(M0, half) + cmulr(SB * is, half);
            const cf SCs = cmulr(SC * is, k.ic2 * k.inv4pi * ar);
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int qq = p; qq < 3; qq++)
#pragma unroll
                    for (int kk = 0; kk < 3; kk++) {
                        cf v = cfmar(M1[sym_index(p, kk)], nn[qq], cmulr(M1[sym_index(qq, kk)], nn[p]));
                        const float t2 = (qq == kk ? nn[p] : 0.f) + (p == kk ? nn[qq] : 0.f);
                        v = cfmar(M0B, t2, v);
                        if (p == qq) v = cfmar(SCs, nn[kk], v);
                        sink(NT + 3 * sym_index(p, qq) + kk, v);
                    }
        }
    }
};

}  // namespace sod
