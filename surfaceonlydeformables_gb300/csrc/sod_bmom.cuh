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
template <int BM> struct BMom {
    static constexpr bool BT = (BM & (1 << SOD_B_TRANS)) != 0, BA = (BM & (1 << SOD_B_ANGULAR)) != 0;
    static constexpr int NT = BT ? 6 : 0, NA = BA ? 18 : 0, NC = NT + NA;
    cf Ms[3], Md, M1[6], M0, SB, SC;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int c = 0; c < 3; c++) Ms[c] = mk(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 6; c++) M1[c] = mk(0.f, 0.f);
        Md = M0 = SB = SC = mk(0.f, 0.f);
    }
    __device__ __forceinline__ void add(const RadialTerms<float, cf> &t, const KConst<float> &k, float r,
                                        const float rh[3], const float nn[3], float w) {
        if (BT) {
            cf sy, di;
            bt_coeffs(t, k, 1.0f, sy, di);
            const cf ws = sy * w;
#pragma unroll
            for (int p = 0; p < 3; p++) cfma(Ms[p], ws, rh[p]);
            cfma(Md, di, w * (rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2]));
        }
        if (BA) {
            cf A, Bq, Cq;
            ba_coeffs(t, k, r, 1.0f, A, Bq, Cq);
            const cf wA = A * w;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int kk = p; kk < 3; kk++) cfma(M1[sym_index(p, kk)], wA, rh[p] * rh[kk]);
            M0 = M0 + wA;
            cfma(SB, Bq, w);
            cfma(SC, Cq, w);
        }
    }
    // face tensor times `ar`, component by component: sink(c, value)
    template <class Sink> __device__ __forceinline__ void emit(const float nn[3], float ar, Sink &&sink) const {
        if (BT) {
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int qq = p; qq < 3; qq++) {
                    cf v = Ms[p] * nn[qq] + Ms[qq] * nn[p];
                    if (p == qq) v = v + Md;
                    sink(sym_index(p, qq), v * ar);
                }
        }
        if (BA) {
            const cf M0B = M0 + SB;
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int qq = p; qq < 3; qq++)
#pragma unroll
                    for (int kk = 0; kk < 3; kk++) {
                        cf v = M1[sym_index(p, kk)] * nn[qq] + M1[sym_index(qq, kk)] * nn[p];
                        const float t2 = (qq == kk ? nn[p] : 0.f) + (p == kk ? nn[qq] : 0.f);
                        v = v + M0B * t2;
                        if (p == qq) v = v + SC * nn[kk];
                        sink(NT + 3 * sym_index(p, qq) + kk, v * ar);
                    }
        }
    }
};

}  // namespace sod
