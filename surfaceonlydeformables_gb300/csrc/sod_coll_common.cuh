// sod_coll_common.cuh -- pieces shared by the collocation kernels of sod_collocation.cu (FP32 regular
// pass, singular passes, batched launches) and sod_coll_compensated.cu (the compensated regular pass):
// the launch arguments, the singular-face test, the output stores and the split-phase colour barrier.
#pragma once
#include "sod_bmom.cuh"
#include "sod_faces.cuh"
#include "sod_internal.h"

namespace sod {

constexpr int KM_G = 1 << SOD_G, KM_BT = 1 << SOD_B_TRANS, KM_BA = 1 << SOD_B_ANGULAR;

struct CollArgs {
    int nV, nF;
    const float4 *faces;   // coloured (scatter kernels) or natural (reduce kernels) order
    const int4 *canonF;    // canonical corner ids per face record, or null
    const int *color_off;  // ncolors+1 (scatter kernels)
    int ncolors;
    int i0;                // first field vertex of the plain kernels' grid (row chunks)
    const float *Vf;       // nV x 3
    const int *canonV;     // canonical id per vertex, or null
    void *out[4];          // per kind (G, H, B_trans, B_angular)
    long long fstride[4];  // elements between frequencies of out[kind]
    int out_c64;           // 1: complex64 output, 0: complex128
    int do_regular;
    const cd *S[4];        // singular corrections per kind (null if none)
    long long S_fstride[4];
    const int *nbr_off;    // G/H: per vertex slot ranges
    const int *nbr_vert;
    int *err;              // device error word of the bounded colour-phase waits (null: not recorded)
    int bar_extra;         // test hook: extra arrivals the colour-phase barrier expects (0 normally)
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

// Final B_trans / B_angular store of field vertex i from the CTA's component sums `bsum` (FP64),
// plus the singular side buffers.
template <int BM>
__device__ __forceinline__ void store_b(const CollArgs &a, const cd *bsum, int i, int fq) {
    using M = BMom<BM>;
    if (M::BT) {
        const long long base = (long long)fq * a.fstride[SOD_B_TRANS] + (long long)(3 * i) * 3;
        for (int e = threadIdx.x; e < 9; e += blockDim.x) {
            const int p = e / 3, qq = e % 3;
            cd s = bsum[sym_index(p, qq)];
            if (a.S[SOD_B_TRANS])
                s = s + a.S[SOD_B_TRANS][(long long)fq * a.S_fstride[SOD_B_TRANS] + (long long)i * 9 + e];
            store_out(a.out[SOD_B_TRANS], a.out_c64, base + e, s.x, s.y);
        }
    }
    if (M::BA) {
        const long long base = (long long)fq * a.fstride[SOD_B_ANGULAR] + (long long)(3 * i) * 9;
        for (int e = threadIdx.x; e < 27; e += blockDim.x) {
            const int p = e / 9, qq = (e / 3) % 3, kk = e % 3;
            cd s = bsum[M::NT + 3 * sym_index(p, qq) + kk];
            if (a.S[SOD_B_ANGULAR])
                s = s + a.S[SOD_B_ANGULAR][(long long)fq * a.S_fstride[SOD_B_ANGULAR] + (long long)i * 27 + e];
            store_out(a.out[SOD_B_ANGULAR], a.out_c64, base + e, s.x, s.y);
        }
    }
}

// -------------------------------------------------------------------------------------------
// Colour phases of the scatter: split arrive / wait on one mbarrier per CTA.  A warp arrives (one
// lane, after __syncwarp) once its adds of a colour are done; a thread waits for the previous
// colour's phase only just before its own row-accumulator adds, so the quadrature of its next face
// overlaps the stragglers of the previous colour.  Phases run on across a CTA's work items: the
// caller's `phase` counts the completed ones.  Every wait is bounded (about a second of clock); on
// expiry the CTA stops waiting (its results are then wrong) and the error word tells the host,
// which reports SOD_ERR_TIMEOUT from its next synchronising call.
constexpr long long COLOUR_WAIT_CYCLES = 2000000000LL;
struct ColourBar {
    unsigned long long bar;
    int abort;
};
__device__ __forceinline__ unsigned colour_bar_addr(ColourBar *cb) {
    return (unsigned)__cvta_generic_to_shared(&cb->bar);
}
// thread 0 initialises (one arrival per warp, plus `extra` for the timeout test); the callers' first
// CTA barrier orders it before any use
__device__ __forceinline__ void colour_bar_init(ColourBar *cb, int extra = 0) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(colour_bar_addr(cb)),
                     "r"(((blockDim.x + 31) >> 5) + (unsigned)extra)
                     : "memory");
        cb->abort = 0;
    }
}
__device__ __forceinline__ void colour_arrive(ColourBar *cb) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(colour_bar_addr(cb)) : "memory");
}
__device__ __forceinline__ void colour_wait(ColourBar *cb, unsigned parity, int *err) {
    volatile int *ab = &cb->abort;
    if (*ab) return;
    const long long t0 = clock64();
    for (;;) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(colour_bar_addr(cb)), "r"(parity)
            : "memory");
        if (ok || *ab) return;
        if (clock64() - t0 > COLOUR_WAIT_CYCLES) {
            *ab = 1;
            if (err) atomicExch(err, 1);
            return;
        }
    }
}


}  // namespace sod
