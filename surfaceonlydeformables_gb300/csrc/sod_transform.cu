// sod_transform.cu -- inverse transform from Laplace frequencies to CQ time weights.
//
// X_n = R^-n / L * sum_{l=0}^{L/2} c_l Re(Xhat_l zeta^-nl)  for every matrix entry, n = 0..L-1
// (reference: src/elastodynamics_cqbem_G.cu:166-179, H.cu:172-195, B_trans.cu:148-163,
// B_angular.cu:151-175).  The reference re-reads every U_l.mat from disk for each n; here each
// CTA stages a tile of entries x all frequencies in shared memory once and produces all L outputs.
//
// Two kernels:
//  * FP64 output: native FP64 accumulation (one DFMA per real multiply-add).  Late weights are the
//    result of heavy cancellation (terms ~R^-n |Xhat|, results far smaller), so only 53-bit
//    accumulation reproduces the reference's FP64 transform to 1e-10 on real data.
//  * FP32 output: double-float arithmetic on the FP32 pipes (GB300 has little FP64 throughput):
//    twiddles split hi+lo, every product hi*x formed exactly with an FMA (TwoProduct), the sum
//    carried as an unevaluated pair with TwoSum -- about 2^-48 of the term magnitude, far below
//    the rounding of the FP32 result.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sod_internal.h"

namespace sod {

// error-free transformations on FP32
// (each operation rounded on its own: _rn intrinsics, which nvcc never contracts into an FMA)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
struct df {
    float hi, lo;
};
// acc += a * x  where a = (ahi + alo) is a double-float constant and x an FP32 value
__device__ __forceinline__ void df_mac(df &acc, float ahi, float alo, float x) {
    const float p = __fmul_rn(ahi, x);
    const float pe = fmaf(ahi, x, -p);  // exact: p + pe = ahi * x
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.lo += e + fmaf(alo, x, pe);
    acc.hi = s;
}
// (A + sign B) g rounded to float, g = (g.x + g.y) a float pair
__device__ __forceinline__ float df_scaled(df A, df B, float sign, float2 g) {
    float s, e;
    two_sum(A.hi, sign * B.hi, s, e);
    const float lo = e + (A.lo + sign * B.lo);
    const float p = __fmul_rn(s, g.x);
    const float pe = fmaf(s, g.x, -p);
    return p + fmaf(s, g.y, fmaf(lo, g.x, pe));
}

// FP32 output, double-float accumulation, on the same n <-> L - n symmetry as the FP64 kernel below:
// A_n = sum_l c_l cos xr_l and B_n = sum_l c_l sin xi_l for n <= L/2, then X_n = g_n (A + B) and
// X_{L-n} = g_{L-n} (A - B), g_n = R^-n / L as a float pair; the combination and the scaling stay in
// float arithmetic (TwoSum / TwoProduct), the output is their rounded sum.
template <int TILE>
__global__ void __launch_bounds__(TILE) inv_transform_df_kernel(const void *__restrict__ Xhat, int in_c128, long long M,
                                                               int nfreq, int L, const float4 *__restrict__ tw,
                                                               const float2 *__restrict__ gsc, float *__restrict__ out) {
    // shared: twiddles [L/2 + 1][nfreq] as float4 (c cos hi, lo, c sin hi, lo), scales [L] (hi, lo),
    // entries [nfreq][TILE] hi (+ lo)
    extern __shared__ float4 sm[];
    const int nh = L / 2;
    float4 *stw = sm;
    float2 *sg = reinterpret_cast<float2 *>(stw + (nh + 1) * nfreq);
    float2 *sx_hi = sg + ((L + 1) & ~1);
    float2 *sx_lo = sx_hi + (size_t)nfreq * TILE;
    for (int t = threadIdx.x; t < (nh + 1) * nfreq; t += TILE) stw[t] = tw[t];
    for (int t = threadIdx.x; t < L; t += TILE) sg[t] = gsc[t];
    const long long e = (long long)blockIdx.x * TILE + threadIdx.x;
    const bool live = e < M;
    for (int l = 0; l < nfreq; l++) {
        float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
        if (live) {
            if (in_c128) {
                const double2 v = reinterpret_cast<const double2 *>(Xhat)[(long long)l * M + e];
                hi = make_float2((float)v.x, (float)v.y);
                lo = make_float2((float)(v.x - (double)hi.x), (float)(v.y - (double)hi.y));
            } else {
                hi = reinterpret_cast<const float2 *>(Xhat)[(long long)l * M + e];
            }
        }
        sx_hi[l * TILE + threadIdx.x] = hi;
        if (in_c128) sx_lo[l * TILE + threadIdx.x] = lo;
    }
    __syncthreads();
    if (!live) return;
    for (int n = 0; n <= nh; n++) {
        df A = {0.f, 0.f}, B = {0.f, 0.f};
        for (int l = 0; l < nfreq; l++) {
            const float4 w = stw[n * nfreq + l];
            const float2 x = sx_hi[l * TILE + threadIdx.x];
            df_mac(A, w.x, w.y, x.x);
            df_mac(B, w.z, w.w, x.y);
            if (in_c128) {
                const float2 xl = sx_lo[l * TILE + threadIdx.x];
                df_mac(A, w.x, w.y, xl.x);
                df_mac(B, w.z, w.w, xl.y);
            }
        }
        out[(long long)n * M + e] = df_scaled(A, B, 1.0f, sg[n]);
        const int m = L - n;
        if (n >= 1 && m != n) out[(long long)m * M + e] = df_scaled(A, B, -1.0f, sg[m]);
    }
}

// FP64 output.  With theta = 2 pi n l / L, Re(Xhat_l zeta^-nl) = xr cos(theta) + xi sin(theta), and
// n -> L - n keeps the cosine and flips the sine, so for n <= L/2
//     A_n = sum_l c_l xr_l cos,  B_n = sum_l c_l xi_l sin,
//     X_n = R^-n / L (A_n + B_n),  X_{L-n} = R^-(L-n) / L (A_n - B_n):
// (L/2 + 1) nfreq multiply-add pairs per entry instead of L nfreq (the same terms, summed as two
// partial sums).
template <int TILE>
__global__ void __launch_bounds__(TILE) inv_transform_f64_kernel(const void *__restrict__ Xhat, int in_c128, long long M,
                                                                int nfreq, int L, const double2 *__restrict__ tw,
                                                                const double *__restrict__ gsc, double *__restrict__ out) {
    extern __shared__ double2 smd[];
    const int nh = L / 2;
    double2 *stw = smd;                                                  // [nh + 1][nfreq] (c_l cos, c_l sin)
    double2 *sx = stw + (size_t)(nh + 1) * nfreq;                        // [nfreq][TILE] inputs
    double *sg = reinterpret_cast<double *>(sx + (size_t)nfreq * TILE);  // [L] R^-n / L
    for (int t = threadIdx.x; t < (nh + 1) * nfreq; t += TILE) stw[t] = tw[t];
    for (int t = threadIdx.x; t < L; t += TILE) sg[t] = gsc[t];
    const long long e = (long long)blockIdx.x * TILE + threadIdx.x;
    const bool live = e < M;
    for (int l = 0; l < nfreq; l++) {
        double2 v = make_double2(0.0, 0.0);
        if (live) {
            if (in_c128) {
                v = reinterpret_cast<const double2 *>(Xhat)[(long long)l * M + e];
            } else {
                const float2 f = reinterpret_cast<const float2 *>(Xhat)[(long long)l * M + e];
                v = make_double2(f.x, f.y);
            }
        }
        sx[l * TILE + threadIdx.x] = v;
    }
    __syncthreads();
    if (!live) return;
    for (int n = 0; n <= nh; n++) {
        double A = 0.0, B = 0.0;
        for (int l = 0; l < nfreq; l++) {
            const double2 w = stw[n * nfreq + l];
            const double2 x = sx[l * TILE + threadIdx.x];
            A = fma(x.x, w.x, A);
            B = fma(x.y, w.y, B);
        }
        out[(long long)n * M + e] = sg[n] * (A + B);
        const int m = L - n;
        if (n >= 1 && m != n) out[(long long)m * M + e] = sg[m] * (A - B);
    }
}

// c_l cos(2 pi n l / L), c_l sin(2 pi n l / L) for n <= L/2, l < nfreq, and R^-n / L for n < L: in FP64
// (tw, gsc) or as float pairs (tw32 = (cos hi, lo, sin hi, lo), g32 = (hi, lo))
__global__ void twiddle_half_kernel(int L, int nfreq, double R, double2 *tw, double *gsc, float4 *tw32, float2 *g32) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nh = L / 2;
    if (t < L) {
        const double g = pow(R, -(double)t) / (double)L;
        if (gsc) gsc[t] = g;
        if (g32) g32[t] = make_float2((float)g, (float)(g - (double)(float)g));
    }
    if (t >= (nh + 1) * nfreq) return;
    const int n = t / nfreq, l = t % nfreq;
    const double c = (l != 0 && (l != L / 2 || L % 2 == 1)) ? 2.0 : 1.0;
    double sn, cs;
    sincospi(2.0 * (double)(((long long)n * l) % L) / (double)L, &sn, &cs);
    const double re = c * cs, im = c * sn;
    if (tw) tw[t] = make_double2(re, im);
    if (tw32) tw32[t] = make_float4((float)re, (float)(re - (double)(float)re), (float)im, (float)(im - (double)(float)im));
}

int launch_inverse_transform(sod_context *ctx, const void *Xhat, int in_dtype, int64_t M, int nfreq, int L, double R,
                             void *out, int out_dtype, cudaStream_t stream) {
    SOD_REQUIRE(L >= 1 && nfreq == L / 2 + 1, "inverse transform: nfreq must equal L/2 + 1");
    SOD_REQUIRE(in_dtype == SOD_C128 || in_dtype == SOD_C64, "inverse transform: input must be complex128 or complex64");
    SOD_REQUIRE(out_dtype == SOD_F64 || out_dtype == SOD_F32, "inverse transform: output must be float64 or float32");
    SOD_REQUIRE(R > 0.0 && M >= 0, "inverse transform: bad R or M");
    if (M == 0) return SOD_OK;
    const int in_c128 = in_dtype == SOD_C128;
    if (out_dtype == SOD_F64) {
        const size_t ntw = (size_t)(L / 2 + 1) * nfreq;
        SOD_TRY(ctx->twiddle.ensure(sizeof(double2) * ntw + sizeof(double) * (size_t)L));
        double2 *dtw = ctx->twiddle.as<double2>();
        double *dg = reinterpret_cast<double *>(dtw + ntw);
        const size_t nt = std::max(ntw, (size_t)L);
        twiddle_half_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, stream>>>(L, nfreq, R, dtw, dg, nullptr, nullptr);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        constexpr int TILE = 128;
        const size_t smem = sizeof(double2) * (ntw + (size_t)nfreq * TILE) + sizeof(double) * (size_t)L;
        if (smem > ctx->smem_optin) {
            set_error("inverse transform: too many frequencies for the shared-memory tile");
            return SOD_ERR_UNSUPPORTED;
        }
        SOD_CHECK_CUDA(cudaFuncSetAttribute(inv_transform_f64_kernel<TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        const long long blocks = (M + TILE - 1) / TILE;
        inv_transform_f64_kernel<TILE><<<(unsigned)blocks, TILE, smem, stream>>>(Xhat, in_c128, M, nfreq, L, dtw, dg,
                                                                                 reinterpret_cast<double *>(out));
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        return SOD_OK;
    }
    const size_t ntw = (size_t)(L / 2 + 1) * nfreq;
    SOD_TRY(ctx->twiddle.ensure(sizeof(float4) * ntw + sizeof(float2) * (size_t)L));
    float4 *dtw = ctx->twiddle.as<float4>();
    float2 *dg = reinterpret_cast<float2 *>(dtw + ntw);
    const size_t nt = std::max(ntw, (size_t)L);
    twiddle_half_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, stream>>>(L, nfreq, R, nullptr, nullptr, dtw, dg);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    constexpr int TILE = 128;
    const size_t smem = sizeof(float4) * ntw + sizeof(float2) * (size_t)((L + 1) & ~1) +
                        sizeof(float2) * (size_t)nfreq * TILE * (in_c128 ? 2 : 1);
    if (smem > ctx->smem_optin) {
        set_error("inverse transform: too many frequencies for the shared-memory tile");
        return SOD_ERR_UNSUPPORTED;
    }
    SOD_CHECK_CUDA(cudaFuncSetAttribute(inv_transform_df_kernel<TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long blocks = (M + TILE - 1) / TILE;
    inv_transform_df_kernel<TILE><<<(unsigned)blocks, TILE, smem, stream>>>(Xhat, in_c128, M, nfreq, L, dtw, dg,
                                                                            reinterpret_cast<float *>(out));
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

}  // namespace sod
