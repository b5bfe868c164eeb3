// sod_history.cu -- the per-step history convolution of a CQBEM object on sm_103a.
//
// Replaces the dense loop of ElastodynamicsCQBEMObject::estimate_next_state
// (src/elastodynamics_cqbem_object.cpp:44-48):
//     b = sum_{i=0}^{min(n, K)-1} ( G_{i+1} p_{n-1-i} - H_{i+1} u_{n-1-i} + B_{i+1} a_{n-1-i} )
// (the reference negates H at load, src/elastodynamics_cqbem_matrix_collection.cpp:140).
//
// A history bank keeps everything device-resident:
//   * weights [K][2][nrow][ldw] -- G_k and -H_k, FP32 or BF16 with one FP32 scale per (k, G/H, row)
//     (rows are normalised to max |w| = 1 before rounding), ldw = ncol rounded up to 8 so that
//     every row starts on a 16-byte boundary;
//   * B weights [K][nrow][6] (FP64, small);
//   * a ring of the last K steps' vectors x [K][2][ldw][R] (p, u; zero-padded) and a [K][6][R].
// push() writes the newest step into the ring (one small kernel), convolve() streams the whole
// bank once: HBM-bound at R = 1 (and for FP32 weights at R = 16); 2 * 2K * nrow * ncol * R flops.
//
// convolve: CTA = 8 warps, each warp owns RW rows and splits a column chunk over its 32 lanes
// (4 FP32 or 8 BF16 consecutive columns per lane and step: one 16-byte weight load per row), accumulates in
// FP32 registers over all matrices, and the lanes' partial sums are combined in FP64 with a fixed
// xor tree; a second kernel sums the column chunks in fixed order and adds the B term in FP64.
// Results are bitwise reproducible.
//
// BF16 banks, and FP32 banks with 16 right-hand sides, run on the tensor cores instead
// (sod_history_tc.cu): with 16 right-hand sides the work is a dense contraction (32 flop per
// weight), and with one the tensor cores unpack the BF16 weights for free.  The ring then also keeps
// the history as hi + lo terms (BF16, or FP32 with a TF32-exact hi), transposed for the MMA's
// K-major B operand: [K][2][hi|lo][16][ldw] for R = 16, [K][2][16][ldw] (rows hi, lo, zeros) for R = 1.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdio>
#include <memory>
#include <vector>

#include "sod_internal.h"

using namespace sod;

struct sod_history {
    sod_context *ctx = nullptr;
    int nrow = 0, ncol = 0, K = 0, R = 0, wdtype = SOD_F32, ldw = 0;
    int head = 0;   // ring slot of the next push
    int count = 0;  // steps pushed (saturates at K)
    DevBuf W, scale, Bw, X, A, partial, tmp;
    bool has_b = false;
    int nchunk = 0, cchunk = 0;
    int engine = SOD_HISTORY_ENGINE_AUTO;
    DevBuf Xt, tcpart, derr;
    DevBuf bsolve;            // b of the fused per-step solve  // tensor-core path: BF16 hi/lo history, per-segment partials, error word
    int *err_host = nullptr;  // pinned copy of the error word (written by the finish kernel)
    HistTcPlan plan;          // tensor maps of W and Xt
    WaveletBank *wav = nullptr;  // wavelet-compressed weights (sod_history_create_compressed)
    bool use_tensor() const {
        if (engine == SOD_HISTORY_ENGINE_AUTO) return wdtype == SOD_BF16 || R == 16;
        return engine == SOD_HISTORY_ENGINE_TENSOR_CORES;
    }
    size_t xt_esz() const { return wdtype == SOD_BF16 ? 2 : 4; }
    int xt_rows() const { return R == 16 ? 2 * 16 : 16; }  // history rows per (slot, G|H)
    ~sod_history() {
        if (err_host) cudaFreeHost(err_host);
        wavelet_bank_free(wav);
    }
};

namespace {

constexpr int HIST_THREADS = 256;

// VEC consecutive weights of one row with a single 16-byte load (4 FP32 or 8 BF16), kept packed in
// registers and unpacked per column at use
template <class WT> struct WVec {
    static constexpr int VEC = 16 / sizeof(WT);
};
__device__ __forceinline__ float wget(const uint4 &q, int k, const float *) {
    const unsigned int u = k == 0 ? q.x : k == 1 ? q.y : k == 2 ? q.z : q.w;
    return __uint_as_float(u);
}
__device__ __forceinline__ float wget(const uint4 &q, int k, const __nv_bfloat16 *) {
    const unsigned int u = (k >> 1) == 0 ? q.x : (k >> 1) == 1 ? q.y : (k >> 1) == 2 ? q.z : q.w;
    return __uint_as_float((k & 1) ? (u & 0xffff0000u) : (u << 16));  // bf16 -> f32 is exact
}
__device__ __forceinline__ void load_w(const float *w, float v[4]) {
    const float4 q = __ldg(reinterpret_cast<const float4 *>(w));
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
}
__device__ __forceinline__ void load_w(const __nv_bfloat16 *w, float v[8]) {
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(w));
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = wget(q, k, w);
}

// partial[chunk][row][j] = sum over the used history of this column chunk (FP64 after the lane tree)
// one right-hand side: enough 16-byte loads in flight per SM -- FP32 with 8 rows per warp at 2 CTAs
// per SM, BF16 (whose weights unpack into twice the registers) with 4 rows per warp at 4 CTAs per SM
template <int R, int RW, class WT> constexpr int hist_min_ctas() { return R == 1 ? (RW == 8 ? 2 : 4) : 1; }

// one (column chunk bx, row block by) tile of a bank; shared by the per-bank and the grouped kernels
template <int R, int RW, class WT>
__device__ __forceinline__ void hist_conv_tile(const WT *__restrict__ W, const float *__restrict__ scale,
                                               const float *__restrict__ X, int used, int head, int K, int nrow,
                                               int ldw, int cchunk, double *__restrict__ partial, int bx, int by) {
    constexpr int VEC = WVec<WT>::VEC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = (by * (HIST_THREADS / 32) + warp) * RW;
    if (row0 >= nrow) return;
    const int c0 = bx * cchunk, c1 = min(ldw, c0 + cchunk);
    float acc[RW][R];
#pragma unroll
    for (int r = 0; r < RW; r++)
#pragma unroll
        for (int j = 0; j < R; j++) acc[r][j] = 0.f;
    int rows[RW];
#pragma unroll
    for (int r = 0; r < RW; r++) rows[r] = min(row0 + r, nrow - 1);  // duplicated tail rows are not stored
    for (int i = 0; i < used; i++) {
        const int slot = (head - 1 - i + 2 * K) % K;
        for (int t = 0; t < 2; t++) {
            const size_t mat = (size_t)i * 2 + t;
            const WT *Wm = W + mat * nrow * (size_t)ldw;
            const float *Xm = X + ((size_t)slot * 2 + t) * ldw * (size_t)R;
            float sc[RW];
#pragma unroll
            for (int r = 0; r < RW; r++) sc[r] = scale ? __ldg(scale + mat * nrow + rows[r]) : 1.0f;
            if (R == 1) {
                // one right-hand side: accumulate the matrix's chunk unscaled, scale once per row
                float part[RW];
#pragma unroll
                for (int r = 0; r < RW; r++) part[r] = 0.f;
                for (int c = c0 + VEC * lane; c < c1; c += 32 * VEC) {
                    uint4 wr[RW];
#pragma unroll
                    for (int r = 0; r < RW; r++) wr[r] = __ldg(reinterpret_cast<const uint4 *>(Wm + (size_t)rows[r] * ldw + c));
#pragma unroll
                    for (int q4 = 0; q4 < VEC; q4 += 4) {
                        const float4 v = __ldg(reinterpret_cast<const float4 *>(Xm + c + q4));
                        const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                        for (int q = 0; q < 4; q++)
#pragma unroll
                            for (int r = 0; r < RW; r++) part[r] = fmaf(wget(wr[r], q4 + q, Wm), x[q], part[r]);
                    }
                }
#pragma unroll
                for (int r = 0; r < RW; r++) acc[r][0] = fmaf(part[r], sc[r], acc[r][0]);
            } else {
            for (int c = c0 + VEC * lane; c < c1; c += 32 * VEC) {
                float w[RW][VEC];
#pragma unroll
                for (int r = 0; r < RW; r++) load_w(Wm + (size_t)rows[r] * ldw + c, w[r]);
                if (scale) {
#pragma unroll
                    for (int r = 0; r < RW; r++)
#pragma unroll
                        for (int q = 0; q < VEC; q++) w[r][q] *= sc[r];
                }
#pragma unroll
                for (int q = 0; q < VEC; q++) {
                    float x[R];
#pragma unroll
                    for (int j = 0; j < R; j += 4) {
                        const float4 v = __ldg(reinterpret_cast<const float4 *>(Xm + (size_t)(c + q) * R + j));
                        x[j] = v.x, x[j + 1] = v.y, x[j + 2] = v.z, x[j + 3] = v.w;
                    }
#pragma unroll
                    for (int r = 0; r < RW; r++)
#pragma unroll
                        for (int j = 0; j < R; j++) acc[r][j] = fmaf(w[r][q], x[j], acc[r][j]);
                }
            }
            }
        }
    }
    // lanes -> one value per (row, j) in FP64, fixed xor tree
#pragma unroll
    for (int r = 0; r < RW; r++)
#pragma unroll
        for (int j = 0; j < R; j++) {
            double v = acc[r][j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && row0 + r < nrow) partial[((size_t)bx * nrow + row0 + r) * R + j] = v;
        }
}

template <int R, int RW, class WT>
__global__ void __launch_bounds__(HIST_THREADS, hist_min_ctas<R, RW, WT>()) hist_conv_kernel(const WT *__restrict__ W,
                                                                 const float *__restrict__ scale,
                                                                 const float *__restrict__ X, int used, int head,
                                                                 int K, int nrow, int ldw, int cchunk,
                                                                 double *__restrict__ partial) {
    hist_conv_tile<R, RW, WT>(W, scale, X, used, head, K, nrow, ldw, cchunk, partial, blockIdx.x, blockIdx.y);
}

// b[row][j] = sum_chunks partial + sum_i B_{i+1}[row][:] a_slot[:][j]   (FP64, fixed order)
__device__ __forceinline__ void hist_finish_elem(const double *__restrict__ partial, int nchunk,
                                                 const double *__restrict__ Bw, const double *__restrict__ A, int used,
                                                 int head, int K, int nrow, int R, double *__restrict__ out, int e) {
    const int row = e / R, j = e % R;
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += partial[(size_t)c * nrow * R + e];
    if (Bw) {
        for (int i = 0; i < used; i++) {
            const int slot = (head - 1 - i + 2 * K) % K;
            const double *b = Bw + ((size_t)i * nrow + row) * 6;
            const double *a = A + (size_t)slot * 6 * R;
            for (int c = 0; c < 6; c++) s += b[c] * a[c * R + j];
        }
    }
    out[e] = s;
}
__global__ void hist_finish_kernel(const double *__restrict__ partial, int nchunk, const double *__restrict__ Bw,
                                   const double *__restrict__ A, int used, int head, int K, int nrow, int R,
                                   double *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nrow * R) return;
    hist_finish_elem(partial, nchunk, Bw, A, used, head, K, nrow, R, out, e);
}

// One matrix (nrow x ncol, FP64 or FP32, row-major) -> bank layout, with `sign` and per-row scale.
template <class WT>
__global__ void hist_pack_kernel(const void *__restrict__ src, int src_f64, int nrow, int ncol, int ldw, double sign,
                                 WT *__restrict__ dst, float *__restrict__ scale) {
    const int row = blockIdx.x;
    if (row >= nrow) return;
    const double *s64 = static_cast<const double *>(src) + (size_t)row * ncol;
    const float *s32 = static_cast<const float *>(src) + (size_t)row * ncol;
    float sc = 1.0f;
    if (scale) {  // power-of-two scale that maps max |w| of the row into [0.5, 1)
        __shared__ double red[HIST_THREADS];
        double m = 0.0;
        for (int c = threadIdx.x; c < ncol; c += blockDim.x) m = fmax(m, fabs(src_f64 ? s64[c] : (double)s32[c]));
        red[threadIdx.x] = m;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
            __syncthreads();
        }
        int ex = 0;
        frexp(red[0], &ex);
        sc = red[0] > 0.0 ? ldexpf(1.0f, max(-126, min(127, ex))) : 1.0f;
        if (threadIdx.x == 0) scale[row] = sc;
    }
    const double inv = 1.0 / sc;
    for (int c = threadIdx.x; c < ldw; c += blockDim.x) {
        const double v = c < ncol ? sign * (src_f64 ? s64[c] : (double)s32[c]) * inv : 0.0;
        if constexpr (sizeof(WT) == 4)
            dst[(size_t)row * ldw + c] = (float)v;
        else
            dst[(size_t)row * ldw + c] = __double2bfloat16(v);
    }
}

// hi + lo split of one history value for the tensor cores: BF16 terms, or FP32 terms whose hi keeps
// the top 19 bits (exact in TF32; the tensor core reads only those bits of lo as well)
__device__ __forceinline__ void split_x(double v, __nv_bfloat16 *h, __nv_bfloat16 *l) {
    *h = __double2bfloat16(v);
    *l = __double2bfloat16(v - (double)__bfloat162float(*h));
}
__device__ __forceinline__ void split_x(double v, float *h, float *l) {
    *h = __uint_as_float(__float_as_uint((float)v) & 0xffffe000u);
    *l = (float)(v - (double)*h);
}

// newest step -> ring slot: x[slot][0] = p, x[slot][1] = u (FP32, zero padded), a[slot] = a;
// with Xt also the split x = hi + lo, transposed: Xt[slot][t][hi|lo][j][c] for R = 16,
// Xt[slot][t][0 = hi | 1 = lo][c] for R = 1
template <class XT>
__global__ void hist_push_kernel(const double *__restrict__ p, const double *__restrict__ u,
                                 const double *__restrict__ a, int ncol, int ldw, int R, int slot,
                                 float *__restrict__ X, double *__restrict__ A, XT *__restrict__ Xt) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < ldw * R) {
        const int c = e / R, j = e % R;
        float *x = X + (size_t)slot * 2 * ldw * R;
        x[e] = c < ncol ? (float)p[e] : 0.0f;
        x[(size_t)ldw * R + e] = c < ncol ? (float)u[e] : 0.0f;
        if (Xt) {
            for (int t = 0; t < 2; t++) {
                const double v = c < ncol ? (t == 0 ? p[e] : u[e]) : 0.0;
                XT hi, lo;
                split_x(v, &hi, &lo);
                XT *xt = Xt + ((size_t)slot * 2 + t) * (R == 16 ? 32 : 16) * ldw;
                xt[(size_t)j * ldw + c] = hi;
                xt[(size_t)(R == 16 ? 16 + j : 1) * ldw + c] = lo;
            }
        }
    }
    if (e < 6 * R) A[(size_t)slot * 6 * R + e] = a ? a[e] : 0.0;
}

// ---- one step of several banks in three launches (the request loop's grouped steps) -----------------
// FP32 banks with one right-hand side on the CUDA-core engine.  Each bank's push, convolution tiles
// and finish run the same device code with the same tiling as sod_history_push + sod_history_convolve,
// so a bank's result is bitwise the same in a group and alone.
struct GroupBank {
    const float *W;
    float *X;
    double *partial, *A, *out;
    const double *Bw, *p, *u;
    int used, head, slot, K, nrow, ncol, ldw, cchunk, nchunk, gy;
};
struct GroupArgs {
    int n;
    int push_off[HIST_GROUP_MAX + 1], conv_off[HIST_GROUP_MAX + 1], fin_off[HIST_GROUP_MAX + 1];
    GroupBank b[HIST_GROUP_MAX];
};
static_assert(sizeof(GroupArgs) <= 16000, "grouped-step arguments exceed the kernel parameter space");
__device__ __forceinline__ int group_of(const int *off, int n, int e) {
    int g = 0;
    while (g + 1 < n && off[g + 1] <= e) g++;
    return g;
}
__global__ void hist_group_push_kernel(const __grid_constant__ GroupArgs ga) {
    const int e0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (e0 >= ga.push_off[ga.n]) return;
    const int g = group_of(ga.push_off, ga.n, e0);
    const GroupBank &b = ga.b[g];
    const int e = e0 - ga.push_off[g];
    if (e < b.ldw) {
        float *x = b.X + (size_t)b.slot * 2 * b.ldw;
        x[e] = e < b.ncol ? (float)b.p[e] : 0.0f;
        x[(size_t)b.ldw + e] = e < b.ncol ? (float)b.u[e] : 0.0f;
    }
    if (e < 6) b.A[(size_t)b.slot * 6 + e] = 0.0;
}
__global__ void __launch_bounds__(HIST_THREADS, hist_min_ctas<1, 8, float>()) hist_group_conv_kernel(
    const __grid_constant__ GroupArgs ga) {
    const int g = group_of(ga.conv_off, ga.n, blockIdx.x);
    const GroupBank &b = ga.b[g];
    const int t = blockIdx.x - ga.conv_off[g];
    hist_conv_tile<1, 8, float>(b.W, nullptr, b.X, b.used, b.head, b.K, b.nrow, b.ldw, b.cchunk, b.partial,
                                t % b.nchunk, t / b.nchunk);
}
__global__ void hist_group_finish_kernel(const __grid_constant__ GroupArgs ga) {
    const int e0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (e0 >= ga.fin_off[ga.n]) return;
    const int g = group_of(ga.fin_off, ga.n, e0);
    const GroupBank &b = ga.b[g];
    hist_finish_elem(b.partial, b.nchunk, b.Bw, b.A, b.used, b.head, b.K, b.nrow, 1, b.out, e0 - ga.fin_off[g]);
}

template <int R, int RW, class WT>
void launch_conv(const sod_history *h, cudaStream_t st, int used) {
    const int rows_per_cta = (HIST_THREADS / 32) * RW;
    const dim3 grid(h->nchunk, (h->nrow + rows_per_cta - 1) / rows_per_cta);
    hist_conv_kernel<R, RW, WT><<<grid, HIST_THREADS, 0, st>>>(
        h->W.as<WT>(), h->wdtype == SOD_BF16 ? h->scale.as<float>() : nullptr, h->X.as<float>(), used, h->head, h->K,
        h->nrow, h->ldw, h->cchunk, h->partial.as<double>());
}

}  // namespace

extern "C" {

int sod_history_create(sod_context *ctx, int nrow, int ncol, int K, int R, int weight_dtype, sod_history **out) {
    SOD_REQUIRE(ctx && out, "null argument");
    SOD_REQUIRE(nrow >= 1 && ncol >= 1 && K >= 1, "history bank needs nrow, ncol, K >= 1");
    SOD_REQUIRE(R == 1 || R == 16, "right-hand sides per step must be 1 or 16");
    SOD_REQUIRE(weight_dtype == SOD_F32 || weight_dtype == SOD_BF16, "weights are SOD_F32 or SOD_BF16");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<sod_history>();
    h->ctx = ctx;
    h->nrow = nrow, h->ncol = ncol, h->K = K, h->R = R, h->wdtype = weight_dtype;
    h->ldw = (ncol + 7) / 8 * 8;
    const size_t esz = weight_dtype == SOD_F32 ? 4 : 2;
    SOD_TRY(h->W.ensure(esz * (size_t)K * 2 * nrow * h->ldw));
    SOD_CHECK_CUDA(cudaMemsetAsync(h->W.p, 0, h->W.bytes, ctx->stream));
    if (weight_dtype == SOD_BF16) {
        SOD_TRY(h->scale.ensure(sizeof(float) * (size_t)K * 2 * nrow));
        SOD_CHECK_CUDA(cudaMemsetAsync(h->scale.p, 0, h->scale.bytes, ctx->stream));
    }
    SOD_TRY(h->X.ensure(sizeof(float) * (size_t)K * 2 * h->ldw * R));
    SOD_CHECK_CUDA(cudaMemsetAsync(h->X.p, 0, h->X.bytes, ctx->stream));
    SOD_TRY(h->A.ensure(sizeof(double) * (size_t)K * 6 * R));
    SOD_CHECK_CUDA(cudaMemsetAsync(h->A.p, 0, h->A.bytes, ctx->stream));
    // column chunks: enough CTAs to cover the SMs several times over
    const int RW = (R == 1 && weight_dtype == SOD_F32) ? 8 : 4;
    const int row_ctas = (nrow + 8 * RW - 1) / (8 * RW);
    const int want = std::max(1, (ctx->num_sms * 8 + row_ctas - 1) / row_ctas);
    const int step = weight_dtype == SOD_F32 ? 128 : 256;  // columns a warp covers per step
    const int steps = (h->ldw + step - 1) / step;
    h->nchunk = std::max(1, std::min(want, steps));
    h->cchunk = ((steps + h->nchunk - 1) / h->nchunk) * step;
    h->nchunk = (h->ldw + h->cchunk - 1) / h->cchunk;
    SOD_TRY(h->partial.ensure(sizeof(double) * (size_t)h->nchunk * nrow * R));
    {  // tensor-core path (either engine can be selected later)
        SOD_TRY(h->Xt.ensure(h->xt_esz() * (size_t)K * 2 * h->xt_rows() * h->ldw));
        SOD_CHECK_CUDA(cudaMemsetAsync(h->Xt.p, 0, h->Xt.bytes, ctx->stream));
        SOD_TRY(h->tcpart.ensure(sizeof(float) * history_tc_partial_floats(ctx->num_sms, nrow, R)));
        SOD_TRY(h->derr.ensure(sizeof(int)));
        SOD_CHECK_CUDA(cudaMemsetAsync(h->derr.p, 0, sizeof(int), ctx->stream));
        if (cudaMallocHost(&h->err_host, sizeof(int)) != cudaSuccess) {
            h->err_host = nullptr;
            set_error("cudaMallocHost failed for the history error word");
            return SOD_ERR_OOM;
        }
        *h->err_host = 0;
        SOD_TRY(history_tc_plan(&h->plan, h->W.p, h->Xt.p, nrow, ncol, h->ldw, K, R, weight_dtype == SOD_F32));
    }
    *out = h.release();
    return SOD_OK;
}

int sod_history_set_weights(sod_history *h, int k, const void *G_k, const void *H_k, int in_dtype) {
    SOD_REQUIRE(h, "null history bank");
    SOD_REQUIRE(k >= 1 && k <= h->K, "weight index k must be in 1..K");
    SOD_REQUIRE(G_k && H_k, "null weight matrix");
    SOD_REQUIRE(in_dtype == SOD_F64 || in_dtype == SOD_F32, "input matrices are SOD_F64 or SOD_F32");
    sod_context *ctx = h->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t isz = in_dtype == SOD_F64 ? 8 : 4, bytes = isz * (size_t)h->nrow * h->ncol;
    const void *src[2] = {G_k, H_k};
    if (h->wav) {
        for (int t = 0; t < 2; t++) {
            const void *d = src[t];
            if (!is_device_pointer(d)) {
                SOD_TRY(h->tmp.ensure(bytes));
                SOD_CHECK_CUDA(cudaMemcpyAsync(h->tmp.p, d, bytes, cudaMemcpyHostToDevice, ctx->stream));
                d = h->tmp.p;
            }
            SOD_TRY(wavelet_set_block(ctx, h->wav, 2 * (k - 1) + t, d, in_dtype == SOD_F64, t == 0 ? 1.0 : -1.0));
        }
        return SOD_OK;
    }
    for (int t = 0; t < 2; t++) {
        const void *d = src[t];
        if (!is_device_pointer(d)) {
            SOD_TRY(h->tmp.ensure(bytes));
            SOD_CHECK_CUDA(cudaMemcpyAsync(h->tmp.p, d, bytes, cudaMemcpyHostToDevice, ctx->stream));
            d = h->tmp.p;
        }
        const size_t mat = (size_t)(k - 1) * 2 + t;
        const double sign = t == 0 ? 1.0 : -1.0;
        if (h->wdtype == SOD_F32)
            hist_pack_kernel<float><<<h->nrow, HIST_THREADS, 0, ctx->stream>>>(
                d, in_dtype == SOD_F64, h->nrow, h->ncol, h->ldw, sign, h->W.as<float>() + mat * h->nrow * h->ldw,
                nullptr);
        else
            hist_pack_kernel<__nv_bfloat16><<<h->nrow, HIST_THREADS, 0, ctx->stream>>>(
                d, in_dtype == SOD_F64, h->nrow, h->ncol, h->ldw, sign,
                h->W.as<__nv_bfloat16>() + mat * h->nrow * h->ldw, h->scale.as<float>() + mat * h->nrow);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
        if (d == h->tmp.p) SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // tmp is reused
    }
    return SOD_OK;
}

int sod_history_set_b(sod_history *h, int k, const double *B_k) {
    SOD_REQUIRE(h && B_k, "null argument");
    SOD_REQUIRE(k >= 1 && k <= h->K, "weight index k must be in 1..K");
    sod_context *ctx = h->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    if (!h->has_b) {
        SOD_TRY(h->Bw.ensure(sizeof(double) * (size_t)h->K * h->nrow * 6));
        SOD_CHECK_CUDA(cudaMemsetAsync(h->Bw.p, 0, h->Bw.bytes, ctx->stream));
        h->has_b = true;
    }
    SOD_CHECK_CUDA(cudaMemcpyAsync(h->Bw.as<double>() + (size_t)(k - 1) * h->nrow * 6, B_k,
                                   sizeof(double) * (size_t)h->nrow * 6, cudaMemcpyDefault, ctx->stream));
    return SOD_OK;
}

int sod_history_push(sod_history *h, const double *p, const double *u, const double *a) {
    SOD_REQUIRE(h && p && u, "null argument");
    sod_context *ctx = h->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t vb = sizeof(double) * (size_t)h->ncol * h->R, ab = sizeof(double) * 6 * (size_t)h->R;
    const double *dp = p, *du = u, *da = a;
    const bool hp = !is_device_pointer(p), hu = !is_device_pointer(u), ha = a && !is_device_pointer(a);
    if (hp || hu || ha) {
        SOD_TRY(h->tmp.ensure(2 * vb + ab));
        char *t = h->tmp.as<char>();
        if (hp) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(t, p, vb, cudaMemcpyHostToDevice, ctx->stream));
            dp = reinterpret_cast<const double *>(t);
        }
        if (hu) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(t + vb, u, vb, cudaMemcpyHostToDevice, ctx->stream));
            du = reinterpret_cast<const double *>(t + vb);
        }
        if (ha) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(t + 2 * vb, a, ab, cudaMemcpyHostToDevice, ctx->stream));
            da = reinterpret_cast<const double *>(t + 2 * vb);
        }
    }
    const int n = h->ldw * h->R;
    if (h->wav)
        SOD_TRY(wavelet_push(ctx, h->wav, dp, du, da, h->head, h->A.as<double>() + (size_t)h->head * 6));
    else if (h->wdtype == SOD_BF16)
        hist_push_kernel<__nv_bfloat16><<<(n + 255) / 256, 256, 0, ctx->stream>>>(
            dp, du, da, h->ncol, h->ldw, h->R, h->head, h->X.as<float>(), h->A.as<double>(),
            h->use_tensor() ? h->Xt.as<__nv_bfloat16>() : nullptr);
    else
        hist_push_kernel<float><<<(n + 255) / 256, 256, 0, ctx->stream>>>(
            dp, du, da, h->ncol, h->ldw, h->R, h->head, h->X.as<float>(), h->A.as<double>(),
            h->use_tensor() ? h->Xt.as<float>() : nullptr);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    h->head = (h->head + 1) % h->K;
    h->count = std::min(h->count + 1, h->K);
    if (hp || hu || ha) SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // staging is reused
    return SOD_OK;
}

int sod_history_convolve(sod_history *h, double *b_out) {
    SOD_REQUIRE(h && b_out, "null argument");
    sod_context *ctx = h->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const bool host = !is_device_pointer(b_out);
    const size_t ob = sizeof(double) * (size_t)h->nrow * h->R;
    double *dst = b_out;
    if (host) {
        SOD_TRY(ctx->staging.ensure(ob));
        dst = ctx->staging.as<double>();
    }
    const int used = h->count;
    if (h->wav) {
        SOD_TRY(wavelet_convolve(ctx, h->wav, used, h->head, h->partial.as<double>()));
    } else if (h->use_tensor()) {
        // a bounded wait that expired in an earlier convolution (read from the pinned copy)
        if (*(volatile int *)h->err_host) {
            set_error("tensor-core history convolution: a bounded mbarrier wait expired (code " +
                      std::to_string(*(volatile int *)h->err_host) + ")");
            return SOD_ERR_TIMEOUT;
        }
        SOD_TRY(launch_history_tc(ctx, &h->plan, h->wdtype == SOD_BF16 ? h->scale.as<float>() : nullptr, used, h->head, h->tcpart.as<float>(),
                                  h->has_b ? h->Bw.as<double>() : nullptr, h->A.as<double>(), dst, h->derr.as<int>(),
                                  h->err_host, ctx->stream));
        if (host) {
            SOD_CHECK_CUDA(cudaMemcpyAsync(b_out, dst, ob, cudaMemcpyDeviceToHost, ctx->stream));
            SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
            if (*(volatile int *)h->err_host) {
                set_error("tensor-core history convolution: a bounded mbarrier wait expired (code " +
                          std::to_string(*(volatile int *)h->err_host) + ")");
                return SOD_ERR_TIMEOUT;
            }
        }
        return SOD_OK;
    } else if (used > 0) {
        const bool bf = h->wdtype == SOD_BF16;
        if (h->R == 1)
            bf ? launch_conv<1, 4, __nv_bfloat16>(h, ctx->stream, used) : launch_conv<1, 8, float>(h, ctx->stream, used);
        else
            bf ? launch_conv<16, 4, __nv_bfloat16>(h, ctx->stream, used) : launch_conv<16, 4, float>(h, ctx->stream, used);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    } else {
        SOD_CHECK_CUDA(cudaMemsetAsync(h->partial.p, 0, h->partial.bytes, ctx->stream));
    }
    const int n = h->nrow * h->R;
    hist_finish_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(h->partial.as<double>(), h->nchunk,
                                                                h->has_b ? h->Bw.as<double>() : nullptr,
                                                                h->A.as<double>(), used, h->head, h->K, h->nrow,
                                                                h->R, dst);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    if (host) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(b_out, dst, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return SOD_OK;
}

int sod_history_convolve_solve(sod_history *h, sod_solver *s, double *u_out) {
    SOD_REQUIRE(h && s && u_out, "null argument");
    SOD_REQUIRE(solver_size(s) == h->nrow, "the solver's matrix size must equal the bank's row count");
    sod_context *ctx = h->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t bytes = sizeof(double) * (size_t)h->nrow * h->R;
    SOD_TRY(h->bsolve.ensure(2 * bytes));
    double *b = h->bsolve.as<double>(), *u = b + (size_t)h->nrow * h->R;
    SOD_TRY(sod_history_convolve(h, b));  // device output: no synchronisation
    const bool host = !is_device_pointer(u_out);
    SOD_TRY(solver_apply_device(s, h->R, b, host ? u : u_out));
    if (host) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(u_out, u, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return SOD_OK;
}

int sod_history_set_engine(sod_history *h, int engine) {
    SOD_REQUIRE(h, "null history bank");
    SOD_REQUIRE(engine == SOD_HISTORY_ENGINE_AUTO || engine == SOD_HISTORY_ENGINE_CUDA_CORES ||
                    engine == SOD_HISTORY_ENGINE_TENSOR_CORES,
                "engine must be SOD_HISTORY_ENGINE_AUTO, _CUDA_CORES or _TENSOR_CORES");
    if (h->wav) {
        SOD_REQUIRE(engine != SOD_HISTORY_ENGINE_TENSOR_CORES,
                    "a wavelet-compressed bank runs its sparse products on the CUDA cores");
        return SOD_OK;
    }
    const bool before = h->use_tensor();
    h->engine = engine;
    if (h->use_tensor() != before) {
        // the two engines keep the history in different ring layouts: switching clears the ring
        h->head = 0;
        h->count = 0;
    }
    return SOD_OK;
}

int sod_history_reset(sod_history *h) {
    SOD_REQUIRE(h, "null history bank");
    h->head = 0;
    h->count = 0;
    return SOD_OK;
}

int sod_history_bytes(const sod_history *h, int64_t *weight_bytes) {
    SOD_REQUIRE(h && weight_bytes, "null argument");
    *weight_bytes = h->wav ? wavelet_bytes(h->wav) : (int64_t)(h->W.bytes + h->scale.bytes);
    return SOD_OK;
}

int sod_history_create_compressed(sod_context *ctx, int nV, int K, double ratio, sod_history **out) {
    SOD_REQUIRE(ctx && out, "null argument");
    SOD_REQUIRE(nV >= 1 && K >= 1, "compressed history bank needs nV, K >= 1");
    SOD_REQUIRE(ratio > 0.0 && ratio <= 1.0, "compression ratio must be in (0, 1]");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    *out = nullptr;
    auto h = std::make_unique<sod_history>();
    h->ctx = ctx;
    h->nrow = h->ncol = 3 * nV, h->K = K, h->R = 1, h->wdtype = SOD_F64;
    h->ldw = h->ncol;
    h->engine = SOD_HISTORY_ENGINE_CUDA_CORES;
    SOD_TRY(wavelet_bank_create(ctx, nV, K, ratio, &h->wav));
    SOD_TRY(h->A.ensure(sizeof(double) * (size_t)K * 6));
    SOD_CHECK_CUDA(cudaMemsetAsync(h->A.p, 0, h->A.bytes, ctx->stream));
    h->nchunk = 1;  // the reconstructed product is the finish kernel's single partial
    SOD_TRY(h->partial.ensure(sizeof(double) * (size_t)h->nrow));
    *out = h.release();
    return SOD_OK;
}

int sod_history_compressed_matrix(sod_history *h, int k, int which, int64_t *nnz, int32_t *row_ptr, int32_t *col,
                                  double *val) {
    SOD_REQUIRE(h && nnz, "null argument");
    SOD_REQUIRE(h->wav, "not a compressed history bank");
    SOD_REQUIRE(k >= 1 && k <= h->K && (which == 0 || which == 1), "k must be in 1..K and which 0 (G) or 1 (H)");
    SOD_CHECK_CUDA(cudaSetDevice(h->ctx->device));
    return wavelet_block(h->wav, 2 * (k - 1) + which, nnz, row_ptr, col, val, h->ctx->stream);
}

int sod_history_write_cpmat(sod_history *h, int k, int which, const char *path) {
    SOD_REQUIRE(h && path, "null argument");
    SOD_REQUIRE(h->wav, "not a compressed history bank");
    SOD_REQUIRE(k >= 1 && k <= h->K && (which == 0 || which == 1), "k must be in 1..K and which 0 (G) or 1 (H)");
    SOD_CHECK_CUDA(cudaSetDevice(h->ctx->device));
    int N = 0, L = 0;
    wavelet_dims(h->wav, &N, &L);
    int64_t nnz = 0;
    SOD_TRY(wavelet_block(h->wav, 2 * (k - 1) + which, &nnz, nullptr, nullptr, nullptr, h->ctx->stream));
    std::vector<int32_t> rp(L + 1), col(nnz);
    std::vector<double> val(nnz);
    SOD_TRY(wavelet_block(h->wav, 2 * (k - 1) + which, &nnz, rp.data(), col.data(), val.data(), h->ctx->stream));
    // save_compressed_matrix (include/wavelets.hpp:474-502): int N; int64 rows, cols, nonZeros,
    // outerSize, innerSize; values; the outerSize row starts; column indices
    FILE *f = fopen(path, "wb");
    if (!f) {
        set_error(std::string("cannot open for writing: ") + path);
        return SOD_ERR_INVALID_ARG;
    }
    const int64_t hdr[5] = {L, L, nnz, L, L};
    bool ok = fwrite(&N, sizeof(int), 1, f) == 1 && fwrite(hdr, sizeof(int64_t), 5, f) == 5 &&
              fwrite(val.data(), sizeof(double), nnz, f) == (size_t)nnz &&
              fwrite(rp.data(), sizeof(int32_t), L, f) == (size_t)L &&
              fwrite(col.data(), sizeof(int32_t), nnz, f) == (size_t)nnz;
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("write failed: ") + path);
        return SOD_ERR_INVALID_ARG;
    }
    return SOD_OK;
}

int sod_history_destroy(sod_history *h) {
    if (h) {
        cudaSetDevice(h->ctx->device);
        delete h;
    }
    return SOD_OK;
}

}  // extern "C"

namespace sod {
bool history_groupable(const sod_history *h) {
    return h && !h->wav && h->wdtype == SOD_F32 && h->R == 1 && !h->use_tensor() && h->ctx;
}
// One step of each of n banks (all groupable, distinct, on contexts sharing ctx's stream): push p[g], u[g]
// (device, ncol doubles) and b[g] (device, nrow doubles) = the convolution, in three launches.
int history_step_group(sod_context *ctx, sod_history *const *banks, int n, const double *const *p,
                       const double *const *u, double *const *b) {
    SOD_REQUIRE(n >= 1 && n <= HIST_GROUP_MAX, "group of 1..HIST_GROUP_MAX banks");
    GroupArgs ga{};
    ga.n = n;
    int push = 0, conv = 0, fin = 0;
    for (int g = 0; g < n; g++) {
        sod_history *h = banks[g];
        SOD_REQUIRE(history_groupable(h), "grouped steps need FP32 banks with one right-hand side");
        for (int q = 0; q < g; q++) SOD_REQUIRE(banks[q] != h, "a bank appears twice in one group");
        const int rows_per_cta = (HIST_THREADS / 32) * 8;
        GroupBank &gb = ga.b[g];
        gb.W = h->W.as<float>();
        gb.X = h->X.as<float>();
        gb.partial = h->partial.as<double>();
        gb.A = h->A.as<double>();
        gb.out = b[g];
        gb.Bw = h->has_b ? h->Bw.as<double>() : nullptr;
        gb.p = p[g];
        gb.u = u[g];
        gb.slot = h->head;
        gb.head = (h->head + 1) % h->K;
        gb.used = std::min(h->count + 1, h->K);
        gb.K = h->K, gb.nrow = h->nrow, gb.ncol = h->ncol, gb.ldw = h->ldw, gb.cchunk = h->cchunk, gb.nchunk = h->nchunk;
        gb.gy = (h->nrow + rows_per_cta - 1) / rows_per_cta;
        ga.push_off[g] = push, ga.conv_off[g] = conv, ga.fin_off[g] = fin;
        push += std::max(h->ldw, 6);
        conv += h->nchunk * gb.gy;
        fin += h->nrow;
    }
    ga.push_off[n] = push, ga.conv_off[n] = conv, ga.fin_off[n] = fin;
    cudaStream_t st = ctx->stream;
    hist_group_push_kernel<<<(push + 255) / 256, 256, 0, st>>>(ga);
    hist_group_conv_kernel<<<conv, HIST_THREADS, 0, st>>>(ga);
    hist_group_finish_kernel<<<(fin + 255) / 256, 256, 0, st>>>(ga);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count(3);
    for (int g = 0; g < n; g++) {
        banks[g]->head = ga.b[g].head;
        banks[g]->count = ga.b[g].used;
    }
    return SOD_OK;
}
}  // namespace sod
