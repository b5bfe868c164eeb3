// sod_wavelet.cu -- wavelet-compressed history weights (Haar non-standard form), on the device.
//
// Replaces CompressedMatrix<1>, CompressedVector<1> and CompressedMatrixVectorProduct<1>
// (include/wavelets.hpp:163-283, 337-436) as the compressed history of ElastodynamicsCQBEMObject uses
// them (src/elastodynamics_cqbem_object.cpp:31-41, 217-226; matrices built at
// src/elastodynamics_cqbem_matrix_collection.cpp:95-131).  The reference instantiates the Daubechies
// basis with M = 1, i.e. Haar: h = (1/sqrt2, 1/sqrt2), g = (1/sqrt2, -1/sqrt2).
//
// Per weight matrix (set up once):
//   1. P (sign W) P^T with the dof permutation P: i -> (i / 3) + (i % 3) nV
//      (src/elastics_bem_matrix_collection.cpp:25-29), zero-padded to Np = 2^ceil(log2 3nV);
//   2. the non-standard 2-D Haar decomposition, level by level: alpha = g g, beta = g h, gamma = h g
//      and the next scale block h h of each 2 x 2 cell.  Every sum runs in the reference's order
//      (k outer, m inner, (f_k f_m) s added to a running sum from zero) with IEEE round-to-nearest
//      multiplies and adds (no contraction), so the coefficients are bit-identical to a plain FP64
//      evaluation of the same expressions;
//   3. the (int)(N^2 ratio) coefficients of largest magnitude are kept (all nonzero ones if that is
//      <= 0), found by an MSB radix select on the bit patterns of |v|.  Ties at the threshold are
//      kept in (row, column) order; the reference's heap keeps an arbitrary subset of them;
//   4. the kept entries as CSR of the (2Np-2)^2 matrix D, columns ascending in each row (the
//      reference's row-major Eigen::SparseMatrix storage order).
// Candidate coefficients are stored row by row of D: row offset+i of a level holds alpha(i, .) then
// beta(i, .) (columns offset + j, j < 2 size), row offset+size+i holds gamma(i, .) (columns
// offset + j, j < size), and the last row also holds the final scale coefficient.  A row's
// candidates are contiguous, and column = first column of the row's level + position in the row.
//
// Per time step:
//   push: the permuted, padded p and u are decomposed (detail then scale coefficients per level,
//         2Np-2 values each) into a ring of the last K steps;
//   convolve: all K x {G, -H} blocks are merged into one CSR whose column word packs (block << 15 |
//         column), so one SpMV over fixed-size chunks of every row reads each weight once; chunk
//         sums and row sums run in a fixed order.  One CTA then reconstructs the vector level by
//         level and applies P^T; the B terms are added by the history bank's finish kernel.
// The product is one FP64 FMA per 12 bytes of kept coefficients: at the HBM rate that is about the
// whole FP64 FMA rate of GB300, so the FP64 pipe, not HBM, bounds this kernel.
#include <cmath>
#include <vector>

#include "sod_internal.h"

using namespace sod;

namespace {

constexpr double HAAR = 0.70710678118654752440;  // M_SQRT1_2
constexpr int COL_BITS = 15;                      // columns of D < 2^15 (Np <= 16384)
constexpr int CHUNK = 2048;                       // nonzeros per SpMV warp task
constexpr int RADIX_BITS = 12;

__device__ __forceinline__ int perm_inv(int q, int nV) { return 3 * (q % nV) + q / nV; }  // dof at position q

// one level of the non-standard decomposition.  Level 0 reads W (FP64 or FP32, row-major N x N)
// through the permutation, zero-padded; deeper levels read the previous scale block s (2size)^2.
__global__ void haar_level_kernel(const void *__restrict__ W, int w_f64, int nV, double sign,
                                  const double *__restrict__ s, int size, double *__restrict__ coef,
                                  double *__restrict__ snew) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (l >= size) return;
    const int n2 = 2 * size, N = 3 * nV;
    double x[2][2];
    for (int k = 0; k < 2; k++)
        for (int m = 0; m < 2; m++) {
            const int p = 2 * i + k, q = 2 * l + m;
            if (W) {
                double v = 0.0;
                if (p < N && q < N) {
                    const size_t e = (size_t)perm_inv(p, nV) * N + perm_inv(q, nV);
                    v = w_f64 ? static_cast<const double *>(W)[e] : (double)static_cast<const float *>(W)[e];
                    v = sign * v;  // exact (sign is +-1)
                }
                x[k][m] = v;
            } else {
                x[k][m] = s[(size_t)p * n2 + q];
            }
        }
    const double h[2] = {HAAR, HAAR}, g[2] = {HAAR, -HAAR};
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int k = 0; k < 2; k++)
        for (int m = 0; m < 2; m++) {
            a = __dadd_rn(a, __dmul_rn(__dmul_rn(g[k], g[m]), x[k][m]));
            b = __dadd_rn(b, __dmul_rn(__dmul_rn(g[k], h[m]), x[k][m]));
            c = __dadd_rn(c, __dmul_rn(__dmul_rn(h[k], g[m]), x[k][m]));
            d = __dadd_rn(d, __dmul_rn(__dmul_rn(h[k], h[m]), x[k][m]));
        }
    coef[(size_t)i * n2 + l] = a;
    coef[(size_t)i * n2 + size + l] = b;
    coef[(size_t)n2 * size + (size_t)i * size + l] = c;
    snew[(size_t)i * size + l] = d;
}

__device__ __forceinline__ unsigned long long mag_key(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}

// histogram of the digit (key >> shift) & (2^width - 1) over nonzero keys whose bits above
// shift + width equal `prefix` (CTA-private shared histogram, flushed with integer atomics)
__global__ void radix_hist_kernel(const double *__restrict__ coef, long long n, int shift, int width,
                                  unsigned long long prefix, unsigned int *__restrict__ hist) {
    __shared__ unsigned int sh[1 << RADIX_BITS];
    const int nb = 1 << width;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    const int hi = shift + width;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const unsigned long long key = mag_key(coef[e]);
        if (key == 0) continue;
        if (hi < 64 && (key >> hi) != prefix) continue;
        atomicAdd(&sh[(key >> shift) & (unsigned long long)(nb - 1)], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nb; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

// per row of D: candidates above the threshold and equal to it (t = 0: nonzero candidates)
__global__ void row_count_kernel(const double *__restrict__ coef, const long long *__restrict__ cand_ptr, int L,
                                 unsigned long long t, int *__restrict__ gt, int *__restrict__ eq) {
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= L) return;
    int ng = 0, ne = 0;
    for (long long e = cand_ptr[r] + lane; e < cand_ptr[r + 1]; e += 32) {
        const unsigned long long key = mag_key(coef[e]);
        ng += key > t;
        ne += t > 0 && key == t;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ng += __shfl_xor_sync(0xffffffffu, ng, o);
        ne += __shfl_xor_sync(0xffffffffu, ne, o);
    }
    if (lane == 0) {
        gt[r] = ng;
        eq[r] = ne;
    }
}

// kept entries of row r in candidate order: key > t, or key == t among the first need_eq ties
__global__ void row_write_kernel(const double *__restrict__ coef, const long long *__restrict__ cand_ptr,
                                 const int *__restrict__ col0, int L, unsigned long long t, long long need_eq,
                                 const long long *__restrict__ eq_before, const int *__restrict__ row_ptr,
                                 int *__restrict__ col, double *__restrict__ val) {
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= L) return;
    const long long c0 = cand_ptr[r], c1 = cand_ptr[r + 1];
    long long eqr = eq_before[r];
    int pos = row_ptr[r];
    const unsigned lt = (1u << lane) - 1u;
    for (long long base = c0; base < c1; base += 32) {
        const long long e = base + lane;
        double v = 0.0;
        unsigned long long key = 0;
        if (e < c1) {
            v = coef[e];
            key = mag_key(v);
        }
        const bool is_eq = e < c1 && t > 0 && key == t;
        const unsigned eqm = __ballot_sync(0xffffffffu, is_eq);
        const bool sel = e < c1 && (key > t || (is_eq && eqr + __popc(eqm & lt) < need_eq));
        const unsigned sm = __ballot_sync(0xffffffffu, sel);
        if (sel) {
            const int o = pos + __popc(sm & lt);
            col[o] = col0[r] + (int)(e - c0);
            val[o] = v;
        }
        pos += __popc(sm);
        eqr += __popc(eqm);
    }
}

struct BlockPtrs {  // per block b = 2 (k - 1) + t: CSR arrays (null if the block is empty)
    const int *ptr;
    const int *col;
    const double *val;
};

// merged CSR: row r = block 0's row r, block 1's row r, ... (columns packed with the block index)
__global__ void merge_kernel(const BlockPtrs *__restrict__ blk, int nblk, int L, const long long *__restrict__ mptr,
                             unsigned int *__restrict__ mcol, double *__restrict__ mval) {
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= L) return;
    long long o = mptr[r];
    for (int b = 0; b < nblk; b++) {
        const BlockPtrs B = blk[b];
        if (!B.ptr) continue;
        const int s = B.ptr[r], e = B.ptr[r + 1];
        for (int j = s + lane; j < e; j += 32) {
            mcol[o + (j - s)] = ((unsigned)b << COL_BITS) | (unsigned)B.col[j];
            mval[o + (j - s)] = B.val[j];
        }
        o += e - s;
    }
}

// the permuted, padded vector (p for CTA 0, u for CTA 1) -> detail and scale coefficients per level
// into the ring slot; CTA 0 also stores a (6 values, zeros if absent)
__global__ void __launch_bounds__(1024) wav_push_kernel(const double *__restrict__ p, const double *__restrict__ u,
                                                        const double *__restrict__ a, int nV, int Np,
                                                        double *__restrict__ xslot, double *__restrict__ aslot) {
    extern __shared__ double s0[];
    const double *x = blockIdx.x == 0 ? p : u;
    double *out = xslot + (size_t)blockIdx.x * (2 * Np - 2);
    const int N = 3 * nV;
    for (int q = threadIdx.x; q < Np; q += blockDim.x) s0[q] = q < N ? x[perm_inv(q, nV)] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x < 6) aslot[threadIdx.x] = a ? a[threadIdx.x] : 0.0;
    __syncthreads();
    const double *s = s0;
    int offset = 0;
    for (int size = Np / 2; size >= 1; size /= 2) {
        for (int k = threadIdx.x; k < size; k += blockDim.x) {
            const double x0 = s[2 * k], x1 = s[2 * k + 1];
            out[offset + k] = __dadd_rn(__dadd_rn(0.0, __dmul_rn(HAAR, x0)), __dmul_rn(-HAAR, x1));
            out[offset + size + k] = __dadd_rn(__dadd_rn(0.0, __dmul_rn(HAAR, x0)), __dmul_rn(HAAR, x1));
        }
        __syncthreads();
        s = out + offset + size;
        offset += 2 * size;
    }
}

// partial[c] = sum over chunk c's nonzeros of v * x.  Each CTA first tabulates, per block
// b = 2 (k - 1) + t, the ring offset of its history vector (-1 beyond the `used` steps).  Each lane
// takes 4 nonzeros 32 apart per batch, with the next batch's columns and values in flight while the
// current batch gathers x; 2 accumulators, fixed order.
constexpr int SPMV_UNROLL = 4;
__global__ void __launch_bounds__(256) wav_spmv_kernel(const longlong2 *__restrict__ chunks, int nchunk,
                                                       const unsigned int *__restrict__ mcol,
                                                       const double *__restrict__ mval,
                                                       const double *__restrict__ xring, int L, int K, int used,
                                                       int head, int nblk, double *__restrict__ partial) {
    extern __shared__ long long xoff[];
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        const int k = b / 2 + 1;
        xoff[b] = k <= used ? ((long long)((head - k + 2 * K) % K) * 2 + (b & 1)) * L : -1LL;
    }
    __syncthreads();
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= nchunk) return;
    const longlong2 ch = chunks[c];
    double acc0 = 0.0, acc1 = 0.0;
    constexpr unsigned MASK = (1u << COL_BITS) - 1u;
    unsigned w[SPMV_UNROLL];
    double v[SPMV_UNROLL];
    long long e = ch.x + lane;
#pragma unroll
    for (int j = 0; j < SPMV_UNROLL; j++) {
        const long long i = e + 32 * j;
        w[j] = i < ch.y ? __ldg(mcol + i) : 0u;
        v[j] = i < ch.y ? __ldg(mval + i) : 0.0;
    }
    for (; e < ch.y; e += 32 * SPMV_UNROLL) {
        unsigned wn[SPMV_UNROLL];
        double vn[SPMV_UNROLL];
#pragma unroll
        for (int j = 0; j < SPMV_UNROLL; j++) {
            const long long i = e + 32 * (SPMV_UNROLL + j);
            wn[j] = i < ch.y ? __ldg(mcol + i) : 0u;
            vn[j] = i < ch.y ? __ldg(mval + i) : 0.0;
        }
        double x[SPMV_UNROLL];
#pragma unroll
        for (int j = 0; j < SPMV_UNROLL; j++) {
            const long long o = xoff[w[j] >> COL_BITS];
            x[j] = (o >= 0 && e + 32 * j < ch.y) ? xring[o + (w[j] & MASK)] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < SPMV_UNROLL; j += 2) {
            acc0 = fma(v[j], x[j], acc0);
            acc1 = fma(v[j + 1], x[j + 1], acc1);
        }
#pragma unroll
        for (int j = 0; j < SPMV_UNROLL; j++) {
            w[j] = wn[j];
            v[j] = vn[j];
        }
    }
    double acc = acc0 + acc1;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) partial[c] = acc;
}

__global__ void wav_rowsum_kernel(const double *__restrict__ partial, const int *__restrict__ chunk_ptr, int L,
                                  double *__restrict__ y) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= L) return;
    double s = 0.0;
    for (int c = chunk_ptr[r]; c < chunk_ptr[r + 1]; c++) s += partial[c];
    y[r] = s;
}

// reconstruction (include/wavelets.hpp:258-283), coarse to fine in shared memory (res: Np values,
// sb: Np / 2), then out[i] = res[P(i)]
__global__ void __launch_bounds__(1024) wav_reconstruct_kernel(const double *__restrict__ y, int nV, int Np,
                                                               double *__restrict__ out) {
    extern __shared__ double shm[];
    double *res = shm, *sb = shm + Np;
    int offset = -2;
    for (int size = 1; size <= Np / 2; size *= 2) {
        const int base = 2 * Np - 2 + offset;
        for (int n = threadIdx.x; n < size; n += blockDim.x) sb[n] = y[base + size + n] + (size > 1 ? res[n] : 0.0);
        __syncthreads();
        for (int n = threadIdx.x; n < size; n += blockDim.x) {
            const double s = sb[n], d = y[base + n];
            res[2 * n] = 0.0 + (HAAR * s + HAAR * d);
            res[2 * n + 1] = 0.0 + (HAAR * s + (-HAAR) * d);
        }
        __syncthreads();
        offset -= 4 * size;
    }
    const int N = 3 * nV;
    for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = res[i / 3 + (i % 3) * nV];
}

}  // namespace

namespace sod {

struct WaveletBank {
    int nV = 0, N = 0, Np = 0, L = 0, K = 0;
    long long keep = 0;
    double ratio = 0.0;
    struct Block {
        DevBuf ptr, col, val;
        std::vector<int> hptr;  // host copy of the row pointers
        long long nnz = 0;
        bool set = false;
    };
    std::vector<std::unique_ptr<Block>> blocks;
    std::vector<long long> cand_ptr;  // per row of D: first candidate (L + 1)
    DevBuf dcand, dcol0, coef, sA, sB, hist, gt, eq, eqb, xring;
    // merged CSR and the SpMV chunks
    DevBuf mptr, mcol, mval, chunks, chunk_ptr, partial, y, dblk;
    int nchunk = 0;
    long long nnz = 0;
    bool dirty = true;
};

void wavelet_bank_free(WaveletBank *w) { delete w; }

int wavelet_bank_create(sod_context *ctx, int nV, int K, double ratio, WaveletBank **out) {
    *out = nullptr;
    auto w = std::make_unique<WaveletBank>();
    w->nV = nV;
    w->N = 3 * nV;
    w->Np = 2;
    while (w->Np < w->N) w->Np *= 2;
    SOD_REQUIRE(w->Np <= (1 << (COL_BITS - 1)), "compressed history supports 3 nV <= 16384");
    SOD_REQUIRE(K <= 2048, "compressed history supports K <= 2048");  // ring offsets per block in shared memory
    w->L = 2 * w->Np - 2;
    w->K = K;
    w->ratio = ratio;
    w->keep = (long long)((double)w->N * (double)w->N * ratio);  // (int)(mat.size() * ratio)
    for (int b = 0; b < 2 * K; b++) w->blocks.push_back(std::make_unique<WaveletBank::Block>());
    // candidate layout of D (see the file header)
    std::vector<int> col0(w->L);
    w->cand_ptr.assign(w->L + 1, 0);
    long long base = 0;
    int offset = 0;
    for (int size = w->Np / 2; size >= 1; size /= 2) {
        for (int i = 0; i < size; i++) {
            w->cand_ptr[offset + i] = base + (long long)i * 2 * size;
            col0[offset + i] = offset;
            w->cand_ptr[offset + size + i] = base + 2LL * size * size + (long long)i * size;
            col0[offset + size + i] = offset;
        }
        base += 3LL * size * size;
        offset += 2 * size;
    }
    w->cand_ptr[w->L] = (long long)w->Np * w->Np;  // the last row also holds the final scale coefficient
    SOD_TRY(w->dcand.ensure(sizeof(long long) * (w->L + 1)));
    SOD_TRY(w->dcol0.ensure(sizeof(int) * w->L));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->dcand.p, w->cand_ptr.data(), sizeof(long long) * (w->L + 1),
                                   cudaMemcpyHostToDevice, ctx->stream));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->dcol0.p, col0.data(), sizeof(int) * w->L, cudaMemcpyHostToDevice, ctx->stream));
    SOD_TRY(w->xring.ensure(sizeof(double) * (size_t)K * 2 * w->L));
    SOD_CHECK_CUDA(cudaMemsetAsync(w->xring.p, 0, w->xring.bytes, ctx->stream));
    SOD_TRY(w->y.ensure(sizeof(double) * w->L));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // host tables above go out of scope
    *out = w.release();
    return SOD_OK;
}

// compress one matrix (device, N x N, FP64 or FP32) into block b
int wavelet_set_block(sod_context *ctx, WaveletBank *w, int b, const void *W, bool f64, double sign) {
    cudaStream_t st = ctx->stream;
    const int Np = w->Np, L = w->L;
    const long long nc = (long long)Np * Np;
    SOD_TRY(w->coef.ensure(sizeof(double) * nc));
    SOD_TRY(w->sA.ensure(sizeof(double) * (size_t)(Np / 2) * (Np / 2)));
    SOD_TRY(w->sB.ensure(sizeof(double) * (size_t)(Np / 2) * (Np / 2)));
    double *coef = w->coef.as<double>();
    // 1-2. decomposition, level by level
    long long base = 0;
    const double *s = nullptr;
    double *bufs[2] = {w->sA.as<double>(), w->sB.as<double>()};
    int which = 0;
    for (int size = Np / 2; size >= 1; size /= 2) {
        double *snew = size == 1 ? coef + nc - 1 : bufs[which];
        const dim3 grid((size + 255) / 256, size);
        haar_level_kernel<<<grid, 256, 0, st>>>(s ? nullptr : W, f64, w->nV, sign, s, size, coef + base, snew);
        SOD_CHECK_CUDA(cudaGetLastError());
        s = snew;
        which ^= 1;
        base += 3LL * size * size;
    }
    ctx->count(30);
    // 3. threshold: MSB radix select of the keep-th largest |v| over nonzero coefficients
    SOD_TRY(w->hist.ensure(sizeof(unsigned int) << RADIX_BITS));
    unsigned long long t = 0;
    long long need_eq = 0;
    std::vector<unsigned int> hh(1 << RADIX_BITS);
    const int grid_h = ctx->num_sms * 4;
    auto histogram = [&](int shift, int width, unsigned long long prefix) -> int {
        SOD_CHECK_CUDA(cudaMemsetAsync(w->hist.p, 0, sizeof(unsigned int) << width, st));
        radix_hist_kernel<<<grid_h, 512, 0, st>>>(coef, nc, shift, width, prefix, w->hist.as<unsigned int>());
        SOD_CHECK_CUDA(cudaGetLastError());
        SOD_CHECK_CUDA(cudaMemcpyAsync(hh.data(), w->hist.p, sizeof(unsigned int) << width, cudaMemcpyDeviceToHost, st));
        SOD_CHECK_CUDA(cudaStreamSynchronize(st));
        return SOD_OK;
    };
    if (w->keep > 0) {
        // digits of 12 bits from bit 63 down: shifts 52, 40, 28, 16, 4 and a last 4-bit digit
        const int shifts[6] = {52, 40, 28, 16, 4, 0}, widths[6] = {12, 12, 12, 12, 12, 4};
        SOD_TRY(histogram(shifts[0], widths[0], 0));
        long long nonzero = 0;
        for (unsigned v : hh) nonzero += v;
        if (nonzero > w->keep) {
            long long remaining = w->keep;
            unsigned long long prefix = 0;
            for (int pass = 0; pass < 6; pass++) {
                if (pass > 0) SOD_TRY(histogram(shifts[pass], widths[pass], prefix));
                const int nb = 1 << widths[pass];
                long long above = 0;
                int d = nb - 1;
                for (; d > 0; d--) {
                    if (above + (long long)hh[d] >= remaining) break;
                    above += hh[d];
                }
                remaining -= above;
                prefix = (prefix << widths[pass]) | (unsigned long long)d;
            }
            t = prefix;
            need_eq = remaining;
        }
    }
    ctx->count(6);
    // 4. per-row counts, row pointers (host), kept entries
    SOD_TRY(w->gt.ensure(sizeof(int) * L));
    SOD_TRY(w->eq.ensure(sizeof(int) * L));
    SOD_TRY(w->eqb.ensure(sizeof(long long) * L));
    const unsigned wb = (unsigned)(((size_t)L * 32 + 255) / 256);
    row_count_kernel<<<wb, 256, 0, st>>>(coef, w->dcand.as<long long>(), L, t, w->gt.as<int>(), w->eq.as<int>());
    SOD_CHECK_CUDA(cudaGetLastError());
    std::vector<int> hg(L), he(L);
    SOD_CHECK_CUDA(cudaMemcpyAsync(hg.data(), w->gt.p, sizeof(int) * L, cudaMemcpyDeviceToHost, st));
    SOD_CHECK_CUDA(cudaMemcpyAsync(he.data(), w->eq.p, sizeof(int) * L, cudaMemcpyDeviceToHost, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));
    WaveletBank::Block &B = *w->blocks[b];
    B.hptr.assign(L + 1, 0);
    std::vector<long long> eqb(L);
    long long eq_seen = 0;
    for (int r = 0; r < L; r++) {
        eqb[r] = eq_seen;
        const long long take_eq = std::max(0LL, std::min<long long>(he[r], need_eq - eq_seen));
        B.hptr[r + 1] = B.hptr[r] + hg[r] + (int)take_eq;
        eq_seen += he[r];
    }
    B.nnz = B.hptr[L];
    SOD_TRY(B.ptr.ensure(sizeof(int) * (L + 1)));
    SOD_TRY(B.col.ensure(sizeof(int) * std::max<long long>(B.nnz, 1)));
    SOD_TRY(B.val.ensure(sizeof(double) * std::max<long long>(B.nnz, 1)));
    SOD_CHECK_CUDA(cudaMemcpyAsync(B.ptr.p, B.hptr.data(), sizeof(int) * (L + 1), cudaMemcpyHostToDevice, st));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->eqb.p, eqb.data(), sizeof(long long) * L, cudaMemcpyHostToDevice, st));
    row_write_kernel<<<wb, 256, 0, st>>>(coef, w->dcand.as<long long>(), w->dcol0.as<int>(), L, t, need_eq,
                                         w->eqb.as<long long>(), B.ptr.as<int>(), B.col.as<int>(), B.val.as<double>());
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count(2);
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));  // host vectors above go out of scope
    B.set = true;
    w->dirty = true;
    return SOD_OK;
}

int wavelet_set_weights(sod_context *ctx, WaveletBank *w, int k, const void *G, const void *H, bool f64) {
    SOD_TRY(wavelet_set_block(ctx, w, 2 * (k - 1), G, f64, 1.0));
    SOD_TRY(wavelet_set_block(ctx, w, 2 * (k - 1) + 1, H, f64, -1.0));
    return SOD_OK;
}

static int wavelet_merge(sod_context *ctx, WaveletBank *w) {
    cudaStream_t st = ctx->stream;
    const int L = w->L, nb = (int)w->blocks.size();
    std::vector<long long> mp(L + 1, 0);
    for (int r = 0; r < L; r++) {
        long long c = 0;
        for (const auto &B : w->blocks)
            if (B->set) c += B->hptr[r + 1] - B->hptr[r];
        mp[r + 1] = mp[r] + c;
    }
    w->nnz = mp[L];
    std::vector<BlockPtrs> bp(nb);
    for (int b = 0; b < nb; b++) {
        const auto &B = *w->blocks[b];
        bp[b] = B.set ? BlockPtrs{B.ptr.as<int>(), B.col.as<int>(), B.val.as<double>()} : BlockPtrs{nullptr, nullptr, nullptr};
    }
    SOD_TRY(w->dblk.ensure(sizeof(BlockPtrs) * nb));
    SOD_TRY(w->mptr.ensure(sizeof(long long) * (L + 1)));
    SOD_TRY(w->mcol.ensure(sizeof(unsigned int) * std::max<long long>(w->nnz, 1)));
    SOD_TRY(w->mval.ensure(sizeof(double) * std::max<long long>(w->nnz, 1)));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->dblk.p, bp.data(), sizeof(BlockPtrs) * nb, cudaMemcpyHostToDevice, st));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->mptr.p, mp.data(), sizeof(long long) * (L + 1), cudaMemcpyHostToDevice, st));
    merge_kernel<<<(unsigned)(((size_t)L * 32 + 255) / 256), 256, 0, st>>>(
        w->dblk.as<BlockPtrs>(), nb, L, w->mptr.as<long long>(), w->mcol.as<unsigned int>(), w->mval.as<double>());
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    // chunks of at most CHUNK nonzeros, row by row
    std::vector<longlong2> ch;
    std::vector<int> cp(L + 1, 0);
    for (int r = 0; r < L; r++) {
        for (long long e = mp[r]; e < mp[r + 1]; e += CHUNK) ch.push_back(make_longlong2(e, std::min(e + CHUNK, mp[r + 1])));
        cp[r + 1] = (int)ch.size();
    }
    w->nchunk = (int)ch.size();
    SOD_TRY(w->chunks.ensure(sizeof(longlong2) * std::max<size_t>(ch.size(), 1)));
    SOD_TRY(w->chunk_ptr.ensure(sizeof(int) * (L + 1)));
    SOD_TRY(w->partial.ensure(sizeof(double) * std::max<size_t>(ch.size(), 1)));
    if (!ch.empty())
        SOD_CHECK_CUDA(cudaMemcpyAsync(w->chunks.p, ch.data(), sizeof(longlong2) * ch.size(), cudaMemcpyHostToDevice, st));
    SOD_CHECK_CUDA(cudaMemcpyAsync(w->chunk_ptr.p, cp.data(), sizeof(int) * (L + 1), cudaMemcpyHostToDevice, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));  // host tables above go out of scope
    w->dirty = false;
    return SOD_OK;
}

int wavelet_push(sod_context *ctx, WaveletBank *w, const double *p, const double *u, const double *a, int slot,
                 double *aslot) {
    const size_t smem = sizeof(double) * w->Np;
    if (smem > 48 * 1024)
        SOD_CHECK_CUDA(cudaFuncSetAttribute(wav_push_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    wav_push_kernel<<<2, 1024, smem, ctx->stream>>>(p, u, a, w->nV, w->Np,
                                                    w->xring.as<double>() + (size_t)slot * 2 * w->L, aslot);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

// out[i] (N values) = P^T reconstruct(sum over the used steps of D x); head = ring slot of the next push
int wavelet_convolve(sod_context *ctx, WaveletBank *w, int used, int head, double *out) {
    if (w->dirty) SOD_TRY(wavelet_merge(ctx, w));
    cudaStream_t st = ctx->stream;
    if (w->nchunk > 0) {
        const int nblk = 2 * w->K;
        wav_spmv_kernel<<<(unsigned)(((size_t)w->nchunk * 32 + 255) / 256), 256, sizeof(long long) * nblk, st>>>(
            w->chunks.as<longlong2>(), w->nchunk, w->mcol.as<unsigned int>(), w->mval.as<double>(),
            w->xring.as<double>(), w->L, w->K, used, head, nblk, w->partial.as<double>());
        SOD_CHECK_CUDA(cudaGetLastError());
    }
    wav_rowsum_kernel<<<(w->L + 255) / 256, 256, 0, st>>>(w->partial.as<double>(), w->chunk_ptr.as<int>(), w->L,
                                                         w->y.as<double>());
    const size_t rsmem = sizeof(double) * (size_t)w->Np * 3 / 2;
    if (rsmem > 48 * 1024)
        SOD_CHECK_CUDA(cudaFuncSetAttribute(wav_reconstruct_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)rsmem));
    wav_reconstruct_kernel<<<1, 1024, rsmem, st>>>(w->y.as<double>(), w->nV, w->Np, out);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count(3);
    return SOD_OK;
}

int64_t wavelet_bytes(const WaveletBank *w) {
    long long nnz = 0;
    for (const auto &B : w->blocks)
        if (B->set) nnz += B->nnz;
    return (int64_t)nnz * (int64_t)(sizeof(double) + sizeof(unsigned int));
}

int wavelet_block(const WaveletBank *w, int b, int64_t *nnz, int *row_ptr, int *col, double *val, cudaStream_t st) {
    const auto &B = *w->blocks[b];
    SOD_REQUIRE(B.set, "weights of this step were not set");
    *nnz = B.nnz;
    if (row_ptr) std::copy(B.hptr.begin(), B.hptr.end(), row_ptr);
    if (col) SOD_CHECK_CUDA(cudaMemcpyAsync(col, B.col.p, sizeof(int) * B.nnz, cudaMemcpyDefault, st));
    if (val) SOD_CHECK_CUDA(cudaMemcpyAsync(val, B.val.p, sizeof(double) * B.nnz, cudaMemcpyDefault, st));
    SOD_CHECK_CUDA(cudaStreamSynchronize(st));
    return SOD_OK;
}

int wavelet_dims(const WaveletBank *w, int *N, int *L) {
    *N = w->N;
    *L = w->L;
    return SOD_OK;
}

}  // namespace sod
