// sod_history_tc.cu -- tensor-core (tcgen05) history convolution on sm_103a.
//
// b[row][r] = sum_seg scale[seg][row] * sum_c W[seg][row][c] * x_seg[c][r]   (seg = (history i, G|-H))
// is a tall-skinny GEMM per segment: M = nrow, N = R, K = ncol.  With BF16 weights and 16
// right-hand sides it must move 2 bytes per weight at HBM speed while doing 32 flop per weight --
// beyond the FP32 pipes; with one right-hand side the tensor cores still unpack the BF16 weights for
// free, which the CUDA-core loop pays for in issue slots.  So:
//   * TMA (cp.async.bulk.tensor, 128-byte swizzle) stages 128 x 64 weight tiles -- a 3D tensor map
//     with the segment as z, so the rows past the end of a matrix in its last row tile are
//     zero-filled instead of read -- and the matching history tile in a 4-stage shared-memory ring
//     (mbarrier full / empty pairs);
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M 128, K 16; BF16 x BF16 -> FP32 in
//     tensor memory).  The history enters as two BF16 terms (hi + lo), so only the weights are
//     rounded to BF16: R = 16 stacks the 16 hi and 16 lo columns into one N = 32 operand and the
//     epilogue adds accumulator columns j and 16 + j; R = 1 puts hi and lo in rows 0 and 1 of an
//     N = 16 operand (rows 2-15 zero) and adds columns 0 and 1.  Two accumulators in TMEM alternate
//     between units;
//   * four epilogue warps read the accumulator with tcgen05.ld (32 lanes each), apply the
//     segment's row scale and add it to the CTA's running FP32 sum for its row tile.
// The grid is a multiple of the row-tile count, G = k * mt (k = floor(2 SMs / mt), at most the
// segment count): CTA b keeps row tile m = b % mt and takes segments c, c + k, c + 2k, ...
// (c = b / mt), so it stores one partial tile at the end, and at any time the whole grid works on
// k neighbouring segments, whose history tiles stay in L2 while the weights stream past.  A second
// kernel adds a row tile's k partials in FP64 in fixed order (deterministic).  Banks with more row
// tiles than 2 CTAs per SM (nrow > 2 SMs x 128) run with k = 1 in several waves.
// FP32 banks (16 right-hand sides) run the same pipeline with 3xTF32 arithmetic and FP32 accuracy:
// 128 x 32 FP32 weight tiles arrive by TMA.  The TF32 MMA reads the top 19 bits of each FP32
// operand (w_hi), so the tile serves as w_hi as it lies; four transform warps form w_lo = w - w_hi,
// one weight row per thread, and store it to tensor memory with tcgen05.st.  The history comes as
// x_hi + x_lo (x_hi TF32-exact); tcgen05.mma.kind::tf32 accumulates w_hi [x_hi | x_lo] (N = 32,
// A from shared memory) and w_lo x_hi (N = 16, A from tensor memory, same accumulator columns),
// dropping only w_lo x_lo (~2^-22 relative).  Shared memory then carries each weight byte three
// times (TMA write, the transform's read, the MMA's read), which keeps it below the HBM rate.
// Every mbarrier wait is bounded (about one second of clock); a timeout sets an error flag that the
// host reports, and the kernel lets its copies and MMAs in flight finish (again bounded) and
// releases its tensor memory before returning.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <mutex>

#include "sod_internal.h"

namespace sod {
namespace {

constexpr int TC_MAX_STAGES = 4;
constexpr int TC_BM = 128;
constexpr int TC_A_BYTES = TC_BM * 128;  // 128 weight rows of 128 bytes: 16 KB
// elements per 128-byte row (the K extent of a stage): 64 BF16 or 32 FP32
template <bool F32> constexpr int tc_bk() { return F32 ? 32 : 64; }
// MMA N (history rows of the B operand: 16 hi + 16 lo, or hi, lo and 14 zero rows)
template <int R> constexpr int tc_n() { return R == 16 ? 32 : 16; }
// stage: weight tile and history tile, 20 / 18 KB (FP32 banks keep the weights' lo parts in tensor memory)
template <int R, bool F32> constexpr int tc_stage_bytes() { return TC_A_BYTES + tc_n<R>() * 128; }
template <bool F32> constexpr int tc_stages() { return 4; }  // 2 CTAs per SM
// producer, MMA, 4 epilogue warps (+ 4 warps that split FP32 weight tiles)
template <bool F32> constexpr int tc_threads() { return F32 ? 320 : 192; }
template <int R, bool F32> constexpr int tc_smem() { return tc_stages<F32>() * tc_stage_bytes<R, F32>() + 1024; }
// Units and accumulators.  A BF16 unit is one segment (its row scale applies to the whole sum).  The
// tensor core's FP32 accumulation does not round to nearest at every step, and its error grows with
// the number of MMAs that feed one accumulator: over a whole 7686-column segment (961 TF32 MMAs
// spread over 4 accumulators) it reached 1e-5 relative.  So an FP32 unit is a run of TC_SUB K tiles
// of a segment, spread round-robin over 2 accumulators (16 MMAs each), and the epilogue adds every
// unit into its FP32 registers, rounding to nearest; two accumulator sets alternate so that the MMAs
// of the next unit overlap the epilogue's reads.  Behind the accumulators, 4 x 32 columns hold the
// stages' w_lo tiles.
constexpr int TC_SUB = 8;
template <bool F32> constexpr int tc_ngroups() { return F32 ? 2 : 1; }
template <bool F32> constexpr int tc_nbuf() { return 2; }
template <bool F32> constexpr int tc_acc_cols() { return tc_nbuf<F32>() * tc_ngroups<F32>() * 32; }
template <bool F32> constexpr int tc_tmem_cols() { return tc_acc_cols<F32>() + (F32 ? tc_stages<F32>() * 32 : 0); }  // 256 / 64
static_assert(tc_tmem_cols<true>() == 256 && tc_tmem_cols<false>() == 64, "tensor memory columns (power of two)");
constexpr long long TC_WAIT_CYCLES = 2000000000LL;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false on timeout or when another role has already aborted
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err, int code) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > TC_WAIT_CYCLES) {
            *abort_flag = 1;
            atomicExch(err, code);
            return false;
        }
    }
    return true;
}
// bounded wait that ignores the abort flag (draining in-flight copies and MMAs before exit)
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    return true;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}
// tcgen05 shared-memory matrix descriptor: K-major operand in the 128-byte swizzled layout
// (rows of 128 B, 8-row atoms of 1024 B): start >> 4, LBO (unused here) 1, SBO 1024 >> 4,
// descriptor version 1 (bit 46), swizzle mode 2 (128 B, bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// instruction descriptor: D F32 (bits 4-5 = 1), A and B format at bits 7-9 / 10-12 (kind::f16: BF16 = 1;
// kind::tf32: TF32 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
template <int N, bool F32> constexpr uint32_t tc_idesc() {
    return (1u << 4) | ((F32 ? 2u : 1u) << 7) | ((F32 ? 2u : 1u) << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(TC_BM >> 4) << 24);
}

// one MMA, M 128 x N x K 16 (BF16) or K 8 (TF32: FP32 operands of which the tensor core uses the top
// 19 bits), FP32 accumulate in tensor memory
template <int N, bool F32>
__device__ __forceinline__ void mma_tc(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    if constexpr (F32)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                d_tmem),
            "l"(a), "l"(b), "r"(tc_idesc<N, true>()), "r"(accumulate));
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                d_tmem),
            "l"(a), "l"(b), "r"(tc_idesc<N, false>()), "r"(accumulate));
}
// W_lo x_hi for FP32 banks: M 128 x N 16 x K 8 TF32 MMA with A in tensor memory (row i in lane i, one
// 32-bit element per column), accumulating into d
__device__ __forceinline__ void mma_tc_ts16(uint32_t d_tmem, uint32_t a_tmem, uint64_t b) {
    asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, 1;" ::"r"(d_tmem), "r"(a_tmem), "l"(b),
                 "r"(tc_idesc<16, true>()));
}
// 32 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]),
        "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]),
        "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

struct TcArgs {
    int nrow, ncol, used, head, K, mt, nseg, k;
    const float *scale;  // [2K][nrow] (matrix = 2 i + t); null for FP32 banks
    float *partial;      // [G = k mt][128][R]
    int *err;
};

template <int R, bool F32>
__global__ void __launch_bounds__(tc_threads<F32>(), 2) hist_tc_kernel(const __grid_constant__ CUtensorMap wmap,
                                                                       const __grid_constant__ CUtensorMap xmap,
                                                                       TcArgs a) {
    constexpr int STAGES = tc_stages<F32>(), BK = tc_bk<F32>(), SB = tc_stage_bytes<R, F32>();
    constexpr int B_OFF = TC_A_BYTES;  // history tile offset in a stage
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[TC_MAX_STAGES], empty[TC_MAX_STAGES], ready[TC_MAX_STAGES], acc_full[2],
        acc_empty[2], drain;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // 1024-byte aligned stage ring (the 128-byte swizzle atoms)
    const uint32_t ring = (smem_u32(smem_raw) + 1023u) & ~1023u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
            mbar_init(smem_u32(&ready[s]), 128);  // FP32: the 128 transform threads
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&acc_full[b]), 1);
            mbar_init(smem_u32(&acc_empty[b]), 4);
        }
        mbar_init(smem_u32(&drain), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(tc_tmem_cols<F32>()));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int KT = (a.ncol + BK - 1) / BK;
    volatile int *ab = &abort_flag;
    const int m = blockIdx.x % a.mt, seg0 = blockIdx.x / a.mt;  // this CTA's row tile and first segment

    if (warp == 0) {
        // ---- producer: TMA loads of weight and history tiles ----
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            int issued[TC_MAX_STAGES];  // phase parity of the last load into each stage, -1 = none
            for (int s = 0; s < STAGES; s++) issued[s] = -1;
            for (int seg = seg0; seg < a.nseg && ok; seg += a.k) {
                const int i = seg >> 1, t = seg & 1;
                const int slot = (a.head - 1 - i + 2 * a.K) % a.K;
                for (int kt = 0; kt < KT && ok; kt++) {
                    ok = mbar_wait(smem_u32(&empty[stage]), phase ^ 1u, ab, a.err, 1);
                    if (!ok) break;
                    const uint32_t fb = smem_u32(&full[stage]);
                    mbar_expect_tx(fb, TC_A_BYTES + tc_n<R>() * 128);
                    const uint32_t sA = ring + stage * SB;
                    tma_load_3d(sA, &wmap, kt * BK, m * TC_BM, seg, fb);
                    tma_load_2d(sA + B_OFF, &xmap, kt * BK, (slot * 2 + t) * tc_n<R>(), fb);
                    issued[stage] = (int)phase;
                    if (++stage == STAGES) stage = 0, phase ^= 1u;
                }
            }
            if (!ok)  // aborted: let the copies in flight land before shared memory is released
                for (int s = 0; s < STAGES; s++)
                    if (issued[s] >= 0) mbar_drain(smem_u32(&full[s]), (uint32_t)issued[s]);
        }
    } else if (warp == 1) {
        // ---- MMA issue (one thread) ----
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            int ul = 0;
            const int SUBT = F32 ? TC_SUB : KT;  // K tiles per unit
            for (int seg = seg0; seg < a.nseg && ok; seg += a.k)
            for (int u0 = 0; u0 < KT && ok; u0 += SUBT, ul++) {
                const int u1 = min(KT, u0 + SUBT);
                const int buf = ul % tc_nbuf<F32>();
                const uint32_t aphase = (ul / tc_nbuf<F32>()) & 1;
                ok = mbar_wait(smem_u32(&acc_empty[buf]), aphase ^ 1u, ab, a.err, 2);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                constexpr int NG = tc_ngroups<F32>();
                for (int kt = u0; kt < u1 && ok; kt++) {
                    // BF16: the TMA tiles; FP32: the tiles after the transform warps split the weights
                    ok = mbar_wait(smem_u32(F32 ? &ready[stage] : &full[stage]), phase, ab, a.err, 3);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t sA = ring + stage * SB;
                    // 4 K steps of 32 bytes: K 16 (BF16) or K 8 (TF32) each
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        // accumulator of this K tile; the first MMA into it overwrites
                        const uint32_t d = tmem + (buf * NG + (kt - u0) % NG) * 32;
                        mma_tc<tc_n<R>(), F32>(d, smem_desc(sA + k * 32), smem_desc(sA + B_OFF + k * 32),
                                               (kt - u0 >= NG) || (k > 0));
                        // FP32: W_lo (tensor memory, 8 columns per K step) x (x_hi rows; for R = 1 the
                        // whole hi/lo tile)
                        if (F32)
                            mma_tc_ts16(d, tmem + tc_acc_cols<F32>() + stage * 32 + k * 8, smem_desc(sA + B_OFF + k * 32));
                    }
                    mma_commit(smem_u32(&empty[stage]));  // frees the stage when these MMAs finish
                    if (++stage == STAGES) stage = 0, phase ^= 1u;
                }
                if (ok) mma_commit(smem_u32(&acc_full[buf]));
            }
            // every MMA this thread issued has finished before tensor memory is released
            mma_commit(smem_u32(&drain));
            if (!mbar_drain(smem_u32(&drain), 0)) atomicExch(a.err, 5);
        }
    } else if (F32 && warp >= 6) {
        // ---- FP32 weights: w_lo = w - w_hi (w_hi = the top 19 bits, the part of w the TF32 MMA reads)
        // of one weight row per thread, into the stage's tensor-memory tile.  Row r of the 128-byte
        // swizzled TMA tile holds its 16-byte chunk j at chunk position j ^ (r & 7).
        const int q = warp & 3;  // TMEM lane quadrant this warp may access
        const int r = q * 32 + lane;
        const uint32_t lo_cols = tmem + ((uint32_t)(q * 32) << 16) + tc_acc_cols<F32>();
        int stage = 0;
        uint32_t phase = 0;
        bool ok = true;
        for (int seg = seg0; seg < a.nseg && ok; seg += a.k)
            for (int kt = 0; kt < KT && ok; kt++) {
                ok = mbar_wait(smem_u32(&full[stage]), phase, ab, a.err, 6);
                if (!ok) break;
                const float4 *w =
                    reinterpret_cast<const float4 *>(smem_raw + (ring - smem_u32(smem_raw)) + stage * SB + r * 128);
                uint32_t l[32];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const float4 v = w[j ^ (r & 7)];
                    l[4 * j + 0] = __float_as_uint(v.x - __uint_as_float(__float_as_uint(v.x) & 0xffffe000u));
                    l[4 * j + 1] = __float_as_uint(v.y - __uint_as_float(__float_as_uint(v.y) & 0xffffe000u));
                    l[4 * j + 2] = __float_as_uint(v.z - __uint_as_float(__float_as_uint(v.z) & 0xffffe000u));
                    l[4 * j + 3] = __float_as_uint(v.w - __uint_as_float(__float_as_uint(v.w) & 0xffffe000u));
                }
                tmem_st32(lo_cols + stage * 32, l);
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                // order the shared-memory reads before the stage is refilled, and the tensor-memory
                // writes before the MMA thread's reads, then signal
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;");
                mbar_arrive(smem_u32(&ready[stage]));
                if (++stage == STAGES) stage = 0, phase ^= 1u;
            }
    } else {
        // ---- epilogue: TMEM -> registers -> scaled sum over the CTA's segments ----
        const int q = warp & 3;  // TMEM lane quadrant this warp may access
        const int row = m * TC_BM + q * 32 + lane;
        // running sum over the CTA's units; FP32 banks add a thousand units or so per row, so the sum is
        // compensated (TwoSum into a correction term) to stay at FP32 accuracy
        float acc[R], cmp[R];
#pragma unroll
        for (int j = 0; j < R; j++) acc[j] = 0.f, cmp[j] = 0.f;
        int ul = 0;
        const int SUBT = F32 ? TC_SUB : KT;  // K tiles per unit
        bool ok = true;
        for (int seg = seg0; seg < a.nseg && ok; seg += a.k)
        for (int u0 = 0; u0 < KT; u0 += SUBT, ul++) {
            const int buf = ul % tc_nbuf<F32>();
            const uint32_t aphase = (ul / tc_nbuf<F32>()) & 1;
            if (!mbar_wait(smem_u32(&acc_full[buf]), aphase, ab, a.err, 4)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            constexpr int NG = tc_ngroups<F32>();
            const int ng = min(NG, min(KT, u0 + SUBT) - u0);  // accumulators this unit wrote
            float vs[32];
#pragma unroll
            for (int j = 0; j < 32; j++) vs[j] = 0.f;
            for (int gi = 0; gi < ng; gi++) {  // fixed order
                uint32_t v[32];
                const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (buf * NG + gi) * 32;
                tmem_ld16(taddr, v);
                if (R == 16) tmem_ld16(taddr + 16, v + 16);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < (R == 16 ? 32 : 16); j++) vs[j] += __uint_as_float(v[j]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acc_empty[buf]));
            // BF16: the row's power-of-two scale; FP32: unscaled
            const float sc = row < a.nrow ? (a.scale ? a.scale[(size_t)seg * a.nrow + row] : 1.f) : 0.f;
#pragma unroll
            for (int j = 0; j < R; j++) {
                const float v = R == 1 ? vs[0] + vs[1] : vs[j] + vs[16 + j];
                if (F32) {  // unscaled: TwoSum of acc and v
                    const float t = acc[j] + v, bp = t - acc[j];
                    cmp[j] += (acc[j] - (t - bp)) + (v - bp);
                    acc[j] = t;
                } else {
                    acc[j] = fmaf(v, sc, acc[j]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < R; j++) acc[j] += cmp[j];
        float *dst = a.partial + ((size_t)blockIdx.x * TC_BM + q * 32 + lane) * R;
        if (R == 1) {
            dst[0] = acc[0];
        } else {
#pragma unroll
            for (int j = 0; j < R; j += 4)
                *reinterpret_cast<float4 *>(dst + j) = make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc_tmem_cols<F32>()));
    }
}

// b[row][r] = sum of the row tile's k partials (FP64, fixed order) + sum_i B_{i+1} a_slot
// (thread 0 also mirrors the device error word into pinned host memory for the host to poll)
__global__ void hist_tc_finish_kernel(const float *__restrict__ partial, int k, int mt, const double *__restrict__ Bw,
                                      const double *__restrict__ A, int used, int head, int K, int nrow, int R,
                                      double *__restrict__ out, const int *__restrict__ err, int *err_mirror) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0 && err_mirror) *(volatile int *)err_mirror = *(volatile const int *)err;
    if (e >= nrow * R) return;
    const int row = e / R, j = e % R;
    const int m = row / TC_BM;
    double s = 0.0;
    for (int c = 0; c < k; c++) s += partial[((size_t)(c * mt + m) * TC_BM + row % TC_BM) * R + j];
    if (Bw) {
        for (int i = 0; i < used; i++) {
            const int slot = (head - 1 - i + 2 * K) % K;
            const double *b = Bw + ((size_t)i * nrow + row) * 6;
            const double *x = A + (size_t)slot * 6 * R;
            for (int c = 0; c < 6; c++) s += b[c] * x[c * R + j];
        }
    }
    out[e] = s;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// BF16 or FP32 tensor map of `rank` dimensions (dims innermost first, byte strides of dims 1.., box
// extents), 128-byte swizzle, zero fill out of bounds
int make_map(CUtensorMap *map, bool f32, const void *base, int rank, const uint64_t *dims, const uint64_t *strides,
             const uint32_t *box) {
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return SOD_ERR_CUDA;
    }
    cuuint64_t d[3], st[2];
    cuuint32_t bx[3], estr[3] = {1, 1, 1};
    for (int r = 0; r < rank; r++) d[r] = dims[r], bx[r] = box[r];
    for (int r = 0; r + 1 < rank; r++) st[r] = strides[r];
    const CUresult res = fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                            (cuuint32_t)rank, const_cast<void *>(base), d, st, bx,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (res != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)res) + ")");
        return SOD_ERR_CUDA;
    }
    return SOD_OK;
}

}  // namespace

namespace {
// segment groups per row tile: fill the 2-CTAs-per-SM grid with whole multiples of the row tiles
int tc_groups(int num_sms, int mt, int nseg) { return std::max(1, std::min(2 * num_sms / mt, nseg)); }
}  // namespace

// FP32 scratch the convolution needs: partial tiles [G][128][R], G = k * mt <= max(2 SMs, mt)
size_t history_tc_partial_floats(int num_sms, int nrow, int R) {
    const int mt = (nrow + TC_BM - 1) / TC_BM;
    return (size_t)std::max(2 * num_sms, mt) * TC_BM * R;
}

// Tensor maps of a bank.  W: [K][2][nrow][ldw] BF16 or FP32, mapped as {ncol, nrow, 2K} with boxes
// of 128 rows x 128 bytes; Xt: the history split into hi + lo (BF16, or FP32 with a TF32-exact hi),
// [K][2][hi|lo][16][ldw] for R = 16 and [K][2][16][ldw] (rows hi, lo, then zeros) for R = 1, mapped
// as {ncol, 2K * N} with N x 128-byte boxes.
int history_tc_plan(HistTcPlan *plan, const void *W, const void *Xt, int nrow, int ncol, int ldw, int K, int R,
                    bool f32) {
    SOD_REQUIRE(ldw % 8 == 0, "tensor-core history: row pitch must be a multiple of 16 bytes");
    SOD_REQUIRE(R == 1 || R == 16, "tensor-core history: 1 or 16 right-hand sides");
    static_assert(sizeof(CUtensorMap) == sizeof(plan->wmap), "CUtensorMap size");
    const int n = R == 16 ? tc_n<16>() : tc_n<1>();
    const uint64_t esz = f32 ? 4 : 2;
    const uint32_t bk = f32 ? tc_bk<true>() : tc_bk<false>();
    const uint64_t wdims[3] = {(uint64_t)ncol, (uint64_t)nrow, (uint64_t)K * 2};
    const uint64_t wstr[2] = {(uint64_t)ldw * esz, (uint64_t)nrow * ldw * esz};
    const uint32_t wbox[3] = {bk, TC_BM, 1};
    SOD_TRY(make_map(reinterpret_cast<CUtensorMap *>(plan->wmap), f32, W, 3, wdims, wstr, wbox));
    const uint64_t xdims[2] = {(uint64_t)ncol, (uint64_t)K * 2 * n};
    const uint64_t xstr[1] = {(uint64_t)ldw * esz};
    const uint32_t xbox[2] = {bk, (uint32_t)n};
    SOD_TRY(make_map(reinterpret_cast<CUtensorMap *>(plan->xmap), f32, Xt, 2, xdims, xstr, xbox));
    plan->nrow = nrow, plan->ncol = ncol, plan->ldw = ldw, plan->K = K, plan->R = R, plan->f32 = f32;
    plan->W = W, plan->Xt = Xt;
    static std::once_flag attr_once;
    static int attr_rc = SOD_OK;
    std::call_once(attr_once, [] {
        const auto A = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (cudaFuncSetAttribute(hist_tc_kernel<16, false>, A, tc_smem<16, false>()) != cudaSuccess ||
            cudaFuncSetAttribute(hist_tc_kernel<1, false>, A, tc_smem<1, false>()) != cudaSuccess ||
            cudaFuncSetAttribute(hist_tc_kernel<16, true>, A, tc_smem<16, true>()) != cudaSuccess ||
            cudaFuncSetAttribute(hist_tc_kernel<1, true>, A, tc_smem<1, true>()) != cudaSuccess)
            attr_rc = SOD_ERR_CUDA;
    });
    if (attr_rc != SOD_OK) {
        set_error("cudaFuncSetAttribute failed for the tensor-core history kernel");
        return attr_rc;
    }
    plan->ready = true;
    return SOD_OK;
}

// Convolution of the `used` most recent steps; partial: FP32 scratch of history_tc_partial_floats().
int launch_history_tc(sod_context *ctx, const HistTcPlan *plan, const float *scale, int used, int head,
                      float *partial, const double *Bw, const double *A, double *out, int *err, int *err_mirror,
                      cudaStream_t stream) {
    SOD_REQUIRE(plan && plan->ready, "tensor-core history: plan not built");
    const int nrow = plan->nrow, K = plan->K, R = plan->R;
    const CUtensorMap &wmap = *reinterpret_cast<const CUtensorMap *>(plan->wmap);
    const CUtensorMap &xmap = *reinterpret_cast<const CUtensorMap *>(plan->xmap);
    TcArgs a;
    a.nrow = nrow, a.ncol = plan->ncol, a.used = used, a.head = head, a.K = K;
    a.mt = (nrow + TC_BM - 1) / TC_BM;
    a.nseg = 2 * used;
    a.k = used > 0 ? tc_groups(ctx->num_sms, a.mt, a.nseg) : 0;
    a.scale = scale;
    a.partial = partial;
    a.err = err;
    const bool f = plan->f32;
    const size_t smem = f ? (R == 16 ? tc_smem<16, true>() : tc_smem<1, true>())
                          : (R == 16 ? tc_smem<16, false>() : tc_smem<1, false>());
    auto kern = f ? (R == 16 ? hist_tc_kernel<16, true> : hist_tc_kernel<1, true>)
                  : (R == 16 ? hist_tc_kernel<16, false> : hist_tc_kernel<1, false>);
    const int threads = f ? tc_threads<true>() : tc_threads<false>();
    const int grid = a.k * a.mt;
    if (grid > 0) {
        kern<<<grid, threads, smem, stream>>>(wmap, xmap, a);
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    const int n = nrow * R;
    hist_tc_finish_kernel<<<(n + 255) / 256, 256, 0, stream>>>(partial, a.k, a.mt, Bw, A, used, head, K, nrow, R, out,
                                                               err, err_mirror);
    SOD_CHECK_CUDA(cudaGetLastError());
    ctx->count();
    return SOD_OK;
}

}  // namespace sod
