// sod_coll_compensated.cu -- compensated (double-float) regular collocation pass.
//
// Why it exists.  The time-domain CQ weights are X_n = R^-n / L sum_l c_l Re(Xhat_l zeta^-nl) with
// R^-N = 1e5 (R = (1e-10)^(1/(2N)), src/elastodynamics_cqbem_G.cu:19,166-179 of the reference).
// Rounding errors of the Laplace-domain entries that vary irregularly from one frequency to the
// next are amplified by up to R^-N in the late weights.  FP32 evaluation of the frequency-dependent
// terms (the two complex exponentials, psi, the kernel coefficients) and FP32 sums leave about 1e-7
// relative noise per entry, which becomes 5e-4 (G) to 7e-3 (B_angular) of the stacked time-domain
// weights -- the reference's own mixed-precision precomputation has the same defect for G and B.
// Rounding of the geometry (r, r-hat, weights) does not vary with the frequency: it is the exact
// answer for a perturbed mesh, and its effect on the time-domain weights stays at ~3e-8.
//
// So this pass keeps the FP32 geometry of the fast pass and evaluates everything that depends on the
// frequency in double-float arithmetic on the FP32 pipes (TwoSum / TwoProd without renormalisation,
// Tang's table-driven exp, sin/cos by reduction with pi/32 and angle addition, with the tables in
// shared memory), with compensated sums at every level: the quadrature points of a face, the
// faces of the row block, and the per-thread B columns.  Measured on a 162-vertex sphere, N = 16:
// per-evaluation relative noise eps in the kernel coefficients costs ~2000 eps of stacked
// time-domain error, and noise eps in the per-face sums ~5500 eps, so the ~1e-14 of double-float
// leaves the FP32 geometry as the only visible error.
//
// Structure (same schedule as the fast pass, one CTA per (field vertex, frequency)):
//   * G or H: colour-ordered scatter into a double-float row block [NC][nV] (float4 = re.hi, re.lo,
//     im.hi, im.lo) in shared memory, or in a global-memory slice per CTA when it does not fit
//     (persistent grid); per-face partial sums in double-float registers;
//   * B_trans / B_angular: per-face moments in registers, the face tensors added into the thread's
//     own double-float column of a shared [NC][T] block, columns summed in fixed order.
// The singular-face side buffers (FP64) of the double-float singular pass are added in the epilogue,
// exactly as in the fast pass.
#include <algorithm>

#include "sod_coll_common.cuh"
#include "sod_dd.cuh"
#include "sod_dd_fast.cuh"

namespace sod {

// per-frequency constants in double-float
struct KDD {
    cdd sc1, sc2, is, is2;  // s/c1, s/c2, 1/s, 1/s^2
    dd c2sq;                // c2^2
    dd ic1, ic2, ic1s, ic2s, six_c2s, inv4pirho, inv4pi;
    dd k4m1, k1m2, k2, k12;  // 4 kappa - 1, 1 - 2 kappa, 2 kappa, 12 kappa
};
__host__ __device__ inline dd kdd_split(double x) {
    const float h = (float)x;
    return dd{h, (float)(x - (double)h)};
}
__host__ __device__ inline KDD kdd_from(const KConst<double> &k) {
    KDD d;
    d.sc1 = cdd{kdd_split(k.sc1r), kdd_split(k.sc1i)};
    d.sc2 = cdd{kdd_split(k.sc2r), kdd_split(k.sc2i)};
    d.is = cdd{kdd_split(k.isr), kdd_split(k.isi)};
    d.is2 = cdd{kdd_split(k.is2r), kdd_split(k.is2i)};
    d.c2sq = kdd_split(k.c2sq);
    d.ic1 = kdd_split(k.ic1), d.ic2 = kdd_split(k.ic2), d.ic1s = kdd_split(k.ic1s), d.ic2s = kdd_split(k.ic2s);
    d.six_c2s = kdd_split(k.six_c2s), d.inv4pirho = kdd_split(k.inv4pirho), d.inv4pi = kdd_split(k.inv4pi);
    d.k4m1 = kdd_split(4.0 * k.kappa - 1.0), d.k1m2 = kdd_split(1.0 - 2.0 * k.kappa);
    d.k2 = kdd_split(2.0 * k.kappa), d.k12 = kdd_split(12.0 * k.kappa);
    return d;
}
// The kernels take the constants as float pairs built on the host: members read straight from the
// parameter space (one constant-cache load when the compiler re-reads one) instead of a per-thread
// conversion from double, which the compiler re-materialises inside the loops under register pressure
// (two conversions and an FP64 add on the slow FP64 pipe for every re-read).
struct KddTable {
    int n;
    KDD k[MAX_FREQ_PER_LAUNCH];
};

struct RadDD {
    cdd z1, z2, e1, e2, psi2, Y;
};
// the frequency-dependent radial terms at distance r (an exact float; rinv ~ 1/r in float).  Since
// c1^2 z1^2 = c2^2 z2^2 = s^2 r^2,  Y = psi(z1)/c1^2 - psi(z2)/c2^2 = ((1 + z1) e1 - (1 + z2) e2) / (s^2 r^2)
// with the -1 of both psi cancelled exactly: above |z1| = 0.1 no reciprocal of a complex number is
// taken, 1 / r^2 comes from one Newton correction of rinv (consistent with r to ~1e-14, so that Y's
// terms stay consistent with each other).  Below |z| = 0.1 the series of psi (sod_dd.cuh).  psi2
// (B_trans) only when PSI2.
template <bool PSI2>
__device__ __forceinline__ RadDD radial_dd(float r, float rinv, const KDD &k, const DdTabs *tb) {
    RadDD t;
    t.z1 = cs_scalef(k.sc1, r);
    t.z2 = cs_scalef(k.sc2, r);
    t.e1 = cs_exp_neg(t.z1, tb);
    t.e2 = cs_exp_neg(t.z2, tb);
    const float az1 = t.z1.x.hi * t.z1.x.hi + t.z1.y.hi * t.z1.y.hi;
    const float az2 = t.z2.x.hi * t.z2.x.hi + t.z2.y.hi * t.z2.y.hi;
    if (az2 < 0.01f) {  // both series
        const cdd psi1 = cdd_psi(t.z1, t.e1);
        t.psi2 = cdd_psi(t.z2, t.e2);
        t.Y = cs_norm(cs_sub(cs_scale(psi1, k.ic1s), cs_scale(t.psi2, k.ic2s)));
        return t;
    }
    const dd ir = dd{rinv, rinv * fmaf(-r, rinv, 1.0f)};  // 1/r: rinv (1 + (1 - r rinv))
    const dd ir2 = sd_mul(ir, ir);
    const cdd W = cdd{sd_mul(k.is2.x, ir2), sd_mul(k.is2.y, ir2)};  // 1 / (s^2 r^2)
    const cdd a2 = cs_add(t.e2, cs_mul(t.z2, t.e2));                 // (1 + z2) e2
    if (az1 < 0.01f) {  // z1 on the series, z2 closed
        const cdd psi1 = cdd_psi(t.z1, t.e1);
        cdd n2 = a2;
        n2.x = sd_norm(sd_add(n2.x, dd{-1.0f, 0.0f}));
        n2.y = sd_norm(n2.y);
        const cdd p2s = cs_mul(n2, W);  // psi2 / c2^2
        if (PSI2) t.psi2 = cs_scale(p2s, k.c2sq);
        t.Y = cs_norm(cs_sub(cs_scale(psi1, k.ic1s), p2s));
        return t;
    }
    const cdd a1 = cs_add(t.e1, cs_mul(t.z1, t.e1));  // (1 + z1) e1
    t.Y = cs_mul(cs_norm(cs_sub(a1, a2)), W);
    if (PSI2) {
        cdd n2 = a2;
        n2.x = sd_norm(sd_add(n2.x, dd{-1.0f, 0.0f}));
        n2.y = sd_norm(n2.y);
        t.psi2 = cs_scale(cs_mul(n2, W), k.c2sq);
    }
    return t;
}

// x * w accumulated into acc: one TwoSum on the high words; the product's rounding error and the low
// words are summed in float.  acc.lo is left unnormalised (a face adds at most a few dozen terms);
// dd_norm() renormalises it.
__device__ __forceinline__ void dd_fma_acc(dd &acc, dd x, float w) {
    const float p = SOD_MUL_RN(x.hi, w);
    const float e = fmaf(x.hi, w, -p);
    const dd s = two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo += s.lo + fmaf(x.lo, w, e);
}
__device__ __forceinline__ void cdd_fma_acc(cdd &acc, const cdd &x, float w) {
    dd_fma_acc(acc.x, x.x, w);
    dd_fma_acc(acc.y, x.y, w);
}
__device__ __forceinline__ dd dd_norm(dd a) { return fast_two_sum(a.hi, a.lo); }
__device__ __forceinline__ cdd cdd_norm(const cdd &a) { return cdd{dd_norm(a.x), dd_norm(a.y)}; }
__device__ __forceinline__ cdd cdd_zero() { return cdd{dd{0.f, 0.f}, dd{0.f, 0.f}}; }
__device__ __forceinline__ float4 f4(const cdd &a) { return make_float4(a.x.hi, a.x.lo, a.y.hi, a.y.lo); }
__device__ __forceinline__ cdd cdd4(const float4 v) { return cdd{dd{v.x, v.y}, dd{v.z, v.w}}; }
__device__ __forceinline__ cdd cdd_scale(const cdd &a, dd s) { return cdd{a.x * s, a.y * s}; }
__device__ __forceinline__ cdd cdd_scale(const cdd &a, float s) { return cdd{a.x * s, a.y * s}; }

// ---------------------------------------------------------------------------------------------
// G / H scatter.  ROW: double-float row block, shared (per-CTA dynamic shared memory) or a global
// slice; layout [NC][nV] float4.
template <int KIND>
__device__ __forceinline__ void comp_scatter_body(const CollArgs &a, const PointTable &pt, const KDD &k,
                                                  int i, int fq, float4 *acc, ColourBar *cb, unsigned &phase,
                                                  const DdTabs *tb) {
    constexpr int NC = KIND == SOD_G ? 6 : 9;
    const int nV = a.nV;
    for (int t = threadIdx.x; t < NC * nV; t += blockDim.x) acc[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    __syncthreads();
    if (a.do_regular) {
        for (int c = 0; c < a.ncolors; c++) {
            const int fend = a.color_off[c + 1];
            bool ready = c == 0;
            for (int f = a.color_off[c] + threadIdx.x; f < fend; f += blockDim.x) {
                const FaceRec fr = load_face(a.faces, f);
                if (is_singular(a, i, ci, f, fr)) continue;
                const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
                cdd part[3][NC];
#pragma unroll
                for (int kk = 0; kk < 3; kk++)
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) part[kk][cc] = cdd_zero();
                for (int q = 0; q < pt.n; q++) {
                    const float4 P = pt.p[q];
                    const float yx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x;
                    const float yy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y;
                    const float yz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z;
                    const float dx = yx - x.x, dy = yy - x.y, dz = yz - x.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    const float rinv = rsqrtf(r2);
                    const float r = r2 * rinv;
                    const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                    const RadDD t = radial_dd<false>(r, rinv, k, tb);
                    cdd u[NC];
                    if (KIND == SOD_G) {
                        // alpha = (3Y + e1/c1^2 - e2/c2^2) / (4 pi rho r), beta = (e2/c2^2 - Y) / (4 pi rho r)
                        const dd p = sd_mulf(k.inv4pirho, rinv);
                        const cdd C2 = cs_scale(t.e2, k.ic2s);
                        const cdd al = cs_scale(cs_norm(cs_sub(cs_add(cs_scalef(t.Y, 3.0f), cs_scale(t.e1, k.ic1s)), C2)), p);
                        const cdd be = cs_scale(cs_norm(cs_sub(C2, t.Y)), p);
#pragma unroll
                        for (int pp = 0; pp < 3; pp++)
#pragma unroll
                            for (int qq = pp; qq < 3; qq++) {
                                cdd v = cs_scalef(al, rh[pp] * rh[qq]);
                                if (pp == qq) v = cs_add(v, be);
                                u[sym_index(pp, qq)] = v;
                            }
                    } else {
                        // a, b, d of the traction kernel, scaled by 1 / (4 pi r^2)
                        const cdd Yc = cs_scale(t.Y, k.six_c2s);
                        const cdd z1e1 = cs_mul(t.z1, t.e1), z2e2 = cs_mul(t.z2, t.e2);
                        const dd p = sd_mulf(k.inv4pi, rinv * rinv);
                        const cdd ha = cs_scale(cs_norm(cs_sub(cs_sub(cs_add(Yc, cs_scale(t.e1, k.k4m1)), cs_scalef(t.e2, 2.0f)),
                                                               cs_scale(z1e1, k.k1m2))),
                                                p);
                        const cdd hb = cs_scale(cs_norm(cs_sub(cs_sub(cs_add(Yc, cs_scale(t.e1, k.k2)), cs_scalef(t.e2, 3.0f)), z2e2)), p);
                        const cdd hd = cs_scale(
                            cs_norm(cs_sub(cs_sub(cs_add(cs_sub(cs_scalef(z2e2, 2.0f), cs_scale(z1e1, k.k2)), cs_scalef(t.e2, 12.0f)),
                                                  cs_scale(t.e1, k.k12)),
                                           cs_scalef(Yc, 5.0f))),
                            p);
                        const float rn = rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2];
                        const cdd hdr = cs_scalef(hd, rn), hbr = cs_scalef(hb, rn);
#pragma unroll
                        for (int pp = 0; pp < 3; pp++)
#pragma unroll
                            for (int qq = 0; qq < 3; qq++) {
                                cdd v = cs_add(cs_add(cs_scalef(hdr, rh[pp] * rh[qq]), cs_scalef(hb, nn[pp] * rh[qq])),
                                               cs_scalef(ha, rh[pp] * nn[qq]));
                                if (pp == qq) v = cs_add(v, hbr);
                                u[3 * pp + qq] = v;
                            }
                    }
                    const float w = P.w * fr.area;
                    const float wl[3] = {w * P.x, w * P.y, w * P.z};
#pragma unroll
                    for (int kk = 0; kk < 3; kk++)
#pragma unroll
                        for (int cc = 0; cc < NC; cc++) cdd_fma_acc(part[kk][cc], u[cc], wl[kk]);
                }
                if (!ready) {
                    colour_wait(cb, (phase + c - 1) & 1u, a.err);
                    ready = true;
                }
                const int jj[3] = {fr.j0, fr.j1, fr.j2};
#pragma unroll
                for (int kk = 0; kk < 3; kk++)
#pragma unroll
                    for (int cc = 0; cc < NC; cc++) {
                        float4 &s = acc[cc * nV + jj[kk]];
                        // sloppy double-float add (TwoSum of the high words, low words summed): a row
                        // entry takes the parts of its ~6 faces, and the epilogue adds hi + lo in FP64
                        s = f4(cs_add(cdd4(s), part[kk][cc]));
                    }
            }
            if (c + 1 < a.ncolors) {
                if (!ready) colour_wait(cb, (phase + c - 1) & 1u, a.err);
                colour_arrive(cb);
            }
        }
        if (a.ncolors > 0) phase += (unsigned)(a.ncolors - 1);
        __syncthreads();
    }
    const long long ld = 3LL * nV;
    const long long base = (long long)fq * a.fstride[KIND] + (long long)(3 * i) * ld;
    const int ncol = 3 * nV;
    for (int p = 0; p < 3; p++) {
        for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
            const int j = col / 3, qq = col - 3 * j;
            const int comp = KIND == SOD_G ? sym_index(p, qq) : 3 * p + qq;
            const float4 v = acc[comp * nV + j];
            store_out(a.out[KIND], a.out_c64, base + p * ld + col, (double)v.x + (double)v.y, (double)v.z + (double)v.w);
        }
    }
    if (a.S[KIND]) {
        __syncthreads();
        const int s0 = a.nbr_off[i], ns = a.nbr_off[i + 1] - s0;
        for (int e = threadIdx.x; e < ns * 9; e += blockDim.x) {
            const int sl = s0 + e / 9, pq = e % 9, p = pq / 3, qq = pq % 3;
            const int j = a.nbr_vert[sl];
            const int comp = KIND == SOD_G ? sym_index(p, qq) : pq;
            const float4 v = acc[comp * nV + j];
            const cd sv = a.S[KIND][(long long)fq * a.S_fstride[KIND] + (long long)sl * 9 + pq];
            store_out(a.out[KIND], a.out_c64, base + p * ld + 3 * j + qq, ((double)v.x + (double)v.y) + sv.x,
                      ((double)v.z + (double)v.w) + sv.y);
        }
    }
}

constexpr int COMP_SCATTER_THREADS = 256;

template <int KIND>
__global__ void __launch_bounds__(COMP_SCATTER_THREADS) comp_scatter_kernel(CollArgs a, PointTable pt,
                                                                          const __grid_constant__ KddTable kt) {
    extern __shared__ float4 acc4[];
    __shared__ ColourBar cb;
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    colour_bar_init(&cb, a.bar_extra);
    unsigned phase = 0;
    comp_scatter_body<KIND>(a, pt, kt.k[blockIdx.y], a.i0 + blockIdx.x, blockIdx.y, acc4, &cb, phase, &tb);
}

// persistent grid, each CTA's row block in its own slice of global memory (L2-resident)
template <int KIND>
__global__ void __launch_bounds__(COMP_SCATTER_THREADS) comp_scatter_global_kernel(CollArgs a, PointTable pt,
                                                                                 const __grid_constant__ KddTable kt,
                                                                                 float4 *scratch, long long per_cta,
                                                                                 int nvert) {
    float4 *acc = scratch + (size_t)blockIdx.x * per_cta;
    __shared__ ColourBar cb;
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    colour_bar_init(&cb, a.bar_extra);
    unsigned phase = 0;
    const int items = nvert * kt.n;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
        const int fq = it / nvert, i = a.i0 + it % nvert;
        comp_scatter_body<KIND>(a, pt, kt.k[fq], i, fq, acc, &cb, phase, &tb);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------
// B_trans / B_angular (MASK subset of KM_BT | KM_BA): per-face moments in double-float registers,
// face tensors into the thread's own column of a shared [NC][T] double-float block, then column sums.
constexpr int COMP_REDUCE_THREADS = 128;

template <int MASK>
__global__ void __launch_bounds__(COMP_REDUCE_THREADS) comp_reduce_kernel(CollArgs a, PointTable pt,
                                                                        const __grid_constant__ KddTable kt) {
    constexpr bool BT = (MASK & KM_BT) != 0, BA = (MASK & KM_BA) != 0;
    constexpr int NT = BT ? 6 : 0, NA = BA ? 18 : 0, NCB = NT + NA;
    extern __shared__ float4 colB[];  // [NCB][T]
    __shared__ cd bsum[24];
    __shared__ DdTabs tb;
    dd_tabs_load(&tb);
    const int i = a.i0 + blockIdx.x, fq = blockIdx.y;
    const KDD &k = kt.k[fq];
    const int T = blockDim.x;
#pragma unroll
    for (int cc = 0; cc < NCB; cc++) colB[cc * T + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 x = make_float3(a.Vf[3 * i], a.Vf[3 * i + 1], a.Vf[3 * i + 2]);
    const int ci = a.canonV ? a.canonV[i] : i;
    __syncthreads();  // the tables
    // B_trans / B_angular scalar factors (with 1/(4 pi))
    const dd hp = k.inv4pi * 0.5f;
    const dd dia_f = k.ic2s * k.inv4pi;
    const cdd bq_f = cdd_scale(k.is, hp);                 // 1 / (2 s) / (4 pi)
    const cdd cq_f = cdd_scale(k.is, k.ic2 * k.inv4pi);   // 1 / (c2 s) / (4 pi)
    if (a.do_regular) {
        for (int f = threadIdx.x; f < a.nF; f += T) {
            const FaceRec fr = load_face(a.faces, f);
            if (is_singular(a, i, ci, f, fr)) continue;
            const float nn[3] = {fr.n.x, fr.n.y, fr.n.z};
            cdd Ms[3], Md, M1[6], M0, SB, SC;
#pragma unroll
            for (int c = 0; c < 3; c++) Ms[c] = cdd_zero();
#pragma unroll
            for (int c = 0; c < 6; c++) M1[c] = cdd_zero();
            Md = M0 = SB = SC = cdd_zero();
            for (int q = 0; q < pt.n; q++) {
                const float4 P = pt.p[q];
                const float dx = P.x * fr.y1.x + P.y * fr.y2.x + P.z * fr.y3.x - x.x;
                const float dy = P.x * fr.y1.y + P.y * fr.y2.y + P.z * fr.y3.y - x.y;
                const float dz = P.x * fr.y1.z + P.y * fr.y2.z + P.z * fr.y3.z - x.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float rinv = rsqrtf(r2);
                const float r = r2 * rinv;
                const float rh[3] = {dx * rinv, dy * rinv, dz * rinv};
                const RadDD t = radial_dd<true>(r, rinv, k, &tb);
                const float w = P.w;
                if (BT) {
                    const cdd ws = cdd_scale(t.Y, hp * w);
#pragma unroll
                    for (int p = 0; p < 3; p++) cdd_fma_acc(Ms[p], ws, rh[p]);
                    cdd_fma_acc(Md, cdd_scale(t.psi2, dia_f), w * (rh[0] * nn[0] + rh[1] * nn[1] + rh[2] * nn[2]));
                }
                if (BA) {
                    const cdd wA = cdd_scale(t.Y, hp * (r * w));
#pragma unroll
                    for (int p = 0; p < 3; p++)
#pragma unroll
                        for (int kk = p; kk < 3; kk++) cdd_fma_acc(M1[sym_index(p, kk)], wA, rh[p] * rh[kk]);
                    cdd_fma_acc(M0, wA, 1.0f);
                    const cdd d21 = cdd_scale(t.e2, k.ic2) - cdd_scale(t.e1, k.ic1);
                    cdd_fma_acc(SB, d21 * bq_f, w);
                    cdd_fma_acc(SC, t.e2 * cq_f, w);
                }
            }
            const float ar = fr.area;
            float4 *col = colB + threadIdx.x;
            if (BT) {
#pragma unroll
                for (int p = 0; p < 3; p++) Ms[p] = cdd_norm(Ms[p]);
                Md = cdd_norm(Md);
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int qq = p; qq < 3; qq++) {
                        cdd v = cdd_scale(Ms[p], nn[qq]) + cdd_scale(Ms[qq], nn[p]);
                        if (p == qq) v = v + Md;
                        float4 &s = col[sym_index(p, qq) * T];
                        s = f4(cdd4(s) + cdd_scale(v, ar));
                    }
            }
            if (BA) {
#pragma unroll
                for (int c = 0; c < 6; c++) M1[c] = cdd_norm(M1[c]);
                const cdd M0B = cdd_norm(M0) + cdd_norm(SB);
                SC = cdd_norm(SC);
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int qq = p; qq < 3; qq++)
#pragma unroll
                        for (int kk = 0; kk < 3; kk++) {
                            cdd v = cdd_scale(M1[sym_index(p, kk)], nn[qq]) + cdd_scale(M1[sym_index(qq, kk)], nn[p]);
                            const float t2 = (qq == kk ? nn[p] : 0.f) + (p == kk ? nn[qq] : 0.f);
                            if (t2 != 0.f) v = v + cdd_scale(M0B, t2);
                            if (p == qq) v = v + cdd_scale(SC, nn[kk]);
                            float4 &s = col[(NT + 3 * sym_index(p, qq) + kk) * T];
                            s = f4(cdd4(s) + cdd_scale(v, ar));
                        }
            }
        }
    }
    __syncthreads();
    // column sums in double-float: 32 lanes per component, strided partial sums, fixed xor tree
    for (int p = threadIdx.x; p < NCB * 32; p += T) {
        const int cc = p >> 5, l = p & 31;
        cdd s = cdd_zero();
        for (int j = l; j < T; j += 32) s = s + cdd4(colB[cc * T + j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const cdd u = cdd{dd{__shfl_xor_sync(0xffffffffu, s.x.hi, o), __shfl_xor_sync(0xffffffffu, s.x.lo, o)},
                              dd{__shfl_xor_sync(0xffffffffu, s.y.hi, o), __shfl_xor_sync(0xffffffffu, s.y.lo, o)}};
            s = s + u;
        }
        if (l == 0) bsum[cc] = mk(dd_to(s.x), dd_to(s.y));
    }
    __syncthreads();
    store_b<MASK>(a, bsum, i, fq);
}

// ---------------------------------------------------------------------------------------------
// host side

static size_t comp_row_bytes(int kind, int nV) { return sizeof(float4) * (size_t)(kind == SOD_G ? 6 : 9) * nV; }
static size_t comp_colb_bytes(int mask) {
    return sizeof(float4) * (size_t)(((mask & KM_BT) ? 6 : 0) + ((mask & KM_BA) ? 18 : 0)) * COMP_REDUCE_THREADS;
}

template <class F> static int raise_smem(sod_context *ctx, F fn) {
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, (const void *)fn));
    SOD_CHECK_CUDA(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(ctx->smem_optin - attr.sharedSizeBytes)));
    return SOD_OK;
}

// CTA size of the compensated scatter for a mesh and kind.  A colour holds at most T faces and the
// CTA waits for each colour's adds, so on small meshes (a few hundred faces in ~10 colours) a 256-thread
// CTA leaves most lanes idle at every colour; smaller CTAs, several per SM, keep them busy.  Cost model
// as for the fast pass: colours x T / occupancy, occupancy = resident warps per SM / 8 (the registers
// of these kernels allow 8 warps of 256 threads), capped at 1.  Row blocks beyond shared memory run in
// the global-memory variant with 256 threads.  Cached on the mesh.
int comp_scatter_threads(sod_context *ctx, sod_mesh *m, int kind, int *threads) {
    const int key = 8192 + kind;
    std::lock_guard<std::recursive_mutex> lock(m->sched_mu);
    auto it = m->tuned.find(key);
    if (it != m->tuned.end()) {
        *threads = it->second;
        return SOD_OK;
    }
    const size_t smem = comp_row_bytes(kind, m->nV);
    const void *fn = kind == SOD_G ? (const void *)comp_scatter_kernel<SOD_G> : (const void *)comp_scatter_kernel<SOD_H>;
    cudaFuncAttributes attr;
    SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
    int best_t = COMP_SCATTER_THREADS;
    if (smem + attr.sharedSizeBytes <= ctx->smem_optin) {
        if (kind == SOD_G) SOD_TRY(raise_smem(ctx, comp_scatter_kernel<SOD_G>));
        else SOD_TRY(raise_smem(ctx, comp_scatter_kernel<SOD_H>));
        double best = 1e300;
        for (int T = 32; T <= COMP_SCATTER_THREADS; T *= 2) {
            int per_sm = 0;
            SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem));
            if (per_sm <= 0) continue;
            const sod_mesh::Coloured *col = nullptr;
            SOD_TRY(m->coloured_for(T, &col));
            const double occ = std::min(1.0, (double)per_sm * T / 32.0 / 8.0);
            const double cost = (double)col->ncolors * T / occ;
            if (cost < best * 0.999) best = cost, best_t = T;
        }
    }
    m->tuned[key] = best_t;
    *threads = best_t;
    return SOD_OK;
}

// The regular pass of one chunk of field vertices [a.i0, a.i0 + nvert) for the kinds in `mask`:
// G / H through the compensated scatter (faces/colours of `colG` / `colH`, coloured for threads[kind]
// from comp_scatter_threads), B kinds through the compensated reduction (natural face order).
int launch_regular_compensated(sod_context *ctx, const sod_mesh *m, CollArgs a, int mask,
                               const sod_mesh::Coloured *colG, const sod_mesh::Coloured *colH, const int threads[2],
                               const PointTable &pt, const FreqTable &ft, int nvert, cudaStream_t stream) {
    const dim3 grid(nvert, ft.n);
    KddTable kt;
    kt.n = ft.n;
    for (int l = 0; l < ft.n; l++) kt.k[l] = kdd_from(ft.kd[l]);
    for (int kd = 0; kd < 2; kd++) {
        if (!(mask & (1 << kd))) continue;
        const sod_mesh::Coloured *col = kd == SOD_G ? colG : colH;
        a.faces = col->dFaces.as<float4>();
        a.canonF = m->has_vmap ? col->dCanonF.as<int4>() : nullptr;
        a.color_off = col->dOff.as<int>();
        a.ncolors = col->ncolors;
        const size_t smem = comp_row_bytes(kd, m->nV);
        const void *fn = kd == SOD_G ? (const void *)comp_scatter_kernel<SOD_G> : (const void *)comp_scatter_kernel<SOD_H>;
        cudaFuncAttributes attr;
        SOD_CHECK_CUDA(cudaFuncGetAttributes(&attr, fn));
        if (smem + attr.sharedSizeBytes <= ctx->smem_optin) {
            if (kd == SOD_G) {
                SOD_TRY(raise_smem(ctx, comp_scatter_kernel<SOD_G>));
                comp_scatter_kernel<SOD_G><<<grid, threads[SOD_G], smem, stream>>>(a, pt, kt);
            } else {
                SOD_TRY(raise_smem(ctx, comp_scatter_kernel<SOD_H>));
                comp_scatter_kernel<SOD_H><<<grid, threads[SOD_H], smem, stream>>>(a, pt, kt);
            }
        } else {
            const void *gfn = kd == SOD_G ? (const void *)comp_scatter_global_kernel<SOD_G>
                                          : (const void *)comp_scatter_global_kernel<SOD_H>;
            int per_sm = 0;
            SOD_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gfn, COMP_SCATTER_THREADS, 0));
            const int g = std::max(1, std::min(ctx->num_sms * std::max(per_sm, 1), nvert * ft.n));
            const long long per_cta = (long long)(smem / sizeof(float4));
            SOD_TRY(ctx->gacc.ensure(sizeof(float4) * (size_t)g * per_cta));
            if (kd == SOD_G)
                comp_scatter_global_kernel<SOD_G><<<g, COMP_SCATTER_THREADS, 0, stream>>>(a, pt, kt, ctx->gacc.as<float4>(),
                                                                                         per_cta, nvert);
            else
                comp_scatter_global_kernel<SOD_H><<<g, COMP_SCATTER_THREADS, 0, stream>>>(a, pt, kt, ctx->gacc.as<float4>(),
                                                                                         per_cta, nvert);
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    const int bm = mask & (KM_BT | KM_BA);
    if (bm) {
        a.faces = m->dFacesNat.as<float4>();
        a.canonF = m->has_vmap ? m->dCanonNat.as<int4>() : nullptr;
        const size_t smem = comp_colb_bytes(bm);
        if (bm == KM_BT) {
            SOD_TRY(raise_smem(ctx, comp_reduce_kernel<KM_BT>));
            comp_reduce_kernel<KM_BT><<<grid, COMP_REDUCE_THREADS, smem, stream>>>(a, pt, kt);
        } else if (bm == KM_BA) {
            SOD_TRY(raise_smem(ctx, comp_reduce_kernel<KM_BA>));
            comp_reduce_kernel<KM_BA><<<grid, COMP_REDUCE_THREADS, smem, stream>>>(a, pt, kt);
        } else {
            SOD_TRY(raise_smem(ctx, comp_reduce_kernel<KM_BT | KM_BA>));
            comp_reduce_kernel<KM_BT | KM_BA><<<grid, COMP_REDUCE_THREADS, smem, stream>>>(a, pt, kt);
        }
        SOD_CHECK_CUDA(cudaGetLastError());
        ctx->count();
    }
    return SOD_OK;
}

}  // namespace sod
