/*
 * sod_oracle.cpp -- CPU oracle for the CQBEM precomputation path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (surfaceonlydeformables_gb300/) links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py use it, and only as the checker or as the timed CPU baseline.
 *
 * PARITY UNPINNED: the reference (rsugimoto/SurfaceOnlyDeformables) ships no tests, fixtures or
 * golden vectors, and cannot be compiled here (its Eigen and libigl submodules are empty and
 * there is no network).  This file restates the reference's algorithms in plain C++ so that
 * they can be checked by known-answer tests (quadrature exactness, closed-form CQ weights,
 * static Kelvin limits of G and H, collocation and Galerkin; the rigid-body identity of H's
 * diagonal with the free term; B_trans and B_angular as the body-force volume integrals of the
 * Kelvin tensor, and Galerkin B as the mass matrix times collocation B; symmetries, rigid-mode
 * null spaces) instead.
 *
 * Precision modes:
 *   mode 0  FP64 everywhere, kernels in their cancellation-free form (the reference's formulas
 *           lose up to ~9 digits in FP64 as |s| r -> 0; see psi_stable)  -> the accuracy oracle
 *   mode 1  "reference-mixed": the scalar types the reference picks per kernel
 *           (FP32 regular G/B_trans/B_angular collocation, FP64 regular H collocation,
 *           FP32 Galerkin non-singular, FP64 singular integrals, FP32 B row accumulators)
 *           -> the restated reference CPU path, used as the timed CPU baseline.
 *   mode 2  FP32 for every regular (non-singular) integral including H  -> precision study only.
 *   mode 3  FP64 everywhere with the reference's literal kernel formulas  -> precision study only
 *           (agrees with mode 0 wherever |s| r is not small).
 *
 * The loop structure (per-component singular integration, per-k B_angular passes, per-face
 * accumulation then scatter) follows the reference so that the baseline's cost is
 * representative.  Every function cites the reference lines it restates.
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.14159265358979323846;

// ---------------------------------------------------------------------------------------------
// small vector type
template <class T> struct V3 {
    T x, y, z;
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T norm(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> V3<T> normalized(V3<T> a) {
    T n = norm(a);
    return n > T(0) ? a / n : a;
}
template <class T> V3<T> load(const double *V, long i) {
    return {(T)V[3 * i], (T)V[3 * i + 1], (T)V[3 * i + 2]};
}
template <class T> using cplx = std::complex<T>;

// ---------------------------------------------------------------------------------------------
// Quadrature tables.
// Triangle rules of Cowper (1973), degrees 1..5, restated from include/integrator.hpp:61-88;
// {l0, l1, l2, weight} with point = l0*x0 + l1*x1 + l2*x2 and weights summing to 1.
const double TRI1[][4] = {{1. / 3., 1. / 3., 1. / 3., 1.}};
const double TRI2[][4] = {{0., .5, .5, 1. / 3.}, {.5, 0., .5, 1. / 3.}, {.5, .5, 0., 1. / 3.}};
const double TRI3[][4] = {{1. / 3., 1. / 3., 1. / 3., -27. / 48.},
                          {11. / 15., 2. / 15., 2. / 15., 25. / 48.},
                          {2. / 15., 11. / 15., 2. / 15., 25. / 48.},
                          {2. / 15., 2. / 15., 11. / 15., 25. / 48.}};
constexpr double A4 = 0.445948490915965, B4 = 0.111690794839005 * 2., C4 = 0.091576213509771,
                 D4 = 0.054975871827661 * 2.;
const double TRI4[][4] = {{1. - 2. * A4, A4, A4, B4}, {A4, 1. - 2. * A4, A4, B4}, {A4, A4, 1. - 2. * A4, B4},
                          {1. - 2. * C4, C4, C4, D4}, {C4, 1. - 2. * C4, C4, D4}, {C4, C4, 1. - 2. * C4, D4}};
constexpr double A5 = 0.470142064105115, B5 = 0.0661970763942530 * 2., C5 = 0.101286507323456,
                 D5 = 0.0629695902724135 * 2.;
const double TRI5[][4] = {{1. / 3., 1. / 3., 1. / 3., 9. / 40.},  {1. - 2. * A5, A5, A5, B5},
                          {A5, 1. - 2. * A5, A5, B5},             {A5, A5, 1. - 2. * A5, B5},
                          {1. - 2. * C5, C5, C5, D5},             {C5, 1. - 2. * C5, C5, D5},
                          {C5, C5, 1. - 2. * C5, D5}};
// 13-point degree-7 rule (Cowper 1973 / Dunavant 1985), digits fixed by oracle/gen_tri13.py.
// Not present in the reference; requested as "order 7" (13 points).
const double TRI7[][4] = {
    {3.3333333333333333333e-1, 3.3333333333333333333e-1, 3.3333333333333333333e-1, -1.4957004446768175063e-1},
    {4.7930806784192034615e-1, 2.6034596607903982693e-1, 2.6034596607903982693e-1, 1.7561525743320781175e-1},
    {2.6034596607903982693e-1, 4.7930806784192034615e-1, 2.6034596607903982693e-1, 1.7561525743320781175e-1},
    {2.6034596607903982693e-1, 2.6034596607903982693e-1, 4.7930806784192034615e-1, 1.7561525743320781175e-1},
    {8.6973979419556837692e-1, 6.5130102902215811538e-2, 6.5130102902215811538e-2, 5.334723560883849127e-2},
    {6.5130102902215811538e-2, 8.6973979419556837692e-1, 6.5130102902215811538e-2, 5.334723560883849127e-2},
    {6.5130102902215811538e-2, 6.5130102902215811538e-2, 8.6973979419556837692e-1, 5.334723560883849127e-2},
    {4.8690315425316411793e-2, 3.1286549600487386141e-1, 6.384441885698097268e-1, 7.711376089025714026e-2},
    {4.8690315425316411793e-2, 6.384441885698097268e-1, 3.1286549600487386141e-1, 7.711376089025714026e-2},
    {3.1286549600487386141e-1, 4.8690315425316411793e-2, 6.384441885698097268e-1, 7.711376089025714026e-2},
    {3.1286549600487386141e-1, 6.384441885698097268e-1, 4.8690315425316411793e-2, 7.711376089025714026e-2},
    {6.384441885698097268e-1, 4.8690315425316411793e-2, 3.1286549600487386141e-1, 7.711376089025714026e-2},
    {6.384441885698097268e-1, 3.1286549600487386141e-1, 4.8690315425316411793e-2, 7.711376089025714026e-2}};

struct TriRule {
    const double (*p)[4];
    int n;
};
TriRule tri_rule(int order) {
    switch (order) {
    case 1: return {TRI1, 1};
    case 2: return {TRI2, 3};
    case 3: return {TRI3, 4};
    case 4: return {TRI4, 6};
    case 5: return {TRI5, 7};
    case 7: return {TRI7, 13};
    default: return {nullptr, 0};
    }
}

// 1-D Gauss-Legendre on [-1, 1], orders 1..5, restated from include/integrator.hpp:117-133.
const double GL1[][2] = {{0., 2.}};
const double GL2[][2] = {{-0.5773502691896257645092, 1.}, {0.5773502691896257645092, 1.}};
const double GL3[][2] = {{-0.7745966692414833770359, 0.5555555555555555555556},
                         {0., 0.8888888888888888888889},
                         {0.7745966692414833770359, 0.555555555555555555556}};
const double GL4[][2] = {{-0.861136311594052575224, 0.3478548451374538573731},
                         {-0.3399810435848562648027, 0.6521451548625461426269},
                         {0.3399810435848562648027, 0.6521451548625461426269},
                         {0.861136311594052575224, 0.3478548451374538573731}};
const double GL5[][2] = {{-0.9061798459386639927976, 0.2369268850561890875143},
                         {-0.5384693101056830910363, 0.4786286704993664680413},
                         {0., 0.5688888888888888888889},
                         {0.5384693101056830910363, 0.4786286704993664680413},
                         {0.9061798459386639927976, 0.2369268850561890875143}};
struct GLRule {
    const double (*p)[2];
    int n;
};
GLRule gl_rule(int order) {
    switch (order) {
    case 1: return {GL1, 1};
    case 2: return {GL2, 2};
    case 3: return {GL3, 3};
    case 4: return {GL4, 4};
    case 5: return {GL5, 5};
    default: return {nullptr, 0};
    }
}

// ---------------------------------------------------------------------------------------------
// Integration drivers

// Sum over subdivided sub-triangles of the Gauss rule (include/integrator.hpp:24-51 and :55-113,
// include/integrator_collocation.hpp:7-17).  `acc(point, weight)` accumulates into a per-triangle
// temporary `tmp`; after each sub-triangle tmp is scaled by the sub-triangle area and added to `out`.
// R must provide zero(), axpy(...) semantics through the callbacks.
template <class T, class PointFn>
void for_each_subtriangle(const V3<T> &x0, const V3<T> &x1, const V3<T> &x2, int subdiv, PointFn sub) {
    const T n = (T)subdiv;
    const V3<T> d1 = x1 - x0, d2 = x2 - x0;
    // first upright triangle, then the loop order of integrator.hpp:30-49
    sub(x0, x0 + d1 / n, x0 + d2 / n);
    for (int i = 0; i < subdiv; i++) {
        for (int j = 0; j < subdiv; j++) {
            const V3<T> o = x0 + ((T)i * d1 + (T)j * d2) / n;
            if (!(i == 0 && j == 0) && i + j < subdiv) sub(o, o + d1 / n, o + d2 / n);
            if (i + j < subdiv - 1) sub(o + d1 / n + d2 / n, o + d1 / n, o + d2 / n);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Kernels.  All return r * K (the "r_" forms of the reference) unless stated.

template <class T> struct Mat {
    T c1, c2, rho;
    cplx<T> s;
    bool stable = false;  // FP64 accuracy mode: the cancellation-free forms below
};
template <class T> inline T kd(int i, int j) { return i == j ? T(1) : T(0); }

// ---- cancellation-free forms of the four kernels (the FP64 accuracy mode) -------------------------
// The reference's formulas subtract terms of size 1/(s r)^2 (and c^2 / r^2 times that in p_hat) that
// cancel to O(1) as s r -> 0; in FP64 the innermost singular quadrature points (s r ~ 1e-4) lose
// about 9 digits there.  The same functions are evaluated through
//   psi(z) = ((1 + z) e^-z - 1) / z^2,  z_a = s r / c_a,  e_a = e^-z_a,
//   Y = psi(z1)/c1^2 - psi(z2)/c2^2,    kappa = c2^2 / c1^2,
// using the exact identities X / r^2 = Y (X of r_u_hat), X2 - X1 = -r^2 Y and
// 1/s^2 - X2 = -(r^2 / c2^2) psi(z2) (tests/test_kernel_identities.py checks each rearranged kernel
// against the literal one to 1e-36 in 40-digit arithmetic).
// psi: 25-term series below |z| = 1 (truncation < 1e-26), closed form above (loss <= 2 eps/|z|^2).
template <class T> cplx<T> psi_stable(cplx<T> z, cplx<T> ez) {
    if (std::abs(z) < T(1)) {
        // -sum_{m>=0} (-1)^m (m+1) z^m / (m+2)!, Horner from m = 24
        double fact = 1.0;  // (m+2)! for m = 24
        for (int t = 2; t <= 26; t++) fact *= t;
        cplx<T> acc(0);
        for (int m = 24; m >= 0; m--) {
            const T c = T(((m % 2) ? 1.0 : -1.0) * (m + 1) / fact);
            acc = acc * z + c;
            fact /= (m + 2);
        }
        return acc;
    }
    return ((T(1) + z) * ez - T(1)) / (z * z);
}
template <class T> struct Radial {
    cplx<T> z1, z2, e1, e2, psi1, psi2, Y;
};
template <class T> Radial<T> radial_stable(T r, const Mat<T> &m) {
    Radial<T> t;
    t.z1 = m.s * (r / m.c1);
    t.z2 = m.s * (r / m.c2);
    t.e1 = std::exp(-t.z1);
    t.e2 = std::exp(-t.z2);
    t.psi1 = psi_stable(t.z1, t.e1);
    t.psi2 = psi_stable(t.z2, t.e2);
    t.Y = t.psi1 / (m.c1 * m.c1) - t.psi2 / (m.c2 * m.c2);
    return t;
}
// r u_hat = [(3Y + e1/c1^2 - e2/c2^2) rh_i rh_j + (e2/c2^2 - Y) d_ij] / (4 pi rho)
template <class T> cplx<T> r_u_hat_stable(const V3<T> &rh, T r, int i, int j, const Mat<T> &m) {
    const Radial<T> t = radial_stable(r, m);
    const cplx<T> B = t.e1 / (m.c1 * m.c1) - t.e2 / (m.c2 * m.c2), C = t.e2 / (m.c2 * m.c2);
    return (T(1. / (4. * PI)) / m.rho) * ((T(3) * t.Y + B) * (rh[i] * rh[j]) + (C - t.Y) * kd<T>(i, j));
}
// p_hat = [a rh_i n_j + b (n_i rh_j + rn d_ij) + d rn rh_i rh_j] / (4 pi r^2)
template <class T> cplx<T> p_hat_stable(const V3<T> &rh, T r, const V3<T> &n, int i, int j, const Mat<T> &m) {
    const Radial<T> t = radial_stable(r, m);
    const T kp = (m.c2 * m.c2) / (m.c1 * m.c1), rn = dot(rh, n);
    const cplx<T> Yc = t.Y * (T(6) * m.c2 * m.c2), z1e1 = t.z1 * t.e1, z2e2 = t.z2 * t.e2;
    const cplx<T> a = Yc + t.e1 * (T(4) * kp - T(1)) - t.e2 * T(2) - z1e1 * (T(1) - T(2) * kp);
    const cplx<T> b = Yc + t.e1 * (T(2) * kp) - t.e2 * T(3) - z2e2;
    const cplx<T> d = Yc * T(-5) - t.e1 * (T(12) * kp) + t.e2 * T(12) - z1e1 * (T(2) * kp) + z2e2 * T(2);
    return (T(1. / (4. * PI)) / (r * r)) *
           (a * (rh[i] * n[j]) + b * (n[i] * rh[j] + kd<T>(i, j) * rn) + d * (rn * rh[i] * rh[j]));
}
// r b_trans_hat = r [(Y/2)(rh_i n_j + rh_j n_i) + psi2/c2^2 rn d_ij] / (4 pi)
template <class T> cplx<T> r_b_trans_stable(const V3<T> &rh, T r, const V3<T> &n, int i, int j, const Mat<T> &m) {
    const Radial<T> t = radial_stable(r, m);
    return (r * T(1. / (4. * PI))) *
           ((t.Y / T(2)) * (rh[i] * n[j] + rh[j] * n[i]) + (t.psi2 / (m.c2 * m.c2)) * (dot(rh, n) * kd<T>(i, j)));
}
// r b_ang_hat = r [(r Y/2) T1 + T2 (e2/c2 - e1/c1)/(2s) + d_ij n_k e2/(c2 s)] / (4 pi),
//   T1 = rh_i rh_k n_j + rh_j rh_k n_i + d_jk n_i + d_ik n_j, T2 = d_jk n_i + d_ik n_j
template <class T>
cplx<T> r_b_ang_stable(const V3<T> &rh, T r, const V3<T> &n, int i, int j, int k, const Mat<T> &m) {
    const Radial<T> t = radial_stable(r, m);
    const T T2 = kd<T>(j, k) * n[i] + kd<T>(i, k) * n[j];
    const T T1 = rh[i] * rh[k] * n[j] + rh[j] * rh[k] * n[i] + T2;
    return (r * T(1. / (4. * PI))) * ((r * t.Y / T(2)) * T1 + (t.e2 / m.c2 - t.e1 / m.c1) / (T(2) * m.s) * T2 +
                                      kd<T>(i, j) * n[k] * t.e2 / (m.c2 * m.s));
}

// r * u_hat_ij, elastodynamic single layer (src/elastodynamics_cqbem_G_collocation.cu:44-60)
template <class T> cplx<T> r_u_hat(const V3<T> &rh, T r, int i, int j, const Mat<T> &m) {
    if (m.stable) return r_u_hat_stable(rh, r, i, j, m);
    const cplx<T> s = m.s;
    const cplx<T> e1 = std::exp(-r * s / m.c1), e2 = std::exp(-r * s / m.c2);
    const cplx<T> X = ((s * r / m.c1 + T(1)) / (s * s)) * e1 - ((s * r / m.c2 + T(1)) / (s * s)) * e2;
    return (T(1. / (4. * PI)) / m.rho) *
           (((T(3) * rh[i] * rh[j] - kd<T>(i, j)) / (r * r)) * X +
            (rh[i] * rh[j]) * (e1 / (m.c1 * m.c1) - e2 / (m.c2 * m.c2)) + (kd<T>(i, j) / (m.c2 * m.c2)) * e2);
}

// p_hat_ij, elastodynamic double layer (src/elastodynamics_cqbem_H_collocation.cu:45-76)
template <class T> cplx<T> p_hat(const V3<T> &rh, T r, const V3<T> &n, int i, int j, const Mat<T> &m) {
    if (m.stable) return p_hat_stable(rh, r, n, i, j, m);
    const cplx<T> s = m.s;
    const T c1 = m.c1, c2 = m.c2;
    const cplx<T> e1 = std::exp(-r * s / c1), e2 = std::exp(-r * s / c2);
    const T rn = dot(rh, n);
    const cplx<T> rs = r * s;
    return T(1. / (4. * PI)) *
           ((T(6) * c2 * c2 / (r * r)) * (rh[i] * n[j] + rh[j] * n[i] + (kd<T>(i, j) - T(5) * rh[i] * rh[j]) * rn) *
                ((e1 / rs) * (T(1) / c1 + T(1) / rs) - (e2 / rs) * (T(1) / c2 + T(1) / rs)) +
            (e1 / (r * r)) * (T(2) * c2 * c2 / (c1 * c1) *
                                  (T(2) * rh[i] * n[j] + rh[j] * n[i] - (T(6) * rh[i] * rh[j] - kd<T>(i, j)) * rn) -
                              rh[i] * n[j]) +
            (e2 / (r * r)) * (T(12) * rh[i] * rh[j] * rn - T(2) * rh[i] * n[j] - T(3) * rh[j] * n[i] -
                              T(3) * kd<T>(i, j) * rn) -
            (e1 * s / (r * c1)) * (rh[i] * n[j] + T(2) * c2 * c2 / (c1 * c1) * (rh[i] * rh[j] * rn - rh[i] * n[j])) +
            (e2 * s / (r * c2)) * (T(2) * rh[i] * rh[j] * rn - kd<T>(i, j) * rn - rh[j] * n[i]));
}

// leading singular part of p_hat (src/elastodynamics_cqbem_H_collocation.cu:78-83)
template <class T> T p_hat_sing(const V3<T> &rh, T r, const V3<T> &n, int i, int j, const Mat<T> &m) {
    return T(1. / (4. * PI)) * (m.c2 * m.c2 / (m.c1 * m.c1)) * (rh[i] * n[j] - rh[j] * n[i]) / (r * r);
}

// r * b_hat_ij, rigid-translation coupling (src/elastodynamics_cqbem_B_trans_collocation.cu:41-58)
template <class T> cplx<T> r_b_trans(const V3<T> &rh, T r, const V3<T> &n, int i, int j, const Mat<T> &m) {
    if (m.stable) return r_b_trans_stable(rh, r, n, i, j, m);
    const cplx<T> s = m.s;
    const cplx<T> e1 = std::exp(-r * s / m.c1), e2 = std::exp(-r * s / m.c2);
    const cplx<T> X2 = ((s * r / m.c2 + T(1)) / (s * s)) * e2, X1 = ((s * r / m.c1 + T(1)) / (s * s)) * e1;
    return -T(1. / (4. * PI)) * (((rh[i] * n[j] + rh[j] * n[i]) / (T(2) * r)) * (X2 - X1) +
                                 kd<T>(i, j) * dot(rh, n) / r * (T(1) / (s * s) - X2));
}

// r * b_hat_ijk, rigid-rotation coupling (src/elastodynamics_cqbem_B_angular_collocation.cu:44-63)
template <class T>
cplx<T> r_b_ang(const V3<T> &rh, T r, const V3<T> &n, int i, int j, int k, const Mat<T> &m) {
    if (m.stable) return r_b_ang_stable(rh, r, n, i, j, k, m);
    const cplx<T> s = m.s;
    const cplx<T> e1 = std::exp(-r * s / m.c1), e2 = std::exp(-r * s / m.c2);
    const cplx<T> X2 = ((s * r / m.c2 + T(1)) / (s * s)) * e2, X1 = ((s * r / m.c1 + T(1)) / (s * s)) * e1;
    return -T(1. / (4. * PI)) *
           ((rh[i] * rh[k] * n[j] + rh[j] * rh[k] * n[i] + kd<T>(j, k) * n[i] + kd<T>(i, k) * n[j]) / T(2) *
                (X2 - X1) -
            r * (kd<T>(j, k) * n[i] + kd<T>(i, k) * n[j]) / (T(2) * s) * (e2 / m.c2 - e1 / m.c1) -
            r * (kd<T>(i, j) * n[k]) / (m.c2 * s) * e2);
}

// ---------------------------------------------------------------------------------------------
// barycentric coordinates of P in (A,B,C) (include/barycentric_coordinates.cuh:14-38), clamped
// to [0,1] as the collocation kernels do (e.g. src/elastodynamics_cqbem_G_collocation.cu:96-97)
template <class T> void bary_clamped(const V3<T> &P, const V3<T> &A, const V3<T> &B, const V3<T> &C, T L[3]) {
    const V3<T> v0 = B - A, v1 = C - A, v2 = P - A;
    const T d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    const T den = d00 * d11 - d01 * d01;
    L[1] = (d11 * d20 - d01 * d21) / den;
    L[2] = (d00 * d21 - d01 * d20) / den;
    L[0] = T(1) - (L[1] + L[2]);
    for (int k = 0; k < 3; k++) L[k] = std::min(T(1), std::max(T(0), L[k]));
}

// ---------------------------------------------------------------------------------------------
// Collocation singular rules (FP64 in the reference)

// Polar rule about vertex y1 for weakly singular integrands (include/integrator_collocation.hpp:19-63).
// integrand(y, r_hat, r, out[NC]) adds nothing; it writes NC complex values to out.
template <int NC, class F>
void weakly_singular(const V3<double> &y1, const V3<double> &y2, const V3<double> &y3, int order, int subdiv,
                     F integrand, cplx<double> res[NC]) {
    const V3<double> v1 = y2 - y1, v2 = y3 - y1;
    const V3<double> v1n = normalized(v1), v2n = normalized(v2);
    const V3<double> xh = v1n;
    const V3<double> yh = normalized(cross(cross(xh, v2n), xh));
    const V3<double> v12 = v1 + dot(v1, normalized(v1 - v2)) * normalized(v2 - v1);
    const double a = norm(v12);
    // the angles as atan2(|u x v|, u . v): the reference's acos(u . v) loses half the digits near 0
    // and pi (beta = 0 exactly for a right angle at y2, ~1.5e-8 rad of rounding noise with acos)
    const double alpha = std::atan2(norm(cross(v1n, v2n)), dot(v1n, v2n));
    const V3<double> v12n = normalized(v12);
    const double beta = std::atan2(norm(cross(v12n, v1n)), dot(v12n, v1n));
    const GLRule g = gl_rule(order);
    for (int c = 0; c < NC; c++) res[c] = 0.0;
    for (int ts = 0; ts < subdiv; ts++) {
        const double ta = alpha * ts / subdiv, tb = alpha * (ts + 1) / subdiv;
        cplx<double> tsum[NC];
        for (int c = 0; c < NC; c++) tsum[c] = 0.0;
        for (int tq = 0; tq < g.n; tq++) {
            const double theta = (tb - ta) * g.p[tq][0] / 2. + (ta + tb) / 2.;
            const V3<double> rh = xh * std::cos(theta) + yh * std::sin(theta);
            const double rmax = a / std::cos(theta - beta);
            cplx<double> rsum[NC];
            for (int c = 0; c < NC; c++) rsum[c] = 0.0;
            for (int rs = 0; rs < subdiv; rs++) {
                const double ra = rmax * rs / subdiv, rb = rmax * (rs + 1) / subdiv;
                cplx<double> qsum[NC];
                for (int c = 0; c < NC; c++) qsum[c] = 0.0;
                for (int rq = 0; rq < g.n; rq++) {
                    const double r = (rb - ra) * g.p[rq][0] / 2. + (ra + rb) / 2.;
                    cplx<double> v[NC];
                    integrand(y1 + r * rh, rh, r, v);
                    for (int c = 0; c < NC; c++) qsum[c] += v[c] * g.p[rq][1];
                }
                for (int c = 0; c < NC; c++) rsum[c] += qsum[c] * ((rb - ra) / 2.0);
            }
            for (int c = 0; c < NC; c++) tsum[c] += rsum[c] * g.p[tq][1];
        }
        for (int c = 0; c < NC; c++) res[c] += tsum[c] * ((tb - ta) / 2.0);
    }
}

// Guiggiani-Gigante CPV rule about vertex y1 (include/integrator_collocation.hpp:68-124) for a
// shape-function-weighted strongly singular integrand.  original(r_hat, r) and cancel(r_hat, r)
// return the (complex / real) kernel value; the result is the 3-vector over the linear shape
// functions of (y1, y2, y3).
template <class Orig, class Canc>
void strongly_singular(const V3<double> &y1, const V3<double> &y2, const V3<double> &y3, int order, int subdiv,
                       Orig original, Canc cancel, cplx<double> res[3]) {
    const V3<double> v1 = y2 - y1, v2 = y3 - y1;
    const double J = norm(cross(v1, v2));
    const GLRule g = gl_rule(order);
    for (int c = 0; c < 3; c++) res[c] = 0.0;
    const double tmax = PI / 2.;
    for (int ts = 0; ts < subdiv; ts++) {
        const double ta = tmax * ts / subdiv, tb = tmax * (ts + 1) / subdiv;
        cplx<double> tsum[3] = {0.0, 0.0, 0.0};
        for (int tq = 0; tq < g.n; tq++) {
            const double theta = (tb - ta) * g.p[tq][0] / 2. + (ta + tb) / 2.;
            const double ct = std::cos(theta), st = std::sin(theta);
            const V3<double> Av = ct * v1 + st * v2;
            const V3<double> Ah = normalized(Av);
            const double A = norm(Av);
            const cplx<double> f0 = cancel(Ah, A) * J;  // times L = (1,0,0)
            const double rho_bar = 1. / (std::cos(theta - PI / 4.) * std::sqrt(2.));
            cplx<double> p1[3] = {0.0, 0.0, 0.0};
            for (int rs = 0; rs < subdiv; rs++) {
                const double ra = rho_bar * rs / subdiv, rb = rho_bar * (rs + 1) / subdiv;
                cplx<double> q[3] = {0.0, 0.0, 0.0};
                for (int rq = 0; rq < g.n; rq++) {
                    const double rho = (rb - ra) * g.p[rq][0] / 2. + (ra + rb) / 2.;
                    const double L[3] = {1. - rho * (ct + st), rho * ct, rho * st};
                    const V3<double> rv = rho * Av;
                    const double r = norm(rv);
                    const V3<double> rh = normalized(rv);
                    const cplx<double> o = original(rh, r);
                    for (int c = 0; c < 3; c++) {
                        cplx<double> F = o * (L[c] * J * rho);
                        if (c == 0) F -= f0 / rho;
                        q[c] += F * g.p[rq][1];
                    }
                }
                for (int c = 0; c < 3; c++) p1[c] += q[c] * ((rb - ra) / 2.0);
            }
            p1[0] += f0 * std::log(rho_bar * A);
            for (int c = 0; c < 3; c++) tsum[c] += p1[c] * g.p[tq][1];
        }
        for (int c = 0; c < 3; c++) res[c] += tsum[c] * ((tb - ta) / 2.0);
    }
}

// ---------------------------------------------------------------------------------------------
// Mesh helpers

struct Mesh {
    const double *V;
    long nV;
    const int *F;
    long nF;
    const double *N;
    const int *vmap;
    int f(long face, int k) const { return F[3 * face + k]; }
    bool same(long a, long b) const { return a == b || (vmap && vmap[a] == vmap[b]); }
};

// which corner of `face` coincides with vertex i (-1 if none), first match as in
// src/elastodynamics_cqbem_G_collocation.cu:79-88
int singular_corner(const Mesh &m, long i, long face) {
    for (int k = 0; k < 3; k++)
        if (m.same(i, m.f(face, k))) return k;
    return -1;
}

// ---------------------------------------------------------------------------------------------
// Collocation row assembly (one field vertex i; out points at the first of its 3 rows)
// kinds: 0=G (3V cols), 1=H (3V cols), 2=B_trans (3 cols), 3=B_angular (9 cols, [j][k])

template <class T>
void coll_G_row(const Mesh &m, long i, const Mat<double> &md, int order, int subdiv, int sorder, int ssub,
                int parts, cplx<double> *U, long ld) {
    const Mat<T> mt{(T)md.c1, (T)md.c2, (T)md.rho, cplx<T>(md.s), md.stable && sizeof(T) == sizeof(double)};
    const TriRule rule = tri_rule(order);
    const V3<T> x = load<T>(m.V, i);
    for (long f = 0; f < m.nF; f++) {
        const int sc = singular_corner(m, i, f);
        if (sc < 0) {
            if (!(parts & 1)) continue;
            const long j[3] = {m.f(f, 0), m.f(f, 1), m.f(f, 2)};
            const V3<T> y1 = load<T>(m.V, j[0]), y2 = load<T>(m.V, j[1]), y3 = load<T>(m.V, j[2]);
            cplx<T> mat[9][3] = {};
            for_each_subtriangle<T>(y1, y2, y3, subdiv, [&](V3<T> a, V3<T> b, V3<T> c) {
                cplx<T> tmp[9][3] = {};
                for (int q = 0; q < rule.n; q++) {
                    const V3<T> y = a * (T)rule.p[q][0] + b * (T)rule.p[q][1] + c * (T)rule.p[q][2];
                    T L[3];
                    bary_clamped(y, y1, y2, y3, L);
                    const V3<T> rv = y - x;
                    const V3<T> rh = normalized(rv);
                    const T r = norm(rv);
                    cplx<T> u[3][3];
                    for (int p = 0; p < 3; p++)
                        for (int qq = 0; qq <= p; qq++) {
                            u[p][qq] = r_u_hat(rh, r, p, qq, mt) / r;
                            u[qq][p] = u[p][qq];
                        }
                    for (int k = 0; k < 3; k++)
                        for (int p = 0; p < 3; p++)
                            for (int qq = 0; qq < 3; qq++) tmp[3 * k + p][qq] += (u[p][qq] * L[k]) * (T)rule.p[q][3];
                }
                const T area = norm(cross(b - a, c - a)) / T(2);
                for (int r = 0; r < 9; r++)
                    for (int cc = 0; cc < 3; cc++) mat[r][cc] += tmp[r][cc] * area;
            });
            for (int k = 0; k < 3; k++)
                for (int p = 0; p < 3; p++)
                    for (int qq = 0; qq < 3; qq++) U[p * ld + 3 * j[k] + qq] += cplx<double>(mat[3 * k + p][qq]);
        } else {
            if (!(parts & 2)) continue;
            const long j[3] = {m.f(f, sc), m.f(f, (sc + 1) % 3), m.f(f, (sc + 2) % 3)};
            const V3<double> y1 = load<double>(m.V, j[0]), y2 = load<double>(m.V, j[1]), y3 = load<double>(m.V, j[2]);
            for (int p = 0; p < 3; p++)
                for (int qq = 0; qq <= p; qq++) {
                    cplx<double> e[3];
                    weakly_singular<3>(
                        y1, y2, y3, sorder, ssub,
                        [&](const V3<double> &y, const V3<double> &rh, double r, cplx<double> *v) {
                            double L[3];
                            bary_clamped(y, y1, y2, y3, L);
                            const cplx<double> k = r_u_hat(rh, r, p, qq, md);
                            for (int c = 0; c < 3; c++) v[c] = k * L[c];
                        },
                        e);
                    for (int c = 0; c < 3; c++) {
                        U[p * ld + 3 * j[c] + qq] += e[c];
                        if (p != qq) U[qq * ld + 3 * j[c] + p] += e[c];
                    }
                }
        }
    }
}

template <class T>
void coll_H_row(const Mesh &m, long i, const Mat<double> &md, int order, int subdiv, int sorder, int ssub,
                int parts, cplx<double> *P, long ld) {
    const Mat<T> mt{(T)md.c1, (T)md.c2, (T)md.rho, cplx<T>(md.s), md.stable && sizeof(T) == sizeof(double)};
    const TriRule rule = tri_rule(order);
    const V3<T> x = load<T>(m.V, i);
    for (long f = 0; f < m.nF; f++) {
        const int sc = singular_corner(m, i, f);
        if (sc < 0) {
            if (!(parts & 1)) continue;
            const V3<T> n = load<T>(m.N, f);
            const long j[3] = {m.f(f, 0), m.f(f, 1), m.f(f, 2)};
            const V3<T> y1 = load<T>(m.V, j[0]), y2 = load<T>(m.V, j[1]), y3 = load<T>(m.V, j[2]);
            cplx<T> mat[9][3] = {};
            for_each_subtriangle<T>(y1, y2, y3, subdiv, [&](V3<T> a, V3<T> b, V3<T> c) {
                cplx<T> tmp[9][3] = {};
                for (int q = 0; q < rule.n; q++) {
                    const V3<T> y = a * (T)rule.p[q][0] + b * (T)rule.p[q][1] + c * (T)rule.p[q][2];
                    T L[3];
                    bary_clamped(y, y1, y2, y3, L);
                    const V3<T> rv = y - x;
                    const V3<T> rh = normalized(rv);
                    const T r = norm(rv);
                    for (int p = 0; p < 3; p++)
                        for (int qq = 0; qq < 3; qq++) {
                            const cplx<T> v = p_hat(rh, r, n, p, qq, mt);
                            for (int k = 0; k < 3; k++) tmp[3 * k + p][qq] += (v * L[k]) * (T)rule.p[q][3];
                        }
                }
                const T area = norm(cross(b - a, c - a)) / T(2);
                for (int r = 0; r < 9; r++)
                    for (int cc = 0; cc < 3; cc++) mat[r][cc] += tmp[r][cc] * area;
            });
            for (int k = 0; k < 3; k++)
                for (int p = 0; p < 3; p++)
                    for (int qq = 0; qq < 3; qq++) P[p * ld + 3 * j[k] + qq] += cplx<double>(mat[3 * k + p][qq]);
        } else {
            if (!(parts & 2)) continue;
            const V3<double> n = load<double>(m.N, f);
            const long j[3] = {m.f(f, sc), m.f(f, (sc + 1) % 3), m.f(f, (sc + 2) % 3)};
            const V3<double> y1 = load<double>(m.V, j[0]), y2 = load<double>(m.V, j[1]), y3 = load<double>(m.V, j[2]);
            for (int p = 0; p < 3; p++)
                for (int qq = 0; qq < 3; qq++) {
                    cplx<double> e[3];
                    strongly_singular(
                        y1, y2, y3, sorder, ssub,
                        [&](const V3<double> &rh, double r) { return p_hat(rh, r, n, p, qq, md); },
                        [&](const V3<double> &rh, double r) { return cplx<double>(p_hat_sing(rh, r, n, p, qq, md)); },
                        e);
                    for (int c = 0; c < 3; c++) P[p * ld + 3 * j[c] + qq] += e[c];
                }
        }
    }
}

template <class T>
void coll_Bt_row(const Mesh &m, long i, const Mat<double> &md, int order, int subdiv, int sorder, int ssub,
                 int parts, cplx<double> *B) {
    const Mat<T> mt{(T)md.c1, (T)md.c2, (T)md.rho, cplx<T>(md.s), md.stable && sizeof(T) == sizeof(double)};
    const TriRule rule = tri_rule(order);
    const V3<T> x = load<T>(m.V, i);
    cplx<T> Bi[3][3] = {};  // row accumulator in the kernel precision (B_trans_collocation.cu:39)
    for (long f = 0; f < m.nF; f++) {
        const int sc = singular_corner(m, i, f);
        if (sc < 0) {
            if (!(parts & 1)) continue;
            const V3<T> n = load<T>(m.N, f);
            const V3<T> y1 = load<T>(m.V, m.f(f, 0)), y2 = load<T>(m.V, m.f(f, 1)), y3 = load<T>(m.V, m.f(f, 2));
            cplx<T> mat[3][3] = {};
            for_each_subtriangle<T>(y1, y2, y3, subdiv, [&](V3<T> a, V3<T> b, V3<T> c) {
                cplx<T> tmp[3][3] = {};
                for (int q = 0; q < rule.n; q++) {
                    const V3<T> y = a * (T)rule.p[q][0] + b * (T)rule.p[q][1] + c * (T)rule.p[q][2];
                    const V3<T> rv = y - x;
                    const V3<T> rh = normalized(rv);
                    const T r = norm(rv);
                    for (int p = 0; p < 3; p++)
                        for (int qq = 0; qq <= p; qq++) {
                            const cplx<T> v = r_b_trans(rh, r, n, p, qq, mt) / r * (T)rule.p[q][3];
                            tmp[p][qq] += v;
                            if (p != qq) tmp[qq][p] += v;
                        }
                }
                const T area = norm(cross(b - a, c - a)) / T(2);
                for (int p = 0; p < 3; p++)
                    for (int qq = 0; qq < 3; qq++) mat[p][qq] += tmp[p][qq] * area;
            });
            for (int p = 0; p < 3; p++)
                for (int qq = 0; qq < 3; qq++) Bi[p][qq] += mat[p][qq];
        } else {
            if (!(parts & 2)) continue;
            const V3<double> n = load<double>(m.N, f);
            const long j[3] = {m.f(f, sc), m.f(f, (sc + 1) % 3), m.f(f, (sc + 2) % 3)};
            const V3<double> y1 = load<double>(m.V, j[0]), y2 = load<double>(m.V, j[1]), y3 = load<double>(m.V, j[2]);
            for (int p = 0; p < 3; p++)
                for (int qq = 0; qq <= p; qq++) {
                    cplx<double> e[1];
                    weakly_singular<1>(
                        y1, y2, y3, sorder, ssub,
                        [&](const V3<double> &, const V3<double> &rh, double r, cplx<double> *v) {
                            v[0] = r_b_trans(rh, r, n, p, qq, md);
                        },
                        e);
                    Bi[p][qq] += cplx<T>(e[0]);
                    if (p != qq) Bi[qq][p] += cplx<T>(e[0]);
                }
        }
    }
    for (int p = 0; p < 3; p++)
        for (int qq = 0; qq < 3; qq++) B[3 * p + qq] = cplx<double>(Bi[p][qq]);
}

template <class T>
void coll_Ba_row(const Mesh &m, long i, const Mat<double> &md, int order, int subdiv, int sorder, int ssub,
                 int parts, cplx<double> *B) {
    const Mat<T> mt{(T)md.c1, (T)md.c2, (T)md.rho, cplx<T>(md.s), md.stable && sizeof(T) == sizeof(double)};
    const TriRule rule = tri_rule(order);
    const V3<T> x = load<T>(m.V, i);
    cplx<T> Bi[27] = {};  // [p][q][k] row-major (B_angular_collocation.cu:37-42)
    for (long f = 0; f < m.nF; f++) {
        const int sc = singular_corner(m, i, f);
        if (sc < 0) {
            if (!(parts & 1)) continue;
            const V3<T> n = load<T>(m.N, f);
            const V3<T> y1 = load<T>(m.V, m.f(f, 0)), y2 = load<T>(m.V, m.f(f, 1)), y3 = load<T>(m.V, m.f(f, 2));
            for (int k = 0; k < 3; k++) {  // the reference integrates each k separately (:97-105)
                cplx<T> mat[3][3] = {};
                for_each_subtriangle<T>(y1, y2, y3, subdiv, [&](V3<T> a, V3<T> b, V3<T> c) {
                    cplx<T> tmp[3][3] = {};
                    for (int q = 0; q < rule.n; q++) {
                        const V3<T> y = a * (T)rule.p[q][0] + b * (T)rule.p[q][1] + c * (T)rule.p[q][2];
                        const V3<T> rv = y - x;
                        const V3<T> rh = normalized(rv);
                        const T r = norm(rv);
                        for (int p = 0; p < 3; p++)
                            for (int qq = 0; qq <= p; qq++) {
                                const cplx<T> v = r_b_ang(rh, r, n, p, qq, k, mt) / r * (T)rule.p[q][3];
                                tmp[p][qq] += v;
                                if (p != qq) tmp[qq][p] += v;
                            }
                    }
                    const T area = norm(cross(b - a, c - a)) / T(2);
                    for (int p = 0; p < 3; p++)
                        for (int qq = 0; qq < 3; qq++) mat[p][qq] += tmp[p][qq] * area;
                });
                for (int p = 0; p < 3; p++)
                    for (int qq = 0; qq < 3; qq++) Bi[9 * p + 3 * qq + k] += mat[p][qq];
            }
        } else {
            if (!(parts & 2)) continue;
            const V3<double> n = load<double>(m.N, f);
            const long j[3] = {m.f(f, sc), m.f(f, (sc + 1) % 3), m.f(f, (sc + 2) % 3)};
            const V3<double> y1 = load<double>(m.V, j[0]), y2 = load<double>(m.V, j[1]), y3 = load<double>(m.V, j[2]);
            for (int p = 0; p < 3; p++)
                for (int qq = 0; qq <= p; qq++)
                    for (int k = 0; k < 3; k++) {
                        cplx<double> e[1];
                        weakly_singular<1>(
                            y1, y2, y3, sorder, ssub,
                            [&](const V3<double> &, const V3<double> &rh, double r, cplx<double> *v) {
                                v[0] = r_b_ang(rh, r, n, p, qq, k, md);
                            },
                            e);
                        Bi[9 * p + 3 * qq + k] += cplx<T>(e[0]);
                        if (p != qq) Bi[9 * qq + 3 * p + k] += cplx<T>(e[0]);
                    }
        }
    }
    for (int c = 0; c < 27; c++) B[c] = cplx<double>(Bi[c]);
}

// ---------------------------------------------------------------------------------------------
// Galerkin integration

// product rule over two subdivided reference triangles (include/integrator_galerkin.hpp:214-260);
// fn(xi_x[2], xi_y[2], weight) receives parametric coordinates; the caller multiplies by Jx*Jy.
// The nesting (inner y sum scaled by the y sub-area, then x) follows the reference.
template <class T, int NC, class Fn>
void galerkin_regular(int order, int subdiv, Fn fn, cplx<T> out[NC]) {
    const TriRule rule = tri_rule(order);
    for (int c = 0; c < NC; c++) out[c] = 0;
    const V3<T> p0{0, 0, 0}, p1{1, 0, 0}, p2{0, 1, 0};
    for_each_subtriangle<T>(p0, p1, p2, subdiv, [&](V3<T> xa, V3<T> xb, V3<T> xc) {
        cplx<T> xs[NC] = {};
        for (int qx = 0; qx < rule.n; qx++) {
            const V3<T> xp = xa * (T)rule.p[qx][0] + xb * (T)rule.p[qx][1] + xc * (T)rule.p[qx][2];
            cplx<T> inner[NC] = {};
            for_each_subtriangle<T>(p0, p1, p2, subdiv, [&](V3<T> ya, V3<T> yb, V3<T> yc) {
                cplx<T> ys[NC] = {};
                for (int qy = 0; qy < rule.n; qy++) {
                    const V3<T> yp = ya * (T)rule.p[qy][0] + yb * (T)rule.p[qy][1] + yc * (T)rule.p[qy][2];
                    fn(xp, yp, (T)rule.p[qy][3], ys);
                }
                const T ar = std::abs((yb.x - ya.x) * (yc.y - ya.y) - (yb.y - ya.y) * (yc.x - ya.x)) / T(2);
                for (int c = 0; c < NC; c++) inner[c] += ys[c] * ar;
            });
            for (int c = 0; c < NC; c++) xs[c] += inner[c] * (T)rule.p[qx][3];
        }
        const T ar = std::abs((xb.x - xa.x) * (xc.y - xa.y) - (xb.y - xa.y) * (xc.x - xa.x)) / T(2);
        for (int c = 0; c < NC; c++) out[c] += xs[c] * ar;
    });
}

// 4-D tensor Gauss rule on [0,1]^4 (include/integrator_galerkin.hpp:10-40)
template <class Fn> void hypercube4(int order, int subdiv, Fn fn) {
    const GLRule g = gl_rule(order);
    std::vector<double> pt, wt;
    for (int s = 0; s < subdiv; s++) {
        const double a = double(s) / subdiv, b = double(s + 1) / subdiv;
        for (int q = 0; q < g.n; q++) {
            pt.push_back((b - a) * g.p[q][0] / 2. + (a + b) / 2.);
            wt.push_back(g.p[q][1] * (b - a) / 2.);
        }
    }
    const int n = (int)pt.size();
    for (int a = 0; a < n; a++)
        for (int b = 0; b < n; b++)
            for (int c = 0; c < n; c++)
                for (int d = 0; d < n; d++) fn(pt[a], pt[b], pt[c], pt[d], wt[a] * wt[b] * wt[c] * wt[d]);
}

// Sauter-Schwab maps.  emit(xh0, xh1, yh0, yh1, weight) is called for every 4-D point of every
// sub-domain; the parametrisation x = x0 + (x1-x0) xh0 + (x2-x1) xh1 with barycentrics
// (1-xh0, xh0-xh1, xh1) is applied by the caller.
// coincident: include/integrator_galerkin.hpp:42-103
template <class Emit> void duffy_coincident(int order, int subdiv, Emit emit) {
    hypercube4(order, subdiv, [&](double e1, double e2, double e3, double xi, double w) {
        const double jac = w * xi * xi * xi * e1 * e1 * e2;
        emit(xi, xi * (1. - e1 + e1 * e2), xi * (1. - e1 * e2 * e3), xi * (1. - e1), jac);
        emit(xi * (1. - e1 * e2 * e3), xi * (1. - e1), xi, xi * (1. - e1 + e1 * e2), jac);
        emit(xi, xi * e1 * (1. - e2 + e2 * e3), xi * (1. - e1 * e2), xi * e1 * (1. - e2), jac);
        emit(xi * (1. - e1 * e2), xi * e1 * (1. - e2), xi, xi * e1 * (1. - e2 + e2 * e3), jac);
        emit(xi * (1. - e1 * e2 * e3), xi * e1 * (1. - e2 * e3), xi, xi * e1 * (1. - e2), jac);
        emit(xi, xi * e1 * (1. - e2), xi * (1. - e1 * e2 * e3), xi * e1 * (1. - e2 * e3), jac);
    });
}
// edge adjacent: include/integrator_galerkin.hpp:106-163
template <class Emit> void duffy_edge(int order, int subdiv, Emit emit) {
    hypercube4(order, subdiv, [&](double e1, double e2, double e3, double xi, double w) {
        const double jac = w * xi * xi * xi * e1 * e1;
        emit(xi, xi * e1 * e3, xi * (1. - e1 * e2), xi * e1 * (1. - e2), jac);
        emit(xi, xi * e1, xi * (1. - e1 * e2 * e3), xi * e1 * e2 * (1. - e3), jac * e2);
        emit(xi * (1. - e1 * e2), xi * e1 * (1. - e2), xi, xi * e1 * e2 * e3, jac * e2);
        emit(xi * (1. - e1 * e2 * e3), xi * e1 * e2 * (1. - e3), xi, xi * e1, jac * e2);
        emit(xi * (1. - e1 * e2 * e3), xi * e1 * (1. - e2 * e3), xi, xi * e1 * e2, jac * e2);
    });
}
// vertex adjacent: include/integrator_galerkin.hpp:166-212
template <class Emit> void duffy_vertex(int order, int subdiv, Emit emit) {
    hypercube4(order, subdiv, [&](double e1, double e2, double e3, double xi, double w) {
        const double jac = w * xi * xi * xi * e2;
        emit(xi, xi * e1, xi * e2, xi * e2 * e3, jac);
        emit(xi * e2, xi * e2 * e3, xi, xi * e1, jac);
    });
}

// Classification of a face pair (include/integrator_galerkin.hpp:262-334).  Returns 0 for
// regular, 1 coincident, 2 edge, 3 vertex; fills the permuted vertex lists j1, j2.
int classify_pair(const Mesh &m, long f1, long f2, long j1[3], long j2[3]) {
    if (f1 == f2) {
        for (int k = 0; k < 3; k++) j1[k] = j2[k] = m.f(f1, k);
        return 1;
    }
    bool edge = false;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const bool hit = (m.f(f1, i) == m.f(f2, j) && m.f(f1, (i + 1) % 3) == m.f(f2, (j + 2) % 3)) ||
                             (m.vmap && m.vmap[m.f(f1, i)] == m.vmap[m.f(f2, j)] &&
                              m.vmap[m.f(f1, (i + 1) % 3)] == m.vmap[m.f(f2, (j + 2) % 3)]);
            if (hit) {
                edge = true;
                j1[0] = m.f(f1, i), j1[1] = m.f(f1, (i + 1) % 3), j1[2] = m.f(f1, (i + 2) % 3);
                j2[0] = m.f(f2, j), j2[1] = m.f(f2, (j + 2) % 3), j2[2] = m.f(f2, (j + 1) % 3);
                break;
            }
        }
    if (edge) return 2;
    bool vert = false;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            if (m.f(f1, i) == m.f(f2, j) || (m.vmap && m.vmap[m.f(f1, i)] == m.vmap[m.f(f2, j)])) {
                vert = true;
                j1[0] = m.f(f1, i), j1[1] = m.f(f1, (i + 1) % 3), j1[2] = m.f(f1, (i + 2) % 3);
                j2[0] = m.f(f2, j), j2[1] = m.f(f2, (j + 1) % 3), j2[2] = m.f(f2, (j + 2) % 3);
                break;
            }
        }
    if (vert) return 3;
    return 0;
}

// Kernel evaluation shared by the Galerkin drivers.  Writes NCOL complex values per (x-corner a, row p):
// out[(3a+p)*NCOL + c].  kind 0: G (NCOL=9: y-corner b, col q), 1: H (9), 2: B_trans (3), 3: B_angular (9: 3k+q)
template <class T> struct GalerkinEval {
    int kind;
    Mat<T> m;
    V3<T> n;  // source face normal
    // x: field point, y: source point, Lx/Ly shape values, w weight; acc has 9*NCOL entries
    void operator()(const V3<T> &x, const V3<T> &y, const T Lx[3], const T Ly[3], T w, cplx<T> *acc) const {
        const V3<T> rv = y - x;
        const V3<T> rh = normalized(rv);
        const T r = norm(rv);
        if (kind == 0) {
            cplx<T> u[3][3];
            for (int p = 0; p < 3; p++)
                for (int q = 0; q <= p; q++) {
                    u[p][q] = r_u_hat(rh, r, p, q, m) / r;
                    u[q][p] = u[p][q];
                }
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    const T lw = Lx[a] * Ly[b] * w;
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) acc[(3 * a + p) * 9 + 3 * b + q] += u[p][q] * lw;
                }
        } else if (kind == 1) {
            cplx<T> pp[3][3];
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) pp[p][q] = p_hat(rh, r, n, p, q, m);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    const T lw = Lx[a] * Ly[b] * w;
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) acc[(3 * a + p) * 9 + 3 * b + q] += pp[p][q] * lw;
                }
        } else if (kind == 2) {
            cplx<T> bb[3][3];
            for (int p = 0; p < 3; p++)
                for (int q = 0; q <= p; q++) {
                    bb[p][q] = r_b_trans(rh, r, n, p, q, m) / r;
                    bb[q][p] = bb[p][q];
                }
            for (int a = 0; a < 3; a++) {
                const T lw = Lx[a] * w;
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) acc[(3 * a + p) * 3 + q] += bb[p][q] * lw;
            }
        } else {
            cplx<T> bb[3][9];
            for (int k = 0; k < 3; k++)
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q <= p; q++) {
                        bb[p][3 * k + q] = r_b_ang(rh, r, n, p, q, k, m) / r;
                        bb[q][3 * k + p] = bb[p][3 * k + q];
                    }
            for (int a = 0; a < 3; a++) {
                const T lw = Lx[a] * w;
                for (int p = 0; p < 3; p++)
                    for (int c = 0; c < 9; c++) acc[(3 * a + p) * 9 + c] += bb[p][c] * lw;
            }
        }
    }
};

inline int galerkin_ncol(int kind) { return kind == 2 ? 3 : 9; }

// non-singular face pair, kernel precision T (src/elastodynamics_cqbem_*_galerkin_non_singular.cu)
template <class T>
void galerkin_pair_regular(const Mesh &m, int kind, long f1, long f2, const Mat<double> &md, int order, int subdiv,
                           cplx<double> *blk /* 9 x NCOL */) {
    const int NC = 9 * galerkin_ncol(kind);
    GalerkinEval<T> ev{kind, {(T)md.c1, (T)md.c2, (T)md.rho, cplx<T>(md.s), md.stable && sizeof(T) == sizeof(double)},
                       load<T>(m.N, f2)};
    const V3<T> x0 = load<T>(m.V, m.f(f1, 0)), x1 = load<T>(m.V, m.f(f1, 1)), x2 = load<T>(m.V, m.f(f1, 2));
    const V3<T> y0 = load<T>(m.V, m.f(f2, 0)), y1 = load<T>(m.V, m.f(f2, 1)), y2 = load<T>(m.V, m.f(f2, 2));
    const V3<T> ax = x1 - x0, bx = x2 - x0, ay = y1 - y0, by = y2 - y0;
    cplx<T> acc[81];
    galerkin_regular<T, 81>(
        order, subdiv,
        [&](const V3<T> &xp, const V3<T> &yp, T w, cplx<T> *out) {
            const V3<T> x = x0 + xp.x * ax + xp.y * bx;
            const V3<T> y = y0 + yp.x * ay + yp.y * by;
            const T Lx[3] = {T(1) - xp.x - xp.y, xp.x, xp.y}, Ly[3] = {T(1) - yp.x - yp.y, yp.x, yp.y};
            ev(x, y, Lx, Ly, w, out);
        },
        acc);
    const T J = norm(cross(ax, bx)) * norm(cross(ay, by));
    for (int c = 0; c < NC; c++) blk[c] = cplx<double>(acc[c] * J);
}

// singular face pair in FP64 (src/elastodynamics_cqbem_galerkin_singular.cpp, integrator_galerkin.hpp:42-212)
void galerkin_pair_singular(const Mesh &m, int kind, int cls, const long j1[3], const long j2[3], long f2,
                            const Mat<double> &md, int sorder, int ssub, cplx<double> *blk) {
    const int NC = 9 * galerkin_ncol(kind);
    GalerkinEval<double> ev{kind, md, load<double>(m.N, f2)};
    for (int c = 0; c < NC; c++) blk[c] = 0.0;
    V3<double> xo, xa, xb, yo, ya, yb;  // x = xo + xa*xh0 + xb*xh1
    double J;
    if (cls == 1) {
        const V3<double> p0 = load<double>(m.V, j1[0]), p1 = load<double>(m.V, j1[1]), p2 = load<double>(m.V, j1[2]);
        xo = yo = p0, xa = ya = p1 - p0, xb = yb = p2 - p1;
        J = norm(cross(xa, xb));
        J = J * J;
    } else if (cls == 2) {
        const V3<double> s0 = load<double>(m.V, j1[0]), s1 = load<double>(m.V, j1[1]);
        const V3<double> x2 = load<double>(m.V, j1[2]), y2 = load<double>(m.V, j2[2]);
        xo = yo = s0, xa = ya = s1 - s0, xb = x2 - s1, yb = y2 - s1;
        J = norm(cross(xa, xb)) * norm(cross(ya, yb));
    } else {
        const V3<double> s0 = load<double>(m.V, j1[0]);
        const V3<double> x1 = load<double>(m.V, j1[1]), x2 = load<double>(m.V, j1[2]);
        const V3<double> y1 = load<double>(m.V, j2[1]), y2 = load<double>(m.V, j2[2]);
        xo = yo = s0, xa = x1 - s0, xb = x2 - x1, ya = y1 - s0, yb = y2 - y1;
        J = norm(cross(xa, xb)) * norm(cross(ya, yb));
    }
    auto emit = [&](double xh0, double xh1, double yh0, double yh1, double w) {
        const V3<double> x = xo + xa * xh0 + xb * xh1, y = yo + ya * yh0 + yb * yh1;
        const double Lx[3] = {1. - xh0, xh0 - xh1, xh1}, Ly[3] = {1. - yh0, yh0 - yh1, yh1};
        ev(x, y, Lx, Ly, w, blk);
    };
    if (cls == 1)
        duffy_coincident(sorder, ssub, emit);
    else if (cls == 2)
        duffy_edge(sorder, ssub, emit);
    else
        duffy_vertex(sorder, ssub, emit);
    for (int c = 0; c < NC; c++) blk[c] *= J;
}

// ---------------------------------------------------------------------------------------------
// Elastostatic Kelvin kernels (src/elastics_bem_matrix_collection.cpp:48-64, 144-169)
struct Static {
    double nu, mu;
    double r_u(const V3<double> &rh, double, int i, int j) const {
        return (1. / (16. * PI * (1. - nu) * mu)) * (kd<double>(i, j) * (3. - 4. * nu) + rh[i] * rh[j]);
    }
    double p(const V3<double> &rh, double r, const V3<double> &n, int i, int j) const {
        return ((1. - 2. * nu) / (8. * PI * (1. - nu))) *
               ((rh[i] * n[j] - rh[j] * n[i]) - (kd<double>(i, j) + (1. / (1. - 2 * nu)) * (3. * rh[i] * rh[j])) * dot(rh, n)) /
               (r * r);
    }
    double p_sing(const V3<double> &rh, double r, const V3<double> &n, int i, int j) const {
        return ((1. - 2. * nu) / (8. * PI * (1. - nu))) * (rh[i] * n[j] - rh[j] * n[i]) / (r * r);
    }
};

}  // namespace

// =============================================================================================
// C ABI for ctypes
extern "C" {

int oracle_version() { return 1; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// Triangle rule table for checks: writes n rows of {l0,l1,l2,w}; returns n (0 for unsupported order).
int oracle_tri_rule(int order, double *out) {
    TriRule r = tri_rule(order);
    for (int q = 0; q < r.n; q++)
        for (int c = 0; c < 4; c++) out[4 * q + c] = r.p[q][c];
    return r.n;
}

// CQ frequencies s_l = gamma(R zeta^l)/dt, l = 0..L/2 (src/elastodynamics_cqbem_G.cu:19-24, 65)
// bdf: 1 or 2.  Writes Lambda complex values; returns Lambda.  R and L are written to R_out, L_out.
int oracle_cq_frequencies(int bdf, double dt, int N, double *s_out, double *R_out, int *L_out) {
    const double R = std::pow(1e-10, 1. / (2. * N));
    const int L = N + 1;
    const std::complex<double> z = std::exp(std::complex<double>(0.0, 1.0) * (2. * PI) / (double)L);
    const int lam = L / 2 + 1;
    for (int l = 0; l < lam; l++) {
        const std::complex<double> w = R * std::pow(z, l);
        const std::complex<double> g = bdf == 1 ? 1. - w : 1.5 - 2. * w + w * w / 2.;
        const std::complex<double> s = g / dt;
        s_out[2 * l] = s.real();
        s_out[2 * l + 1] = s.imag();
    }
    *R_out = R;
    *L_out = L;
    return lam;
}

// Collocation assembly of the rows of the listed field vertices for one Laplace frequency s.
// kind: 0=G 1=H 2=B_trans 3=B_angular;  mode: 0 FP64, 1 reference-mixed, 2 FP32 regular, 3 FP64 literal;
// parts: 1 regular, 2 singular, 3 both.
// out: complex128 interleaved, (3*nrows) x ncols (ncols = 3V, 3V, 3, 9).  rows=NULL -> all vertices.
int oracle_collocation(int kind, int mode, const double *V, int nV, const int *F, int nF, const double *N,
                       const int *vmap, double c1, double c2, double rho, double s_re, double s_im, int order,
                       int subdiv, int sorder, int ssub, const int *rows, int nrows, int parts, double *out) {
    if (!tri_rule(order).n || !gl_rule(sorder).n || subdiv < 1 || ssub < 1) return 1;
    Mesh m{V, nV, F, nF, N, vmap};
    Mat<double> md{c1, c2, rho, {s_re, s_im}, mode == 0};
    const long ncol = (kind <= 1) ? 3L * nV : (kind == 2 ? 3 : 9);
    const int nr = rows ? nrows : nV;
    cplx<double> *O = reinterpret_cast<cplx<double> *>(out);
    std::memset(out, 0, sizeof(double) * 2 * 3 * (size_t)nr * ncol);
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < nr; r++) {
        const long i = rows ? rows[r] : r;
        cplx<double> *row = O + 3L * r * ncol;
        const bool mixed = mode == 1 || mode == 2;
        switch (kind) {
        case 0:
            if (mixed) coll_G_row<float>(m, i, md, order, subdiv, sorder, ssub, parts, row, ncol);
            else coll_G_row<double>(m, i, md, order, subdiv, sorder, ssub, parts, row, ncol);
            break;
        case 1:  // the reference keeps regular H in FP64 in both builds (H_collocation.cu:15)
            if (mode == 2) coll_H_row<float>(m, i, md, order, subdiv, sorder, ssub, parts, row, ncol);
            else coll_H_row<double>(m, i, md, order, subdiv, sorder, ssub, parts, row, ncol);
            break;
        case 2:
            if (mixed) coll_Bt_row<float>(m, i, md, order, subdiv, sorder, ssub, parts, row);
            else coll_Bt_row<double>(m, i, md, order, subdiv, sorder, ssub, parts, row);
            break;
        case 3:
            if (mixed) coll_Ba_row<float>(m, i, md, order, subdiv, sorder, ssub, parts, row);
            else coll_Ba_row<double>(m, i, md, order, subdiv, sorder, ssub, parts, row);
            break;
        }
    }
    return 0;
}

// Galerkin assembly of the rows of the listed vertices (all rows if rows == NULL) for one frequency.
// Sums every face pair (f1, f2) with f1 in the star of a listed vertex; only rows of listed
// vertices are scattered, so those rows are exact.  parts: 1 non-singular pairs, 2 singular pairs.
int oracle_galerkin(int kind, int mode, const double *V, int nV, const int *F, int nF, const double *N,
                    const int *vmap, double c1, double c2, double rho, double s_re, double s_im, int order,
                    int subdiv, int sorder, int ssub, const int *rows, int nrows, int parts, double *out) {
    if (!tri_rule(order).n || !gl_rule(sorder).n || subdiv < 1 || ssub < 1) return 1;
    Mesh m{V, nV, F, nF, N, vmap};
    Mat<double> md{c1, c2, rho, {s_re, s_im}, mode == 0};
    const long ncol = (kind <= 1) ? 3L * nV : (kind == 2 ? 3 : 9);
    const int nr = rows ? nrows : nV;
    std::vector<int> slot(nV, -1);
    for (int r = 0; r < nr; r++) slot[rows ? rows[r] : r] = r;
    std::vector<char> use(nF, 0);
    for (long f = 0; f < nF; f++)
        for (int k = 0; k < 3; k++)
            if (slot[F[3 * f + k]] >= 0) use[f] = 1;
    cplx<double> *O = reinterpret_cast<cplx<double> *>(out);
    std::memset(out, 0, sizeof(double) * 2 * 3 * (size_t)nr * ncol);
    const int NCOL = galerkin_ncol(kind);
#pragma omp parallel for schedule(dynamic, 1)
    for (long f1 = 0; f1 < nF; f1++) {
        if (!use[f1]) continue;
        cplx<double> blk[81];
        for (long f2 = 0; f2 < nF; f2++) {
            long j1[3], j2[3];
            const int cls = classify_pair(m, f1, f2, j1, j2);
            if (cls == 0) {
                if (!(parts & 1)) continue;
                for (int k = 0; k < 3; k++) j1[k] = m.f(f1, k), j2[k] = m.f(f2, k);
                if (mode == 1) galerkin_pair_regular<float>(m, kind, f1, f2, md, order, subdiv, blk);
                else galerkin_pair_regular<double>(m, kind, f1, f2, md, order, subdiv, blk);
            } else {
                if (!(parts & 2)) continue;
                galerkin_pair_singular(m, kind, cls, j1, j2, f2, md, sorder, ssub, blk);
            }
#pragma omp critical
            for (int a = 0; a < 3; a++) {
                const int r = slot[j1[a]];
                if (r < 0) continue;
                for (int p = 0; p < 3; p++) {
                    cplx<double> *row = O + (3L * r + p) * ncol;
                    if (kind <= 1) {
                        for (int b = 0; b < 3; b++)
                            for (int q = 0; q < 3; q++) row[3 * j2[b] + q] += blk[(3 * a + p) * NCOL + 3 * b + q];
                    } else {
                        for (int c = 0; c < NCOL; c++) row[c] += blk[(3 * a + p) * NCOL + c];
                    }
                }
            }
        }
    }
    // B_angular output layout [row][j][k]; the Galerkin kernels produce (3a+p, 3k+q) -> [p][q][k]
    if (kind == 3) {
        for (long r = 0; r < 3L * nr; r++) {
            cplx<double> tmp[9];
            for (int c = 0; c < 9; c++) tmp[c] = O[r * 9 + c];
            for (int k = 0; k < 3; k++)
                for (int q = 0; q < 3; q++) O[r * 9 + 3 * q + k] = tmp[3 * k + q];
        }
    }
    return 0;
}

// Inverse transform X_n = R^-n / L * sum_l Re(c_l Xhat_l zeta^-nl), n = 0..L-1
// (src/elastodynamics_cqbem_G.cu:166-179).  Xhat: nfreq x M complex, out: L x M real.
int oracle_inverse_transform(int nfreq, int L, double R, const double *Xhat, long M, double *out) {
    if (nfreq != L / 2 + 1) return 1;
    const std::complex<double> z = std::exp(std::complex<double>(0.0, 1.0) * (2. * PI) / (double)L);
    const std::complex<double> *X = reinterpret_cast<const std::complex<double> *>(Xhat);
    for (int n = 0; n < L; n++) {
        std::vector<std::complex<double>> w1(nfreq), w2(nfreq);
        std::vector<char> two(nfreq);
        for (int l = 0; l < nfreq; l++) {
            w1[l] = std::pow(z, -(double)n * l);
            two[l] = (l != 0 && (l != L / 2 || L % 2 == 1));
            w2[l] = std::pow(z, -(double)n * (L - l));
        }
        const double sc = std::pow(R, -(double)n) / (double)L;
#pragma omp parallel for
        for (long e = 0; e < M; e++) {
            double acc = 0.0;
            for (int l = 0; l < nfreq; l++) {
                const std::complex<double> x = X[(size_t)l * M + e];
                acc += (x * w1[l]).real();
                if (two[l]) acc += (std::conj(x) * w2[l]).real();
            }
            out[(size_t)n * M + e] = acc * sc;
        }
    }
    return 0;
}

// Collocation free-term (jump) blocks C, 3V x 3 (src/elastics_bem_matrix_collection.cpp:387-445).
// With traction-discontinuity splitting (vmap = vertex_map_inverse, may be NULL) the reference computes
// C on the original mesh, i.e. with every face corner mapped to its canonical vertex, and copies the
// canonical vertex's block to each split vertex (:395-400, :434-441).
int oracle_c_matrix_collocation(const double *V, int nV, const int *F_in, int nF, const double *N, double nu,
                                const int *vmap, double *out) {
    std::vector<int> Fc(F_in, F_in + 3 * (size_t)nF);
    if (vmap)
        for (auto &v : Fc) v = vmap[v];
    const int *F = Fc.data();
    std::memset(out, 0, sizeof(double) * 9 * nV);
    for (int i = 0; i < nV; i++)
        for (int d = 0; d < 3; d++) out[9 * i + 4 * d] += 0.5;
    // unique undirected edges: directed edge k of face f joins F(f,(k+1)%3) -> F(f,(k+2)%3)
    struct E {
        long a, b;
        long de;
    };
    std::vector<E> es;
    for (long f = 0; f < nF; f++)
        for (int k = 0; k < 3; k++) {
            long a = F[3 * f + (k + 1) % 3], b = F[3 * f + (k + 2) % 3];
            es.push_back({std::min(a, b), std::max(a, b), f + k * (long)nF});
        }
    std::sort(es.begin(), es.end(), [](const E &x, const E &y) {
        return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : x.de < y.de);
    });
    for (size_t s = 0; s + 1 < es.size(); s++) {
        if (es[s].a != es[s + 1].a || es[s].b != es[s + 1].b) continue;
        const long e1 = es[s].de, e2 = es[s + 1].de;
        const long f1 = e1 % nF, f2 = e2 % nF, k1 = e1 / nF;
        const long a = F[3 * f1 + (k1 + 1) % 3], b = F[3 * f1 + (k1 + 2) % 3];
        const V3<double> n1 = load<double>(N, f1), n2 = load<double>(N, f2);
        const V3<double> r = normalized(load<double>(V, a) - load<double>(V, b));
        const double sx = dot(cross(n1, n2), r);
        const double sg = std::abs(sx) < 1e-12 ? 0.0 : (sx > 0 ? 1.0 : -1.0);
        const double w = (1. / (4. * PI)) * sg * std::atan2(norm(cross(n1, n2)), dot(n1, n2));  // dihedral angle
        for (int d = 0; d < 3; d++) {
            out[9 * a + 4 * d] += w;
            out[9 * b + 4 * d] += w;
        }
        s++;
    }
    for (long f = 0; f < nF; f++) {
        const V3<double> n = load<double>(N, f);
        for (int i = 0; i < 3; i++) {
            const long vi = F[3 * f + i];
            const V3<double> r1 = normalized(load<double>(V, F[3 * f + (i + 1) % 3]) - load<double>(V, vi));
            const V3<double> r2 = normalized(load<double>(V, F[3 * f + (i + 2) % 3]) - load<double>(V, vi));
            const V3<double> c = cross(r2 - r1, n);
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) out[9 * vi + 3 * p + q] -= (1. / (8. * PI * (1. - nu))) * c[p] * n[q];
        }
    }
    if (vmap)
        for (int v = 0; v < nV; v++)
            if (vmap[v] != v)
                for (int t = 0; t < 9; t++) out[9 * v + t] = out[9 * vmap[v] + t];
    return 0;
}

// Galerkin mass-matrix C, dense 3V x 3V (src/elastics_bem_matrix_collection.cpp:447-467)
int oracle_c_matrix_galerkin(const double *V, int nV, const int *F, int nF, double *out) {
    const long n3 = 3L * nV;
    std::memset(out, 0, sizeof(double) * n3 * n3);
    for (long f = 0; f < nF; f++) {
        const V3<double> a = load<double>(V, F[3 * f]), b = load<double>(V, F[3 * f + 1]), c = load<double>(V, F[3 * f + 2]);
        const double A = norm(cross(b - a, c - a));
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int d = 0; d < 3; d++)
                    out[(3L * F[3 * f + i] + d) * n3 + 3L * F[3 * f + j] + d] += (i == j ? A / 24. : A / 48.);
    }
    return 0;
}

// Elastostatic G (kind 0) / H (kind 1), collocation (galerkin=0) or Galerkin (galerkin=1), FP64,
// including the rigid-mode diagonal correction of H (src/elastics_bem_matrix_collection.cpp:43-385).
// out: dense 3V x 3V row-major.
int oracle_elastostatic(int kind, int galerkin, const double *V, int nV, const int *F, int nF, const double *N,
                        double nu, double mu, int order, int subdiv, int sorder, int ssub, double *out) {
    if (!tri_rule(order).n || !gl_rule(sorder).n) return 1;
    Mesh m{V, nV, F, nF, N, nullptr};
    Static st{nu, mu};
    const long n3 = 3L * nV;
    std::memset(out, 0, sizeof(double) * n3 * n3);
    const TriRule rule = tri_rule(order);
    if (!galerkin) {
#pragma omp parallel for schedule(dynamic, 1)
        for (long i = 0; i < nV; i++) {
            const V3<double> x = load<double>(V, i);
            double *row = out + 3 * i * n3;
            for (long f = 0; f < nF; f++) {
                const int sc = singular_corner(m, i, f);
                const V3<double> n = load<double>(N, f);
                if (sc < 0) {
                    const long j[3] = {m.f(f, 0), m.f(f, 1), m.f(f, 2)};
                    const V3<double> y1 = load<double>(V, j[0]), y2 = load<double>(V, j[1]), y3 = load<double>(V, j[2]);
                    double mat[9][3] = {};
                    for_each_subtriangle<double>(y1, y2, y3, subdiv, [&](V3<double> a, V3<double> b, V3<double> c) {
                        double tmp[9][3] = {};
                        for (int q = 0; q < rule.n; q++) {
                            const V3<double> y = a * rule.p[q][0] + b * rule.p[q][1] + c * rule.p[q][2];
                            double L[3];
                            bary_clamped(y, y1, y2, y3, L);
                            const V3<double> rv = y - x;
                            const V3<double> rh = normalized(rv);
                            const double r = norm(rv);
                            for (int p = 0; p < 3; p++)
                                for (int qq = 0; qq < 3; qq++) {
                                    const double v = kind == 0 ? st.r_u(rh, r, p, qq) / r : st.p(rh, r, n, p, qq);
                                    for (int k = 0; k < 3; k++) tmp[3 * k + p][qq] += v * L[k] * rule.p[q][3];
                                }
                        }
                        const double area = norm(cross(b - a, c - a)) / 2.;
                        for (int r = 0; r < 9; r++)
                            for (int cc = 0; cc < 3; cc++) mat[r][cc] += tmp[r][cc] * area;
                    });
                    for (int k = 0; k < 3; k++)
                        for (int p = 0; p < 3; p++)
                            for (int qq = 0; qq < 3; qq++) row[p * n3 + 3 * j[k] + qq] += mat[3 * k + p][qq];
                } else {
                    const long j[3] = {m.f(f, sc), m.f(f, (sc + 1) % 3), m.f(f, (sc + 2) % 3)};
                    const V3<double> y1 = load<double>(V, j[0]), y2 = load<double>(V, j[1]), y3 = load<double>(V, j[2]);
                    for (int p = 0; p < 3; p++)
                        for (int qq = 0; qq < 3; qq++) {
                            if (kind == 0 && qq > p) continue;
                            cplx<double> e[3];
                            if (kind == 0) {
                                weakly_singular<3>(
                                    y1, y2, y3, sorder, ssub,
                                    [&](const V3<double> &y, const V3<double> &rh, double r, cplx<double> *v) {
                                        double L[3];
                                        bary_clamped(y, y1, y2, y3, L);
                                        for (int c = 0; c < 3; c++) v[c] = st.r_u(rh, r, p, qq) * L[c];
                                    },
                                    e);
                            } else {
                                strongly_singular(
                                    y1, y2, y3, sorder, ssub,
                                    [&](const V3<double> &rh, double r) { return cplx<double>(st.p(rh, r, n, p, qq)); },
                                    [&](const V3<double> &rh, double r) { return cplx<double>(st.p_sing(rh, r, n, p, qq)); },
                                    e);
                            }
                            for (int c = 0; c < 3; c++) {
                                row[p * n3 + 3 * j[c] + qq] += e[c].real();
                                if (kind == 0 && p != qq) row[qq * n3 + 3 * j[c] + p] += e[c].real();
                            }
                        }
                }
            }
        }
    } else {
        // Galerkin: every pair through the singular classifier, else the regular product rule, FP64
#pragma omp parallel for schedule(dynamic, 1)
        for (long f1 = 0; f1 < nF; f1++) {
            for (long f2 = 0; f2 < nF; f2++) {
                long j1[3], j2[3];
                const int cls = classify_pair(m, f1, f2, j1, j2);
                double blk[81] = {};
                const V3<double> n = load<double>(N, f2);
                auto ev = [&](const V3<double> &x, const V3<double> &y, const double Lx[3], const double Ly[3], double w,
                              double *acc) {
                    const V3<double> rv = y - x;
                    const V3<double> rh = normalized(rv);
                    const double r = norm(rv);
                    for (int p = 0; p < 3; p++)
                        for (int q = 0; q < 3; q++) {
                            const double v = kind == 0 ? st.r_u(rh, r, p, q) / r : st.p(rh, r, n, p, q);
                            for (int a = 0; a < 3; a++)
                                for (int b = 0; b < 3; b++) acc[(3 * a + p) * 9 + 3 * b + q] += v * Lx[a] * Ly[b] * w;
                        }
                };
                if (cls == 0) {
                    for (int k = 0; k < 3; k++) j1[k] = m.f(f1, k), j2[k] = m.f(f2, k);
                    const V3<double> x0 = load<double>(V, j1[0]), x1 = load<double>(V, j1[1]), x2 = load<double>(V, j1[2]);
                    const V3<double> y0 = load<double>(V, j2[0]), y1 = load<double>(V, j2[1]), y2 = load<double>(V, j2[2]);
                    const V3<double> ax = x1 - x0, bx = x2 - x0, ay = y1 - y0, by = y2 - y0;
                    cplx<double> acc[81];
                    galerkin_regular<double, 81>(
                        order, subdiv,
                        [&](const V3<double> &xp, const V3<double> &yp, double w, cplx<double> *o) {
                            const V3<double> x = x0 + xp.x * ax + xp.y * bx, y = y0 + yp.x * ay + yp.y * by;
                            const double Lx[3] = {1. - xp.x - xp.y, xp.x, xp.y}, Ly[3] = {1. - yp.x - yp.y, yp.x, yp.y};
                            double tmp[81] = {};
                            ev(x, y, Lx, Ly, w, tmp);
                            for (int c = 0; c < 81; c++) o[c] += tmp[c];
                        },
                        acc);
                    const double J = norm(cross(ax, bx)) * norm(cross(ay, by));
                    for (int c = 0; c < 81; c++) blk[c] = acc[c].real() * J;
                } else {
                    V3<double> xo, xa, xb, yo, ya, yb;
                    double J;
                    if (cls == 1) {
                        const V3<double> p0 = load<double>(V, j1[0]), p1 = load<double>(V, j1[1]), p2 = load<double>(V, j1[2]);
                        xo = yo = p0, xa = ya = p1 - p0, xb = yb = p2 - p1;
                        J = norm(cross(xa, xb));
                        J *= J;
                    } else if (cls == 2) {
                        const V3<double> s0 = load<double>(V, j1[0]), s1 = load<double>(V, j1[1]);
                        xo = yo = s0, xa = ya = s1 - s0, xb = load<double>(V, j1[2]) - s1, yb = load<double>(V, j2[2]) - s1;
                        J = norm(cross(xa, xb)) * norm(cross(ya, yb));
                    } else {
                        const V3<double> s0 = load<double>(V, j1[0]);
                        xo = yo = s0, xa = load<double>(V, j1[1]) - s0, xb = load<double>(V, j1[2]) - load<double>(V, j1[1]);
                        ya = load<double>(V, j2[1]) - s0, yb = load<double>(V, j2[2]) - load<double>(V, j2[1]);
                        J = norm(cross(xa, xb)) * norm(cross(ya, yb));
                    }
                    auto emit = [&](double xh0, double xh1, double yh0, double yh1, double w) {
                        const V3<double> x = xo + xa * xh0 + xb * xh1, y = yo + ya * yh0 + yb * yh1;
                        const double Lx[3] = {1. - xh0, xh0 - xh1, xh1}, Ly[3] = {1. - yh0, yh0 - yh1, yh1};
                        ev(x, y, Lx, Ly, w, blk);
                    };
                    if (cls == 1) duffy_coincident(sorder, ssub, emit);
                    else if (cls == 2) duffy_edge(sorder, ssub, emit);
                    else duffy_vertex(sorder, ssub, emit);
                    for (int c = 0; c < 81; c++) blk[c] *= J;
                }
#pragma omp critical
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++)
                        for (int p = 0; p < 3; p++)
                            for (int q = 0; q < 3; q++)
                                out[(3 * j1[a] + p) * n3 + 3 * j2[b] + q] += blk[(3 * a + p) * 9 + 3 * b + q];
            }
        }
        if (kind == 1) {  // H += C (Galerkin mass matrix), :372-373
            for (long f = 0; f < nF; f++) {
                const V3<double> a = load<double>(V, F[3 * f]), b = load<double>(V, F[3 * f + 1]), c = load<double>(V, F[3 * f + 2]);
                const double A = norm(cross(b - a, c - a));
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int d = 0; d < 3; d++)
                            out[(3L * F[3 * f + i] + d) * n3 + 3L * F[3 * f + j] + d] += (i == j ? A / 24. : A / 48.);
            }
        }
    }
    if (kind == 1) {  // rigid-mode diagonal correction H_ii = -sum_{j!=i} H_ij (:236-243, :375-382)
#pragma omp parallel for
        for (long i = 0; i < nV; i++) {
            double d[3][3] = {};
            for (long j = 0; j < nV; j++) {
                if (j == i) continue;
                for (int p = 0; p < 3; p++)
                    for (int q = 0; q < 3; q++) d[p][q] -= out[(3 * i + p) * n3 + 3 * j + q];
            }
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) out[(3 * i + p) * n3 + 3 * i + q] = d[p][q];
        }
    }
    return 0;
}

// Rigid-mode matrix T (6 x 3V) of src/elastostatics_bem_matrix_collection.cpp:59-78
int oracle_rigid_modes(const double *V, int nV, const int *F, int nF, double *T) {
    const long n3 = 3L * nV;
    std::memset(T, 0, sizeof(double) * 6 * n3);
    for (long e = 0; e < nF; e++) {
        const V3<double> a = load<double>(V, F[3 * e]), b = load<double>(V, F[3 * e + 1]), c = load<double>(V, F[3 * e + 2]);
        const double A = norm(cross(b - a, c - a));
        for (int i = 0; i < 3; i++) {
            const long v = F[3 * e + i];
            for (int d = 0; d < 3; d++) T[d * n3 + 3 * v + d] += A / 6.;
            const V3<double> s = a + b + c + load<double>(V, v);
            const double M[3][3] = {{0.0, -s.z, s.y}, {s.z, 0.0, -s.x}, {-s.y, s.x, 0.0}};
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) T[(3 + p) * n3 + 3 * v + q] += A / 6. * 0.25 * M[p][q];
        }
    }
    return 0;
}

}  // extern "C"
