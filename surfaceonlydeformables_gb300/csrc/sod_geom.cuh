// sod_geom.cuh -- FP64 triangle geometry of the singular quadrature rules (device helpers).
#pragma once
#include <cuda_runtime.h>

namespace sod {

__device__ __forceinline__ double3 ld3(const double *p, int i) { return make_double3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ double3 operator-(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 operator+(double3 a, double3 b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 operator*(double3 a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double norm3(double3 a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ double3 nrmz(double3 a) {
    const double n = norm3(a);
    return n > 0.0 ? a * (1.0 / n) : a;
}

// barycentrics of P in (A,B,C), clamped (include/barycentric_coordinates.cuh:14-38)
__device__ __forceinline__ void bary_clamped(double3 P, double3 A, double3 B, double3 C, double L[3]) {
    const double3 v0 = B - A, v1 = C - A, v2 = P - A;
    const double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1), d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    const double den = d00 * d11 - d01 * d01;
    L[1] = (d11 * d20 - d01 * d21) / den;
    L[2] = (d00 * d21 - d01 * d20) / den;
    L[0] = 1.0 - (L[1] + L[2]);
    for (int c = 0; c < 3; c++) L[c] = fmin(1.0, fmax(0.0, L[c]));
}

// Polar-rule geometry about the singular vertex (include/integrator_collocation.hpp:28-36)
struct Polar {
    double3 y1, y2, y3, xh, yh;
    double a, alpha, beta;
};
__device__ __forceinline__ Polar polar_setup(double3 y1, double3 y2, double3 y3) {
    Polar g;
    g.y1 = y1, g.y2 = y2, g.y3 = y3;
    const double3 v1 = y2 - y1, v2 = y3 - y1;
    const double3 v1n = nrmz(v1), v2n = nrmz(v2);
    g.xh = v1n;
    g.yh = nrmz(cross3(cross3(g.xh, v2n), g.xh));
    const double3 v12 = v1 + nrmz(v2 - v1) * dot3(v1, nrmz(v1 - v2));
    g.a = norm3(v12);
    // The angles of include/integrator_collocation.hpp:35-36 are acos of dot products, which loses
    // half the digits when the angle is near 0 or pi: beta is exactly 0 when the triangle has its
    // right angle at y2 (common on structured meshes), and acos then turns one ulp of the dot
    // product into ~1.5e-8 rad.  The same angles as atan2(|u x v|, u . v) are well conditioned.
    g.alpha = atan2(norm3(cross3(v1n, v2n)), dot3(v1n, v2n));
    const double3 v12n = nrmz(v12);
    g.beta = atan2(norm3(cross3(v12n, v1n)), dot3(v12n, v1n));
    return g;
}

}  // namespace sod
