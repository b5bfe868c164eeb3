// sod_faces.cuh -- the 64-byte face record of the regular (FP32) collocation passes:
// {y1, area}, {y2, nx}, {y3, ny}, {nz, j0, j1, j2 (int bits)} as four float4.
#pragma once
#include <cuda_runtime.h>

namespace sod {

struct FaceRec {
    float3 y1, y2, y3, n;
    float area;
    int j0, j1, j2;
};
__device__ __forceinline__ FaceRec load_face(const float4 *__restrict__ faces, int f) {
    const float4 q0 = __ldg(faces + 4 * f), q1 = __ldg(faces + 4 * f + 1), q2 = __ldg(faces + 4 * f + 2),
                 q3 = __ldg(faces + 4 * f + 3);
    FaceRec r;
    r.y1 = make_float3(q0.x, q0.y, q0.z);
    r.area = q0.w;
    r.y2 = make_float3(q1.x, q1.y, q1.z);
    r.y3 = make_float3(q2.x, q2.y, q2.z);
    r.n = make_float3(q1.w, q2.w, q3.x);
    r.j0 = __float_as_int(q3.y);
    r.j1 = __float_as_int(q3.z);
    r.j2 = __float_as_int(q3.w);
    return r;
}

}  // namespace sod
