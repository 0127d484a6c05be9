// Device float arithmetic in the reference's operation order.
//
// Every helper is built from __fadd_rn / __fsub_rn / __fmul_rn / __fdiv_rn /
// __fsqrt_rn, which the compiler never fuses or reassociates, so each result is
// the IEEE single-precision value that glm 0.9.9 computes on the host with
// -ffp-contract=off:
//   dot3  (a.x*b.x + a.y*b.y) + a.z*b.z          glm/detail/func_geometric.inl:54-61
//   dot4  (x + y) + (z + w)                       glm/detail/func_geometric.inl:63-71
//   cross glm/detail/func_geometric.inl:74-84
//   normalize  v * (1 / sqrt(dot(v, v)))          glm/detail/func_geometric.inl:88-94
//   mat4*vec4  (c0*x + c1*y) + (c2*z + c3*w)      glm/detail/type_mat4x4.inl:512-523
//   mat3*vec3  (c0*x + c1*y) + c2*z               glm/detail/type_mat3x3.inl:418-424
#pragma once

namespace pico {
namespace ex {

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }

struct V3 { float x, y, z; };

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return v3(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return v3(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ V3 vmul(V3 a, V3 b) { return v3(mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z)); }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return v3(mul(a.x, s), mul(a.y, s), mul(a.z, s)); }
__device__ __forceinline__ V3 vneg(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, float bx, float by, float bz, float bw)
{
    return add(add(mul(ax, bx), mul(ay, by)), add(mul(az, bz), mul(aw, bw)));
}
__device__ __forceinline__ V3 cross(V3 a, V3 b)
{
    return v3(sub(mul(a.y, b.z), mul(b.y, a.z)), sub(mul(a.z, b.x), mul(b.z, a.x)), sub(mul(a.x, b.y), mul(b.x, a.y)));
}
__device__ __forceinline__ float length(V3 a) { return sqrt_(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return vscale(a, div(1.0f, sqrt_(dot(a, a)))); }
// std::min / std::max (and glm::min / glm::max) as selects: NaN handling follows the operand order.
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// Row-major 3x4 / 4x4 rows of a column-major glm matrix: row r = (M[0][r], M[1][r], M[2][r], M[3][r]).
__device__ __forceinline__ float row4(const float4& r, float x, float y, float z, float w)
{
    return add(add(mul(r.x, x), mul(r.y, y)), add(mul(r.z, z), mul(r.w, w)));
}
__device__ __forceinline__ float row3(const float4& r, float x, float y, float z)
{
    return add(add(mul(r.x, x), mul(r.y, y)), mul(r.z, z));
}

}  // namespace ex
}  // namespace pico
