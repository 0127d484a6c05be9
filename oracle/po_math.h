/*
 * Oracle (test infrastructure only): float vector arithmetic in the exact
 * operation order of glm 0.9.9.0, which the Pico reference uses for every
 * geometric quantity on its rendering path.  Compiled with -ffp-contract=off
 * so that no multiply-add is fused; each helper performs the same IEEE float
 * operations, in the same association, as the glm routine it names:
 *
 *   dot3  : (a.x*b.x + a.y*b.y) + a.z*b.z          glm/detail/func_geometric.inl:54-61
 *   dot4  : (a.x*b.x + a.y*b.y) + (a.z*b.z + a.w*b.w)  func_geometric.inl:63-71
 *   cross : func_geometric.inl:74-84
 *   normalize : v * (1 / sqrt(dot(v, v)))           func_geometric.inl:88-94, func_exponential.inl:132-135
 *   mat4 * vec4 : (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w)  detail/type_mat4x4.inl:512-523
 *   mat3 * vec3 : (c0*v.x + c1*v.y) + c2*v.z          detail/type_mat3x3.inl:418-424
 *   min/max : (y < x) ? y : x  /  (x < y) ? y : x     (glm::min/max on vectors)
 *
 * Matrices are column-major like glm: m[c][r] is column c, row r.
 */
#ifndef PICO_ORACLE_MATH_H
#define PICO_ORACLE_MATH_H

#include <math.h>
#include <stdint.h>

typedef struct { float x, y; } po_v2;
typedef struct { float x, y, z; } po_v3;
typedef struct { float x, y, z, w; } po_v4;
typedef struct { float m[4][4]; } po_m4;
typedef struct { float m[3][3]; } po_m3;

static inline po_v2 v2(float x, float y) { po_v2 r = {x, y}; return r; }
static inline po_v3 v3(float x, float y, float z) { po_v3 r = {x, y, z}; return r; }
static inline po_v4 v4(float x, float y, float z, float w) { po_v4 r = {x, y, z, w}; return r; }
static inline po_v3 v3_of4(po_v4 a) { return v3(a.x, a.y, a.z); }
static inline po_v4 v4_of3(po_v3 a, float w) { return v4(a.x, a.y, a.z, w); }

static inline po_v3 v3_add(po_v3 a, po_v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline po_v3 v3_sub(po_v3 a, po_v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline po_v3 v3_mul(po_v3 a, po_v3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline po_v3 v3_scale(po_v3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline po_v3 v3_sdiv(po_v3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline po_v3 v3_neg(po_v3 a) { return v3(-a.x, -a.y, -a.z); }
static inline po_v4 v4_add(po_v4 a, po_v4 b) { return v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline po_v4 v4_sub(po_v4 a, po_v4 b) { return v4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline po_v4 v4_scale(po_v4 a, float s) { return v4(a.x * s, a.y * s, a.z * s, a.w * s); }

static inline float v3_dot(po_v3 a, po_v3 b)
{
    const float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (x + y) + z;
}
static inline float v4_dot(po_v4 a, po_v4 b)
{
    const float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z, w = a.w * b.w;
    return (x + y) + (z + w);
}
static inline po_v3 v3_cross(po_v3 a, po_v3 b)
{
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline float v3_length(po_v3 a) { return sqrtf(v3_dot(a, a)); }
static inline float v4_length(po_v4 a) { return sqrtf(v4_dot(a, a)); }
static inline po_v3 v3_normalize(po_v3 a) { return v3_scale(a, 1.0f / sqrtf(v3_dot(a, a))); }

static inline float f_min(float x, float y) { return (y < x) ? y : x; }
static inline float f_max(float x, float y) { return (x < y) ? y : x; }
static inline po_v3 v3_min(po_v3 a, po_v3 b) { return v3(f_min(a.x, b.x), f_min(a.y, b.y), f_min(a.z, b.z)); }
static inline po_v3 v3_max(po_v3 a, po_v3 b) { return v3(f_max(a.x, b.x), f_max(a.y, b.y), f_max(a.z, b.z)); }
static inline po_v4 v4_min(po_v4 a, po_v4 b) { return v4(f_min(a.x, b.x), f_min(a.y, b.y), f_min(a.z, b.z), f_min(a.w, b.w)); }
static inline po_v4 v4_max(po_v4 a, po_v4 b) { return v4(f_max(a.x, b.x), f_max(a.y, b.y), f_max(a.z, b.z), f_max(a.w, b.w)); }

static inline po_v4 m4_mul_v4(const po_m4* m, po_v4 v)
{
    po_v4 r;
    r.x = (m->m[0][0] * v.x + m->m[1][0] * v.y) + (m->m[2][0] * v.z + m->m[3][0] * v.w);
    r.y = (m->m[0][1] * v.x + m->m[1][1] * v.y) + (m->m[2][1] * v.z + m->m[3][1] * v.w);
    r.z = (m->m[0][2] * v.x + m->m[1][2] * v.y) + (m->m[2][2] * v.z + m->m[3][2] * v.w);
    r.w = (m->m[0][3] * v.x + m->m[1][3] * v.y) + (m->m[2][3] * v.z + m->m[3][3] * v.w);
    return r;
}
/* glm::mat3x3(mat4) * vec3: the upper-left 3x3 block. */
static inline po_v3 m4_mul_v3(const po_m4* m, po_v3 v)
{
    po_v3 r;
    r.x = (m->m[0][0] * v.x + m->m[1][0] * v.y) + m->m[2][0] * v.z;
    r.y = (m->m[0][1] * v.x + m->m[1][1] * v.y) + m->m[2][1] * v.z;
    r.z = (m->m[0][2] * v.x + m->m[1][2] * v.y) + m->m[2][2] * v.z;
    return r;
}
static inline po_v3 m3_mul_v3(const po_m3* m, po_v3 v)
{
    po_v3 r;
    r.x = (m->m[0][0] * v.x + m->m[1][0] * v.y) + m->m[2][0] * v.z;
    r.y = (m->m[0][1] * v.x + m->m[1][1] * v.y) + m->m[2][1] * v.z;
    r.z = (m->m[0][2] * v.x + m->m[1][2] * v.y) + m->m[2][2] * v.z;
    return r;
}

#endif
