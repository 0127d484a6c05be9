// Closest-hit traversal of the two-level BVH: one ray per thread, one stack.
//
// What it computes is UpperLevelBVH::get_closest_intersection
// (Core/UpperLevelBVH.cpp:12-20, 59-80 over Core/BVH.cpp:16-63):
//   * a TLAS node is entered when its slab distance (Core/AABB.cpp:108-147,
//     same arithmetic and NaN behaviour) does not exceed the best world
//     distance so far;
//   * each instance reached through a TLAS leaf is searched on its own, in
//     object space (transform_ray, Core/AABB.cpp:43-52) with a fresh best,
//     by Moeller-Trumbore (Core/LowerLevelMeshBVH.cpp:165-207);
//   * the instance's candidate is its closest triangle by object-space t; its
//     world distance is |T * interpolate(u, v) - O| as a 4-vector
//     (Core/LowerLevelMeshBVH.cpp:134-163, Core/UpperLevelBVH.cpp:70-73).
// The reference walks children in order 0, 1 and keeps the first of equal
// distances; this walk visits the nearer child first and instead breaks ties by
// the item's depth-first rank (its array position), which selects the same
// item.  Nodes at exactly the current best distance are therefore still entered.
#pragma once

#include "exact_math.cuh"
#include "layout.h"
#include "traverse_status.h"

#include <stdint.h>

#include <type_traits>

namespace pico {

constexpr uint32_t kNoHit = 0xffffffffu;
constexpr uint32_t kImplicitTri = 0xfffffffeu;   // TraceHit::tri of a hit on an implicit shape

struct TraceHit {
    float t;          // world distance, +inf on a miss
    uint32_t rank;    // TLAS rank of the instance
    uint32_t tri;     // global triangle slot, or kImplicitTri
    float u, v;       // barycentrics; an implicit hit keeps its object-space t in u
};

struct TraceCounters {
    unsigned long long nodes, tris, insts, blas_nodes;   // blas_nodes: the part of nodes inside instances
};

// AABB::intersection_distance; `hit` is false where the reference returns INFINITY.
__device__ __forceinline__ float slab(float lox, float hix, float loy, float hiy, float loz, float hiz, float ox,
                                      float oy, float oz, float ix, float iy, float iz, bool& hit)
{
    using namespace ex;
    const float t1 = mul(sub(lox, ox), ix), t2 = mul(sub(hix, ox), ix);
    const float t3 = mul(sub(loy, oy), iy), t4 = mul(sub(hiy, oy), iy);
    const float t5 = mul(sub(loz, oz), iz), t6 = mul(sub(hiz, oz), iz);
    const bool s1 = t1 > t2, s2 = t3 > t4, s3 = t5 > t6;
    const float a1 = s1 ? t2 : t1, b1 = s1 ? t1 : t2;
    const float a2 = s2 ? t4 : t3, b2 = s2 ? t3 : t4;
    const float a3 = s3 ? t6 : t5, b3 = s3 ? t5 : t6;
    const float tmin = smax(smax(a1, a2), a3);
    const float tmax = smin(smin(b1, b2), b3);
    hit = !(tmax < 0.0f || tmin > tmax);
    return tmin;
}

// The same slab distance and hit flag for data where no t can be NaN (finite
// origin, inverse direction and box): the reference's select-based min / max
// then equal the hardware ones (up to the sign of a zero, which compares equal),
// and an empty child's all-NaN box still reports a miss.
__device__ __forceinline__ float slab_fast(float lox, float hix, float loy, float hiy, float loz, float hiz, float ox,
                                           float oy, float oz, float ix, float iy, float iz, bool& hit)
{
    using namespace ex;
    const float t1 = mul(sub(lox, ox), ix), t2 = mul(sub(hix, ox), ix);
    const float t3 = mul(sub(loy, oy), iy), t4 = mul(sub(hiy, oy), iy);
    const float t5 = mul(sub(loz, oz), iz), t6 = mul(sub(hiz, oz), iz);
    const float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
    const float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
    hit = tmax >= 0.0f && tmin <= tmax;
    return tmin;
}

// max / min that return NaN when either input is NaN (PTX max.NaN / min.NaN).
__device__ __forceinline__ float max_nan(float a, float b)
{
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float min_nan(float a, float b)
{
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// One axis of slab_robust: the entry and exit distances of the face pair [lo - e, hi + e], each
// rounded outwards (entry down, exit up), then widened by 2^-23 of its magnitude for the error of
// the rounded reciprocal r (within 2^-24 of 1 / d).  An infinite r (a zero direction component)
// becomes +-2^64: the ray is taken as nearly parallel, which still meets a slab it lies in and
// puts a slab it lies outside beyond any finite distance (or at an infinite one, a miss).
__device__ __forceinline__ void robust_axis(float lo, float hi, float o, float r, float e, float& tn, float& tf)
{
    const float lo_w = __fsub_rd(lo, e), hi_w = __fadd_ru(hi, e);
    const float rr = fabsf(r) == __int_as_float(0x7f800000) ? copysignf(0x1p64f, r) : r;
    const bool pos = rr >= 0.0f;
    const float n = __fmul_rd(pos ? __fsub_rd(lo_w, o) : __fsub_ru(hi_w, o), rr);
    const float f = __fmul_ru(pos ? __fsub_ru(hi_w, o) : __fsub_rd(lo_w, o), rr);
    tn = __fmaf_rd(-fabsf(n), 0x1p-23f, n);
    tf = __fmaf_ru(fabsf(f), 0x1p-23f, f);
}

// The watertight variant's box test (after Ize, "Robust BVH Ray Traversal", JCGT 2(2), 2013): it
// never rejects a box that the exact ray meets, nor one holding a triangle that the watertight
// test can report hit.  That test decides coverage from the vertices translated to the ray origin
// and sheared, rounding each step once, so what it counts as a hit can lie a few ulps of the
// coordinates in play (the origin's and the vertices') off the exact triangle; every face of the
// box moves outwards by 2^-18 of the largest such magnitude (omag: the ray origin's, plus the
// box's own), far above that error.  A vertex shared by a closed fan lies on the faces of the
// fan's sub-boxes, where the exact slab arithmetic can reject every one of them.  NaN in a box
// (an empty child) gives a NaN entry distance and a miss.
__device__ __forceinline__ float slab_robust(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                             float ox, float oy, float oz, float ix, float iy, float iz, float omag,
                                             bool& hit)
{
    const float bmag = fmaxf(fmaxf(fmaxf(fabsf(lox), fabsf(hix)), fmaxf(fabsf(loy), fabsf(hiy))),
                             fmaxf(fabsf(loz), fabsf(hiz)));
    const float e = __fmul_ru(__fadd_ru(omag, bmag), 0x1p-18f);
    float n1, f1, n2, f2, n3, f3;
    robust_axis(lox, hix, ox, ix, e, n1, f1);
    robust_axis(loy, hiy, oy, iy, e, n2, f2);
    robust_axis(loz, hiz, oz, iz, e, n3, f3);
    const float tmin = max_nan(max_nan(n1, n2), n3);
    const float tmax = min_nan(min_nan(f1, f2), f3);
    hit = tmax >= 0.0f && tmin <= tmax;
    return tmin;
}

// The box test of a traversal: slab_robust in the watertight variant, else the
// reference's slab arithmetic (its NaN-free form where `fast`).
template <bool kWT>
__device__ __forceinline__ float box_test(float lox, float hix, float loy, float hiy, float loz, float hiz, float ox,
                                          float oy, float oz, float ix, float iy, float iz, float omag, bool fast,
                                          bool& hit)
{
    if constexpr (kWT) return slab_robust(lox, hix, loy, hiy, loz, hiz, ox, oy, oz, ix, iy, iz, omag, hit);
    if (fast) return slab_fast(lox, hix, loy, hiy, loz, hiz, ox, oy, oz, ix, iy, iz, hit);
    return slab(lox, hix, loy, hiy, loz, hiz, ox, oy, oz, ix, iy, iz, hit);
}

__device__ __forceinline__ float max_abs3(float a, float b, float c) { return fmaxf(fmaxf(fabsf(a), fabsf(b)), fabsf(c)); }

__device__ __forceinline__ bool all_finite(float a, float b, float c, float d, float e, float f)
{
    return isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d) && isfinite(e) && isfinite(f);
}

// Mesh_Intersector::intersects without the interpolation (done once per instance).
__device__ __forceinline__ bool intersect_triangle(const GpuTri* tri, float ox, float oy, float oz, float dx,
                                                   float dy, float dz, float& t_out, float& u_out, float& v_out)
{
    using namespace ex;
    const float4* p = reinterpret_cast<const float4*>(tri);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    const V3 v0 = v3(a.x, a.y, a.z);
    const V3 e1 = vsub(v3(b.x, b.y, b.z), v0), e2 = vsub(v3(c.x, c.y, c.z), v0);
    const V3 D = v3(dx, dy, dz);
    const V3 h = cross(D, e2);
    const float det = dot(e1, h);
    if (det > -0.0000001f && det < 0.0000001f) return false;
    const float f = __frcp_rn(det);   // (float)(1.0 / det): correctly rounded either way
    const V3 s = vsub(v3(ox, oy, oz), v0);
    const float u = mul(f, dot(s, h));
    if (u < 0.0f || u > 1.0f) return false;
    const V3 q = cross(s, e1);
    const float v = mul(f, dot(D, q));
    if (v < 0.0f || add(u, v) > 1.0f) return false;
    const float t = mul(f, dot(e2, q));
    if (t > 0.0000001f) {
        t_out = t; u_out = u; v_out = v;
        return true;
    }
    return false;
}

// Watertight ray / triangle test (Woop, Benthin and Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013), the opt-in alternative to the reference's
// Moeller-Trumbore.  The vertices are translated to the ray origin and sheared so
// that the ray runs along +z of its dominant axis (the other two axes swapped when
// that component is negative, which keeps the winding); three 2D edge functions
// then decide coverage.  Every product and difference is rounded once and shared
// vertices are stored bit-identically, so the edge function of an edge shared by
// two triangles comes out exactly negated in the other; one that is exactly 0 is
// recomputed in double precision.  A ray through a shared edge or vertex therefore
// hits at least one of the triangles meeting there.  Both sides count (no back-face
// culling) and hits at t <= 1e-7 are rejected, as the reference's test does; (u, v)
// are the weights of v1 and v2, the Moeller-Trumbore meaning.
__device__ __forceinline__ float pick3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ bool intersect_triangle_wt(const GpuTri* tri, float ox, float oy, float oz, float dx,
                                                      float dy, float dz, float& t_out, float& u_out, float& v_out)
{
    using namespace ex;
    const float4* p = reinterpret_cast<const float4*>(tri);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    const float mx = fabsf(dx), my = fabsf(dy), mz = fabsf(dz);
    const int kz = (mx > my) ? ((mx > mz) ? 0 : 2) : ((my > mz) ? 1 : 2);
    const int kx0 = kz == 2 ? 0 : kz + 1, ky0 = kx0 == 2 ? 0 : kx0 + 1;
    const float dkz = pick3(dx, dy, dz, kz);
    const int kx = dkz < 0.0f ? ky0 : kx0, ky = dkz < 0.0f ? kx0 : ky0;
    const float sx = __fdiv_rn(pick3(dx, dy, dz, kx), dkz), sy = __fdiv_rn(pick3(dx, dy, dz, ky), dkz);
    const float sz = __frcp_rn(dkz);
    const float A[3] = {sub(a.x, ox), sub(a.y, oy), sub(a.z, oz)};
    const float B[3] = {sub(b.x, ox), sub(b.y, oy), sub(b.z, oz)};
    const float C[3] = {sub(c.x, ox), sub(c.y, oy), sub(c.z, oz)};
    const float akz = pick3(A[0], A[1], A[2], kz), bkz = pick3(B[0], B[1], B[2], kz), ckz = pick3(C[0], C[1], C[2], kz);
    const float ax = sub(pick3(A[0], A[1], A[2], kx), mul(sx, akz)), ay = sub(pick3(A[0], A[1], A[2], ky), mul(sy, akz));
    const float bx = sub(pick3(B[0], B[1], B[2], kx), mul(sx, bkz)), by = sub(pick3(B[0], B[1], B[2], ky), mul(sy, bkz));
    const float cx = sub(pick3(C[0], C[1], C[2], kx), mul(sx, ckz)), cy = sub(pick3(C[0], C[1], C[2], ky), mul(sy, ckz));
    float U = sub(mul(cx, by), mul(cy, bx));
    float V = sub(mul(ax, cy), mul(ay, cx));
    float W = sub(mul(bx, ay), mul(by, ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)cx * (double)by - (double)cy * (double)bx);
        V = (float)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (float)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = add(add(U, V), W);
    if (det == 0.0f) return false;
    const float T = add(add(mul(U, mul(sz, akz)), mul(V, mul(sz, bkz))), mul(W, mul(sz, ckz)));
    const float rcp = __frcp_rn(det);
    const float t = mul(T, rcp);
    if (!(t > 0.0000001f)) return false;
    t_out = t; u_out = mul(V, rcp); v_out = mul(W, rcp);
    return true;
}

template <bool kWatertight>
__device__ __forceinline__ bool intersect(const GpuTri* tri, float ox, float oy, float oz, float dx, float dy, float dz,
                                          float& t, float& u, float& v)
{
    if (kWatertight) return intersect_triangle_wt(tri, ox, oy, oz, dx, dy, dz, t, u, v);
    return intersect_triangle(tri, ox, oy, oz, dx, dy, dz, t, u, v);
}

// Traversal orders.  kNearFirst enters the nearer child first, breaks equal
// distances by rank, walks a refitted TLAS whose boxes bound each instance's
// transformed vertices (tighter than the reference's transformed mesh AABB,
// still containing every point the instance can be hit at; rays with a zero
// direction component walk the reference's TLAS instead), and bounds each
// BLAS walk by the best world distance so far.  kReferenceOrder walks the
// reference's own boxes, children 0 then 1, keeps the first of equal distances
// and re-tests a deferred child against the best distance when it is reached,
// exactly like the reference's recursion (Core/BVH.cpp:27-63).  Both return the
// reference's answer except where the reference's own float slab test rejects a
// box whose triangle lies a few ulp nearer than the current best (triangles on
// box faces meeting at an edge): there only the reference order reproduces its
// choice.
enum TraversalOrder : int { kNearFirst = 0, kReferenceOrder = 1 };

// Kernel variants: a traversal order, plus kWithImplicit when the scene holds implicit
// shapes (the instance-entry check for them is compiled out otherwise), plus kBounded
// when the launching context set traversal bounds other than the defaults
// (pico_gpu_set_traversal_limits): only those walks read the bounds at run time, so
// the default kernels keep their compile-time bounds and their register allocation.
constexpr int kWithImplicit = 2;
constexpr int kBounded = 4;
constexpr int kWatertight = 8;   // the watertight triangle test (pico_gpu_set_triangle_test)
__host__ __device__ constexpr int traversal_variant(int order, bool implicit, bool bounded, bool watertight)
{
    return (order == kReferenceOrder ? kReferenceOrder : kNearFirst) | (implicit ? kWithImplicit : 0) |
           (bounded ? kBounded : 0) | (watertight ? kWatertight : 0);
}

// Object-space ray of an instance (transform_ray, Core/AABB.cpp:43-52) and its BLAS root.
struct ObjectRay {
    float ox, oy, oz, dx, dy, dz, ix, iy, iz;
    float4 root_lo, root_hi;   // root box xyz; .w carries the root reference / instance id
};

__device__ __forceinline__ ObjectRay to_object(const GpuInstance* inst, const float4 o, const float4 d)
{
    using namespace ex;
    const float4* ip = reinterpret_cast<const float4*>(inst);
    const float4 i0 = __ldg(ip), i1 = __ldg(ip + 1), i2 = __ldg(ip + 2);
    ObjectRay r;
    r.root_lo = __ldg(ip + 7);
    r.root_hi = __ldg(ip + 8);
    r.ox = row4(i0, o.x, o.y, o.z, o.w); r.oy = row4(i1, o.x, o.y, o.z, o.w); r.oz = row4(i2, o.x, o.y, o.z, o.w);
    r.dx = row3(i0, d.x, d.y, d.z); r.dy = row3(i1, d.x, d.y, d.z); r.dz = row3(i2, d.x, d.y, d.z);
    // 1.0f / x correctly rounded (Core/AABB.cpp:48): the same bits as the IEEE division
    r.ix = __frcp_rn(r.dx); r.iy = __frcp_rn(r.dy); r.iz = __frcp_rn(r.dz);
    return r;
}

// |T * (p, 1) - O| as a 4-vector (Core/UpperLevelBVH.cpp:70-73).
__device__ __forceinline__ float world_distance_at(const SceneView& sc, uint32_t rank, float px, float py, float pz,
                                                   const float4 o)
{
    using namespace ex;
    const float4* ip = reinterpret_cast<const float4*>(sc.insts + rank);
    const float4 f0 = __ldg(ip + 3), f1 = __ldg(ip + 4), f2 = __ldg(ip + 5), f3 = __ldg(ip + 6);
    const float ex_ = sub(row4(f0, px, py, pz, 1.0f), o.x), ey = sub(row4(f1, px, py, pz, 1.0f), o.y);
    const float ez = sub(row4(f2, px, py, pz, 1.0f), o.z), ew = sub(row4(f3, px, py, pz, 1.0f), o.w);
    return sqrt_(dot4(ex_, ey, ez, ew, ex_, ey, ez, ew));
}

// Object-space hit of an implicit asset: LowerLevelSphereBVH::calculate_intersection
// (radius 0.5; a ray starting inside hits at t = 0) and LowerLevelCube's slab test
// (Core/LowerLevelImplicitShapesBVH.cpp:24-52, 71-91).  Returns the ray parameter t
// and the hit point.
__device__ __forceinline__ bool implicit_hit(uint32_t root, const ObjectRay& q, float& t, float& px, float& py,
                                             float& pz)
{
    using namespace ex;
    if (root == PICO_REF_SPHERE) {
        const V3 m = v3(q.ox, q.oy, q.oz);
        const float b = dot(m, v3(q.dx, q.dy, q.dz));
        const float c = sub(dot(m, m), 0.25f);
        if (c > 0.0f && b > 0.0f) return false;
        const float discr = sub(mul(b, b), c);
        if (discr < 0.0f) return false;
        t = (float)(-(double)b - sqrt((double)discr));
        if (t < 0.0f) t = 0.0f;
        px = add(q.ox, mul(t, q.dx)); py = add(q.oy, mul(t, q.dy)); pz = add(q.oz, mul(t, q.dz));
        return true;
    }
    bool h;
    const float tm = slab(-0.5f, 0.5f, -0.5f, 0.5f, -0.5f, 0.5f, q.ox, q.oy, q.oz, q.ix, q.iy, q.iz, h);
    if (!h || tm == __int_as_float(0x7f800000)) return false;
    t = tm;
    px = add(q.ox, mul(q.dx, t)); py = add(q.oy, mul(q.dy, t)); pz = add(q.oz, mul(q.dz, t));
    return true;
}

// The candidate of an implicit instance: its world distance and object-space t.
// Kept out of line so the traversal loop does not pay registers for the rare case.
static __device__ __noinline__ bool implicit_candidate(const GpuInstance* inst, const float4 o, const float4 d, float& tw,
                                                float& t)
{
    const ObjectRay q = to_object(inst, o, d);
    float px, py, pz;
    if (!implicit_hit(__float_as_uint(q.root_lo.w), q, t, px, py, pz)) return false;
    using namespace ex;
    const float4* ip = reinterpret_cast<const float4*>(inst);
    const float4 f0 = __ldg(ip + 3), f1 = __ldg(ip + 4), f2 = __ldg(ip + 5), f3 = __ldg(ip + 6);
    const float ex_ = sub(row4(f0, px, py, pz, 1.0f), o.x), ey = sub(row4(f1, px, py, pz, 1.0f), o.y);
    const float ez = sub(row4(f2, px, py, pz, 1.0f), o.z), ew = sub(row4(f3, px, py, pz, 1.0f), o.w);
    tw = sqrt_(dot4(ex_, ey, ez, ew, ex_, ey, ez, ew));
    return true;
}

__device__ __forceinline__ bool is_implicit_root(const GpuInstance* inst)
{
    const uint32_t root = __ldg(&inst->root_ref);
    return root == PICO_REF_SPHERE || root == PICO_REF_CUBE;
}

// World distance of an instance's closest triangle: |T * interpolate(u, v) - O|
// as a 4-vector (Core/LowerLevelMeshBVH.cpp:134-163, Core/UpperLevelBVH.cpp:70-73).
__device__ __forceinline__ float world_distance(const SceneView& sc, uint32_t rank, uint32_t tri, float u, float v,
                                                const float4 o)
{
    using namespace ex;
    const float4* tp = reinterpret_cast<const float4*>(sc.tris + tri);
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    const float w = sub(sub(1.0f, v), u);
    const float px = add(add(mul(w, a.x), mul(u, b.x)), mul(v, c.x));
    const float py = add(add(mul(w, a.y), mul(u, b.y)), mul(v, c.y));
    const float pz = add(add(mul(w, a.z), mul(u, b.z)), mul(v, c.z));
    return world_distance_at(sc, rank, px, py, pz, o);
}

// The state of one near-first walk (the traversal stack is kept apart, in the
// caller's local array, so that the state itself can live in registers).
//
// The ray the node tests use is the world ray in the TLAS and the object-space
// ray inside an instance, switched on entering and leaving an instance.  `limit`
// is the distance a child box may not exceed (the best world distance in the
// TLAS, min(object-space best, BLAS bound) inside), clamped to the largest
// finite float so that one comparison also rejects boxes at +inf.
struct NearFirstState {
    float4 o, d;                     // the world ray
    TraceHit best;
    float exit_below;                // the walk ends once its best hit lies below this
    float cx, cy, cz, cix, ciy, ciz; // the ray of the current level and its reciprocals
    float wmag, cmag;                // the watertight box slack's origin term (world, current)
    float limit;
    float qdx, qdy, qdz;             // object-space direction of the instance being searched
    float lt, lu, lv;                // the instance's best triangle so far (object-space t)
    uint32_t ltri, cur, ref, iter;
    int sp;
    bool wfast, cfast, in_blas;
};

// Sets a walk up.  tmax bounds the hits that count; `occlusion` gives the
// occlusion query: only hits strictly below tmax count (best starts at (tmax,
// rank 0), so no candidate ties it) and the walk ends at the first instance
// whose candidate is one, reported as best.tri != kNoHit.  Otherwise the walk
// ends early once its best hit lies below exit_below: the closest hit then lies
// below it too, and a caller that only asks what kind of instance is hit (a
// shadow ray whose lights all lie at or beyond exit_below) has its answer.
template <bool kWT>
__device__ __forceinline__ void nf_start(NearFirstState& w, const SceneView& sc, const float4 o, const float4 d,
                                         float tmax, float exit_below, bool occlusion)
{
    const float kInf = __int_as_float(0x7f800000);
    const float kMaxFinite = __int_as_float(0x7f7fffff);
    w.o = o; w.d = d;
    w.best.t = tmax; w.best.rank = occlusion ? 0u : kNoHit; w.best.tri = kNoHit; w.best.u = 0.0f; w.best.v = 0.0f;
    w.exit_below = occlusion ? kInf : exit_below;
    const float wix = __frcp_rn(d.x), wiy = __frcp_rn(d.y), wiz = __frcp_rn(d.z);
    // node tests take the NaN-free form when the ray (world or object space) and the boxes are finite
    w.wfast = sc.finite_boxes && all_finite(o.x, o.y, o.z, wix, wiy, wiz);
    w.cx = o.x; w.cy = o.y; w.cz = o.z; w.cix = wix; w.ciy = wiy; w.ciz = wiz;
    w.cfast = w.wfast;
    w.wmag = kWT ? max_abs3(o.x, o.y, o.z) : 0.0f;
    w.cmag = w.wmag;
    w.limit = fminf(tmax, kMaxFinite);
    w.qdx = 0.0f; w.qdy = 0.0f; w.qdz = 0.0f;
    w.lt = kInf; w.lu = 0.0f; w.lv = 0.0f;
    w.ltri = kNoHit; w.cur = 0; w.iter = 0; w.sp = 0;
    w.in_blas = false;
    // A ray with a zero direction component whose origin lies on a box plane gets
    // a NaN slab distance there, and the reference skips that box.  Such rays walk
    // the reference's own TLAS boxes so those decisions stay the reference's; every
    // other ray walks the near-first TLAS, where no slab distance can be NaN.
    w.ref = PICO_REF_DONE;
    const bool axis = d.x == 0.0f || d.y == 0.0f || d.z == 0.0f;
    float lo[3], hi[3];   // selected by value: the scene view lives in kernel parameters
    for (int a = 0; a < 3; ++a) {
        lo[a] = axis ? sc.tlas_lo[a] : sc.tlas_fast_lo[a];
        hi[a] = axis ? sc.tlas_hi[a] : sc.tlas_fast_hi[a];
    }
    bool h;
    const float tm = box_test<kWT>(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], o.x, o.y, o.z, wix, wiy, wiz, w.wmag,
                                   false, h);
    if (h && tm < kInf) w.ref = axis ? sc.tlas_root_ref : sc.tlas_fast_root_ref;
}

// One move of a walk: an inner node, a BLAS leaf, an instance entry or an
// instance exit.  Returns -1 while the walk goes on, else its final status
// (kTraceOk, or the code of the bound it ran into).  One exit at the end: the
// form with a return per case made the renders 2.4 % slower.
template <bool kCount, bool kImplicit, bool kRuntimeBounds, bool kWT>
__device__ __forceinline__ int nf_move(NearFirstState& w, const SceneView& sc, uint32_t* stack, TraceCounters* cnt)
{
    using namespace ex;
    const uint32_t max_iter = kRuntimeBounds ? sc.max_iterations : kTraceMaxIter;
    const int max_stack = kRuntimeBounds ? (int)sc.stack_entries : kTraceStack;
    const float kInf = __int_as_float(0x7f800000);
    const float kMaxFinite = __int_as_float(0x7f7fffff);
    int status = -1;
    if (w.iter >= max_iter) {
        status = kTraceIterLimit;
    } else if (w.ref == PICO_REF_DONE) {
        status = kTraceOk;
    } else {
        ++w.iter;
        if (!pico_is_leaf(w.ref)) {
            const float4* np = reinterpret_cast<const float4*>(sc.nodes + w.ref);
            const float4 n0v = __ldg(np), n1v = __ldg(np + 1), n2v = __ldg(np + 2);
            const uint4 n3v = __ldg(reinterpret_cast<const uint4*>(np) + 3);
            if (kCount) {
                cnt->nodes++;
                if (w.in_blas) cnt->blas_nodes++;
            }
            bool h0, h1;
            float t0, t1;
            if constexpr (kWT) {
                t0 = slab_robust(n0v.x, n0v.y, n0v.z, n0v.w, n2v.x, n2v.y, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, w.cmag, h0);
                t1 = slab_robust(n1v.x, n1v.y, n1v.z, n1v.w, n2v.z, n2v.w, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, w.cmag, h1);
            } else if (w.cfast) {
                t0 = slab_fast(n0v.x, n0v.y, n0v.z, n0v.w, n2v.x, n2v.y, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, h0);
                t1 = slab_fast(n1v.x, n1v.y, n1v.z, n1v.w, n2v.z, n2v.w, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, h1);
            } else {
                t0 = slab(n0v.x, n0v.y, n0v.z, n0v.w, n2v.x, n2v.y, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, h0);
                t1 = slab(n1v.x, n1v.y, n1v.z, n1v.w, n2v.z, n2v.w, w.cx, w.cy, w.cz, w.cix, w.ciy, w.ciz, h1);
            }
            // t <= limit (finite) also rejects t = +inf and NaN, like "t <= best && t < inf"
            const bool v0 = h0 && t0 <= w.limit;
            const bool v1 = h1 && t1 <= w.limit;
            if (v0 && v1) {
                const bool swap = t1 < t0;
                if (w.sp >= max_stack) {
                    status = kTraceStackOverflow;
                } else {
                    stack[w.sp++] = swap ? n3v.x : n3v.y;
                    w.ref = swap ? n3v.y : n3v.x;
                }
            } else if (v0) {
                w.ref = n3v.x;
            } else if (v1) {
                w.ref = n3v.y;
            } else {
                w.ref = w.sp ? stack[--w.sp] : PICO_REF_DONE;
            }
        } else if (w.ref == PICO_REF_END_BLAS) {
            // leave the instance: its candidate is the closest triangle by object-space t
            if (w.ltri != kNoHit) {
                const float tw = world_distance(sc, w.cur, w.ltri, w.lu, w.lv, w.o);
                if (tw < w.best.t || (tw == w.best.t && w.cur < w.best.rank)) {
                    w.best.t = tw; w.best.rank = w.cur; w.best.tri = w.ltri; w.best.u = w.lu; w.best.v = w.lv;
                    if (tw < w.exit_below) status = kTraceOk;
                }
            }
            w.in_blas = false;
            // back to the world ray (its reciprocals recomputed rather than kept in registers)
            w.cx = w.o.x; w.cy = w.o.y; w.cz = w.o.z;
            w.cix = __frcp_rn(w.d.x); w.ciy = __frcp_rn(w.d.y); w.ciz = __frcp_rn(w.d.z);
            w.cfast = w.wfast;
            w.cmag = w.wmag;
            w.limit = fminf(w.best.t, kMaxFinite);
            w.ref = w.sp ? stack[--w.sp] : PICO_REF_DONE;
        } else {
            const uint32_t first = pico_leaf_first(w.ref), count = pico_leaf_count(w.ref);
            if (count == 0) {
                w.ref = w.sp ? stack[--w.sp] : PICO_REF_DONE;
            } else if (w.in_blas) {
                for (uint32_t k = 0; k < count; ++k) {
                    const uint32_t tri = first + k;
                    float t, u, v;
                    if (kCount) cnt->tris++;
                    if (intersect<kWT>(sc.tris + tri, w.cx, w.cy, w.cz, w.qdx, w.qdy, w.qdz, t, u, v) &&
                        (t < w.lt || (t == w.lt && tri < w.ltri))) {
                        w.lt = t; w.ltri = tri; w.lu = u; w.lv = v;
                    }
                }
                w.limit = fminf(w.limit, w.lt);
                w.ref = stack[--w.sp];   // the END_BLAS sentinel is below, so sp > 0 here
            } else if (count > 1 && w.sp >= max_stack) {
                status = kTraceStackOverflow;
            } else {
                // TLAS leaf: search the instance of item `first`; the rest of the leaf waits on the stack
                if (count > 1) stack[w.sp++] = pico_leaf_ref(first + 1, count - 1);
                const uint32_t rank = __ldg(sc.tlas_items + first);
                if (kCount) cnt->insts++;
                if (kImplicit && is_implicit_root(sc.insts + rank)) {
                    // an implicit shape: one candidate, no BLAS and no root box test
                    float tw, t;
                    if (implicit_candidate(sc.insts + rank, w.o, w.d, tw, t) &&
                        (tw < w.best.t || (tw == w.best.t && rank < w.best.rank))) {
                        w.best.t = tw; w.best.rank = rank; w.best.tri = kImplicitTri; w.best.u = t; w.best.v = 0.0f;
                        if (tw < w.exit_below) status = kTraceOk;
                        w.limit = fminf(w.best.t, kMaxFinite);
                    }
                    w.ref = w.sp ? stack[--w.sp] : PICO_REF_DONE;
                } else {
                    const ObjectRay q = to_object(sc.insts + rank, w.o, w.d);
                    // A triangle of an instance at object-space t lies at world distance t |D|
                    // up to float error (relative ~1e-6, absolute ~1e-7 |O|); the BLAS bound
                    // adds 0.1 % and 1e-4 (|O| + 1), far above that error, so it never cuts a
                    // triangle that could beat or tie the best world distance.
                    const float4 o = w.o, d = w.d;
                    const float inv_len = rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
                    const float omag = 1e-4f * (fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z)) + 1.0f);
                    const float gl = (w.best.t * 1.001f + omag) * inv_len;
                    bool h;
                    const float qmag = kWT ? max_abs3(q.ox, q.oy, q.oz) : 0.0f;
                    const float tm = box_test<kWT>(q.root_lo.x, q.root_hi.x, q.root_lo.y, q.root_hi.y, q.root_lo.z,
                                                   q.root_hi.z, q.ox, q.oy, q.oz, q.ix, q.iy, q.iz, qmag, false, h);
                    if (!(h && tm < kInf && tm <= gl)) {
                        w.ref = w.sp ? stack[--w.sp] : PICO_REF_DONE;
                    } else if (w.sp >= max_stack) {
                        status = kTraceStackOverflow;
                    } else {
                        stack[w.sp++] = PICO_REF_END_BLAS;
                        w.in_blas = true;
                        w.cx = q.ox; w.cy = q.oy; w.cz = q.oz; w.cix = q.ix; w.ciy = q.iy; w.ciz = q.iz;
                        w.qdx = q.dx; w.qdy = q.dy; w.qdz = q.dz;
                        w.cfast = sc.finite_boxes && all_finite(q.ox, q.oy, q.oz, q.ix, q.iy, q.iz);
                        w.cmag = qmag;
                        w.limit = fminf(gl, kMaxFinite);   // lt starts at +inf
                        w.cur = rank;
                        w.lt = kInf; w.ltri = kNoHit;
                        w.ref = __float_as_uint(q.root_lo.w);
                    }
                }
            }
        }
    }
    return status;
}

// Whether a lane's next move waits: a move other than an inner node (a leaf, an
// instance entry or exit, or handing in a finished walk) waits while lanes of the
// warp walk inner nodes, until 5/8 of the busy lanes wait.  The warp then runs
// those rarer branches for many lanes at once instead of for one or two in most
// of its steps.  Measured on the 1080p lit-field renders, first with warps that
// held their 32 rays to the end, against no waiting: a fixed count of 4 waiting
// lanes 1.5 % slower, 8 2.4 % faster, 12 3.4 %, 16 2.8 %, 20 1.6 %, 24 no
// faster, 32 (a while-while walk) 1.5 % slower; exempting the BLAS leaves 9 %
// slower; a share of the busy lanes instead of a count: 3/8 6 %, 7/16 6.8 %,
// 1/2 7.1 %, 9/16 6.6 %, 5/8 6.5 %, 3/4 5.1 % faster; releasing one kind of move
// at a time 2 % slower than all at once.  Then with idle lanes refilled (see
// walk_queue), against 1/2: 3/8 4.8 % slower, 5/8 1.3 % faster, 11/16 1.0 %,
// 3/4 no faster, 7/8 2.5 % slower.  `busy`: the lanes holding a walk, `inner`:
// this lane's next move is an inner node (false for a lane without a walk).
// Every lane of `busy` must call it.
__device__ __forceinline__ bool nf_release(unsigned busy, bool inner, unsigned& at_node)
{
    at_node = __ballot_sync(busy, inner);
    return at_node == 0 || 8 * __popc(busy & ~at_node) >= 5 * __popc(busy);
}

// One ray's closest hit by the near-first walk (or its occlusion query, kAnyHit).
template <bool kCount, bool kImplicit, bool kAnyHit = false, bool kRuntimeBounds = false, bool kWT = false>
__device__ __forceinline__ int trace_near_first(const SceneView& sc, const float4 o, const float4 d, TraceHit& best,
                                                TraceCounters* cnt, float tmax = INFINITY,
                                                float exit_below = -INFINITY)
{
    NearFirstState w;
    uint32_t stack[kTraceStack];
    nf_start<kWT>(w, sc, o, d, tmax, exit_below, kAnyHit);
    int status;
    for (;;) {
        // lanes that finished their walk have left the loop: the rest of the warp is busy
        unsigned at_node;
        const bool inner = !pico_is_leaf(w.ref);
        if (!nf_release(__activemask(), inner, at_node) && !inner) continue;
        status = nf_move<kCount, kImplicit, kRuntimeBounds, kWT>(w, sc, stack, cnt);
        if (status >= 0) break;
    }
    best = w.best;
    if (kAnyHit && best.tri == kNoHit) best.rank = kNoHit;
    return status;
}

// Walks every ray of a queue of n entries with a warp's lanes, refilling idle
// lanes in batches.  The walks and their hits are trace_near_first's; only the
// order in which a warp's lanes make their moves differs.  `Rays` supplies the
// entries:
//   rays.load(k, o, d, tmax, exit_below, occlusion) -> a lane tag for entry k,
//   rays.finish(tag, best, status) hands in a finished walk;
// `Rays::Tag` is the tag's type, `Rays::Index` that of the entry indices.  A
// lane whose walk ended waits (see
// nf_release) to hand it in; once kRefillIdle lanes of the warp are idle they
// take the next entries of the warp's claim together, and the warp claims
// kClaim entries of the shared counter `work` at a time.  The earlier form, a
// warp holding its 32 rays until the slowest ended, left lanes idle for most
// of a walk's tail.  The 1080p renders: refilling at 8 idle lanes with one
// atomic per refill 4.4 % faster (16 lanes 2.3 %, 12 4.3 %, 4 2.2 %, 2 and 1
// slower), then claims of 64 entries another 4.8 % (the atomics on one counter
// had become frequent), but 35 % slower Cornell-box renders, whose launches
// hold a few dozen rays per warp: a warp then walked two or three claims'
// worth of rays while others had none, so a launch with fewer than kClaim rays
// per warp claims 32 at a time (the Cornell box back to 21 % slower than before
// the refills, the 1080p renders unchanged), and the bar at 1024 rays per warp
// instead of 64 brought the Cornell box to 17 % slower (the 1080p renders 0.1 %
// faster); refilling only fully idle warps below the bar would bring it to 8 %
// slower but cost the 1080p renders 1.5 %, whose small late-depth launches are
// long-tailed.  A 32-bit Index for queues of fewer than 2^32 entries keeps the
// extension kernel free of spills.
constexpr uint32_t kRefillIdle = 8;
constexpr uint32_t kClaim = 64;   // queue entries a warp claims at a time
// A claim must cover a refill of all 32 lanes, or the claimed range [next, end)
// could run backwards and the warp would never claim again.
static_assert(kClaim >= 32, "a claim covers a whole warp's refill");
constexpr uint32_t kBigLaunch = 1024;   // rays per warp from which a launch claims kClaim at a time
template <bool kCount, bool kImplicit, bool kRuntimeBounds, bool kWT, class Rays>
__device__ __forceinline__ void walk_queue(const SceneView& sc, Rays& rays, typename Rays::Index n,
                                           unsigned long long* work, TraceCounters* cnt)
{
    using Index = typename Rays::Index;
    const unsigned lane = threadIdx.x & 31u;
    NearFirstState w;
    uint32_t stack[kTraceStack];
    typename Rays::Tag tag = 0;
    bool live = false;
    unsigned busy = 0;   // warp-uniform: the lanes holding a walk (lanes whose walk ended on a bound may linger)
    bool more = true;    // warp-uniform: the queue may hold entries
    Index next = 0, end = 0;   // warp-uniform: the warp's claimed entries [next, end)
    // a launch with fewer than kBigLaunch rays per warp claims 32 at a time, so that its rays spread over the warps
    const bool big = (uint64_t)n >= (uint64_t)gridDim.x * (blockDim.x >> 5) * kBigLaunch;
    const uint32_t claim = big ? kClaim : 32u;
    for (;;) {
        if (more && __popc(busy) <= 32 - kRefillIdle) {
            const unsigned idle = ~busy;
            const uint32_t need = __popc(idle);
            const uint32_t avail = (uint32_t)(end - next);
            Index fresh = 0;
            if (need > avail) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(work, (unsigned long long)claim);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= (unsigned long long)n) {
                    more = false;
                    fresh = n;
                } else {
                    fresh = (Index)base;
                }
            }
            const uint32_t r = __popc(idle & ((1u << lane) - 1u));
            const Index k = r < avail ? next + r : fresh + (r - avail);
            if (need > avail) {
                next = fresh + (need - avail);
                end = fresh + claim;
            } else {
                next += need;
            }
            if (!live && ((idle >> lane) & 1u) && k < n && (r < avail || more)) {
                float4 o, d;
                float tmax, exit_below;
                bool occlusion;
                tag = rays.load(k, o, d, tmax, exit_below, occlusion);
                nf_start<kWT>(w, sc, o, d, tmax, exit_below, occlusion);
                live = true;
            }
            busy = __ballot_sync(0xffffffffu, live);
        }
        if (busy == 0) {
            if (!more) break;
            continue;
        }
        unsigned at_node;
        const bool inner = live && !pico_is_leaf(w.ref);
        const bool release = nf_release(0xffffffffu, inner, at_node);
        if (live && (inner || release)) {
            const int status = nf_move<kCount, kImplicit, kRuntimeBounds, kWT>(w, sc, stack, cnt);
            if (status >= 0) {
                rays.finish(tag, w.best, status);
                live = false;
            }
        }
        if (release) busy = __ballot_sync(0xffffffffu, live);
    }
}

// A deferred child of the reference-order walk and its slab distance (NaN: box
// missed; -inf: nothing to test).
struct StackEntry { uint32_t ref; float tmin; };

template <bool kCount, bool kImplicit, bool kRuntimeBounds = false, bool kWT = false>
__device__ __forceinline__ int trace_reference_order(const SceneView& sc, const float4 o, const float4 d,
                                                     TraceHit& best, TraceCounters* cnt)
{
    using namespace ex;
    const uint32_t max_iter = kRuntimeBounds ? sc.max_iterations : kTraceMaxIter;
    const int max_stack = kRuntimeBounds ? (int)sc.stack_entries : kTraceStack;
    const float kInf = __int_as_float(0x7f800000);
    const float kNan = __int_as_float(0x7fffffff);
    StackEntry stack[kTraceStack];
    int sp = 0;
    best.t = kInf; best.rank = kNoHit; best.tri = kNoHit; best.u = 0.0f; best.v = 0.0f;
    const float wix = __frcp_rn(d.x), wiy = __frcp_rn(d.y), wiz = __frcp_rn(d.z);
    ObjectRay q{};
    float lt = kInf, lu = 0.0f, lv = 0.0f;
    uint32_t ltri = kNoHit, cur = 0;
    bool in_blas = false;
    // the next deferred entry whose box still passes against the best distance now
    auto pop = [&]() -> uint32_t {
        while (sp > 0) {
            const StackEntry e = stack[--sp];
            if (e.tmin == -kInf || e.tmin < (in_blas ? lt : best.t)) return e.ref;
        }
        return PICO_REF_DONE;
    };

    const float wmag = kWT ? max_abs3(o.x, o.y, o.z) : 0.0f;   // the box slack's origin term (watertight only)
    float qmag = 0.0f;
    uint32_t ref = PICO_REF_DONE;
    {
        bool h;
        const float tm = box_test<kWT>(sc.tlas_lo[0], sc.tlas_hi[0], sc.tlas_lo[1], sc.tlas_hi[1], sc.tlas_lo[2],
                                       sc.tlas_hi[2], o.x, o.y, o.z, wix, wiy, wiz, wmag, false, h);
        if (h && tm < kInf) ref = sc.tlas_root_ref;
    }
    for (uint32_t iter = 0;; ++iter) {
        if (iter >= max_iter) return kTraceIterLimit;
        if (ref == PICO_REF_DONE) break;
        if (!pico_is_leaf(ref)) {
            const float4* np = reinterpret_cast<const float4*>(sc.nodes + ref);
            const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
            const uint4 n3 = __ldg(reinterpret_cast<const uint4*>(np) + 3);
            if (kCount) cnt->nodes++;
            const float rx = in_blas ? q.ox : o.x, ry = in_blas ? q.oy : o.y, rz = in_blas ? q.oz : o.z;
            const float rix = in_blas ? q.ix : wix, riy = in_blas ? q.iy : wiy, riz = in_blas ? q.iz : wiz;
            const float rmag = in_blas ? qmag : wmag;
            bool h0, h1;
            const float t0 = box_test<kWT>(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, rx, ry, rz, rix, riy, riz, rmag, false, h0);
            const float t1 = box_test<kWT>(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, rx, ry, rz, rix, riy, riz, rmag, false, h1);
            // child 1 waits on the stack and is tested when reached
            if (n3.y != PICO_REF_EMPTY) {
                if (sp >= max_stack) return kTraceStackOverflow;
                stack[sp++] = StackEntry{n3.y, h1 ? t1 : kNan};
            }
            ref = (n3.x != PICO_REF_EMPTY && h0 && t0 < (in_blas ? lt : best.t)) ? n3.x : pop();
            continue;
        }
        if (ref == PICO_REF_END_BLAS) {
            if (ltri != kNoHit) {
                const float tw = world_distance(sc, cur, ltri, lu, lv, o);
                if (tw < best.t) {
                    best.t = tw; best.rank = cur; best.tri = ltri; best.u = lu; best.v = lv;
                }
            }
            in_blas = false;
            ref = pop();
            continue;
        }
        const uint32_t first = pico_leaf_first(ref), count = pico_leaf_count(ref);
        if (count == 0) {
            ref = pop();
            continue;
        }
        if (in_blas) {
            for (uint32_t k = 0; k < count; ++k) {
                const uint32_t tri = first + k;
                float t, u, v;
                if (kCount) cnt->tris++;
                if (intersect<kWT>(sc.tris + tri, q.ox, q.oy, q.oz, q.dx, q.dy, q.dz, t, u, v) && t < lt) {
                    lt = t; ltri = tri; lu = u; lv = v;
                }
            }
            ref = pop();
            continue;
        }
        if (count > 1) {
            if (sp >= max_stack) return kTraceStackOverflow;
            stack[sp++] = StackEntry{pico_leaf_ref(first + 1, count - 1), -kInf};
        }
        const uint32_t rank = __ldg(sc.tlas_items + first);   // the identity on the reference's tree
        if (kCount) cnt->insts++;
        if (kImplicit && is_implicit_root(sc.insts + rank)) {
            float tw, t;
            if (implicit_candidate(sc.insts + rank, o, d, tw, t) && tw < best.t) {
                best.t = tw; best.rank = rank; best.tri = kImplicitTri; best.u = t; best.v = 0.0f;
            }
            ref = pop();
            continue;
        }
        q = to_object(sc.insts + rank, o, d);
        if (kWT) qmag = max_abs3(q.ox, q.oy, q.oz);
        bool h;
        const float tm = box_test<kWT>(q.root_lo.x, q.root_hi.x, q.root_lo.y, q.root_hi.y, q.root_lo.z, q.root_hi.z,
                                       q.ox, q.oy, q.oz, q.ix, q.iy, q.iz, qmag, false, h);
        if (!(h && tm < kInf)) {
            ref = pop();
            continue;
        }
        if (sp >= max_stack) return kTraceStackOverflow;
        stack[sp++] = StackEntry{PICO_REF_END_BLAS, -kInf};
        in_blas = true;
        cur = rank;
        lt = kInf; ltri = kNoHit;
        ref = __float_as_uint(q.root_lo.w);
    }
    return kTraceOk;
}

// The closest hit; the near-first walk may return early with a hit below
// exit_below instead (see trace_near_first), the reference order never does.
template <bool kCount, int kVariant>
__device__ __forceinline__ int trace_closest(const SceneView& sc, const float4 o, const float4 d, TraceHit& best,
                                             TraceCounters* cnt, float exit_below = -INFINITY)
{
    constexpr bool kImplicit = (kVariant & kWithImplicit) != 0;
    constexpr bool kRuntime = (kVariant & kBounded) != 0;
    constexpr bool kWT = (kVariant & kWatertight) != 0;
    if ((kVariant & kReferenceOrder) != 0)
        return trace_reference_order<kCount, kImplicit, kRuntime, kWT>(sc, o, d, best, cnt);
    return trace_near_first<kCount, kImplicit, false, kRuntime, kWT>(sc, o, d, best, cnt, INFINITY, exit_below);
}

// A lower bound on the world distance of every hit on a NEE light seen from o:
// the distance from o to the nearest light's widened world box (a hit's world
// distance |T p - o| is at least that of its xyz part, and T p lies in its light's
// box up to float error far below the widening), or -inf when the scene has no
// such boxes.  A NaN origin gives 0.
__device__ __forceinline__ float light_distance_bound(const SceneView& sc, const float4 o)
{
    if (!sc.light_bounds) return -INFINITY;
    const float4* box = reinterpret_cast<const float4*>(sc.light_boxes);
    float b2 = INFINITY;
    for (uint32_t l = 0; l < sc.nlights; ++l) {
        const float4 lo = __ldg(box + 2 * l), hi = __ldg(box + 2 * l + 1);
        const float gx = fmaxf(fmaxf(lo.x - o.x, o.x - hi.x), 0.0f);
        const float gy = fmaxf(fmaxf(lo.y - o.y, o.y - hi.y), 0.0f);
        const float gz = fmaxf(fmaxf(lo.z - o.z, o.z - hi.z), 0.0f);
        b2 = fminf(b2, gx * gx + gy * gy + gz * gz);
    }
    return sqrtf(b2);
}

// Whether anything lies at a world distance below tmax along the ray (closest-hit
// semantics: exactly when the closest hit is nearer than tmax).  The near-first
// walk bounds its search by tmax and stops at the first such instance; the
// reference order runs the closest hit.
template <int kVariant, bool kCount = false>
__device__ __forceinline__ int trace_occluded(const SceneView& sc, const float4 o, const float4 d, float tmax,
                                              bool& occluded, TraceCounters* cnt = nullptr)
{
    constexpr bool kImplicit = (kVariant & kWithImplicit) != 0;
    constexpr bool kRuntime = (kVariant & kBounded) != 0;
    constexpr bool kWT = (kVariant & kWatertight) != 0;
    TraceHit h;
    int s;
    if ((kVariant & kReferenceOrder) != 0) {
        s = trace_reference_order<kCount, kImplicit, kRuntime, kWT>(sc, o, d, h, cnt);
        occluded = h.rank != kNoHit && h.t < tmax;
    } else {
        s = trace_near_first<kCount, kImplicit, true, kRuntime, kWT>(sc, o, d, h, cnt, tmax);
        occluded = h.rank != kNoHit;
    }
    return s;
}

// Adds a thread's work counters to counters[0..3] (nodes, triangles, instance
// entries, nodes inside instances) with one atomic per warp and counter; the
// whole warp must call it.
__device__ __forceinline__ void flush_counters(TraceCounters c, unsigned long long* counters)
{
    for (int off = 16; off > 0; off >>= 1) {
        c.nodes += __shfl_down_sync(0xffffffffu, c.nodes, off);
        c.tris += __shfl_down_sync(0xffffffffu, c.tris, off);
        c.insts += __shfl_down_sync(0xffffffffu, c.insts, off);
        c.blas_nodes += __shfl_down_sync(0xffffffffu, c.blas_nodes, off);
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(&counters[0], c.nodes);
        atomicAdd(&counters[1], c.tris);
        atomicAdd(&counters[2], c.insts);
        atomicAdd(&counters[3], c.blas_nodes);
    }
}

// Whether a launch with this view reads its traversal bounds at run time.
__host__ __device__ inline bool bounded_view(const SceneView& sc)
{
    return sc.max_iterations != kTraceMaxIter || sc.stack_entries != (uint32_t)kTraceStack;
}

// Calls f(std::integral_constant<int, V>) for the kernel variant V of (order, scene).
template <class F>
__host__ auto with_variant(int order, const SceneView& sc, F&& f)
{
    switch (traversal_variant(order, sc.has_implicit != 0, bounded_view(sc), sc.watertight != 0)) {
    case 0: return f(std::integral_constant<int, 0>{});
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 3: return f(std::integral_constant<int, 3>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 5: return f(std::integral_constant<int, 5>{});
    case 6: return f(std::integral_constant<int, 6>{});
    case 7: return f(std::integral_constant<int, 7>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 9: return f(std::integral_constant<int, 9>{});
    case 10: return f(std::integral_constant<int, 10>{});
    case 11: return f(std::integral_constant<int, 11>{});
    case 12: return f(std::integral_constant<int, 12>{});
    case 13: return f(std::integral_constant<int, 13>{});
    case 14: return f(std::integral_constant<int, 14>{});
    default: return f(std::integral_constant<int, 15>{});
    }
}

}  // namespace pico
