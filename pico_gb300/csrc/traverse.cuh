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

namespace pico {

constexpr int kTraceStack = 96;
constexpr uint32_t kTraceMaxIter = 1u << 24;
constexpr uint32_t kNoHit = 0xffffffffu;

struct TraceHit {
    float t;          // world distance, +inf on a miss
    uint32_t rank;    // TLAS rank of the instance
    uint32_t tri;     // global triangle slot
    float u, v;
};

struct TraceCounters {
    unsigned long long nodes, tris, insts;
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

// Traversal orders.  kNearFirst enters the nearer child first and breaks
// equal distances by rank; kReferenceOrder walks children 0 then 1 and keeps the
// first of equal distances, re-testing a deferred child against the best
// distance at the moment it is reached, exactly like the reference's recursion
// (Core/BVH.cpp:27-63).  Both return the reference's answer except where the
// reference's own float slab test rejects a box whose triangle lies a few ulp
// nearer than the current best (triangles on box faces meeting at an edge):
// there only the reference order reproduces its choice.
enum TraversalOrder : int { kNearFirst = 0, kReferenceOrder = 1 };

// A stack entry: a reference and the slab distance of its box (NaN = box
// missed; -inf = no box to test).
struct StackEntry { uint32_t ref; float tmin; };

// One ray's traversal as a resumable state machine: start() loads the ray,
// step() advances by one unit of work (an inner node, a leaf, entering or
// leaving an instance) and reports when the ray is finished, so a persistent
// kernel can refill finished lanes while the others keep going.
template <bool kCount, int kOrder>
struct Traversal {
    // world ray
    float ox, oy, oz, ow, dx, dy, dz;
    float wix, wiy, wiz;
    // object-space ray of the instance being searched
    float qox, qoy, qoz, qdx, qdy, qdz, qix, qiy, qiz;
    float lt, lu, lv;     // closest triangle of the current instance (object-space t)
    float gl;             // near-first only: object-space bound implied by the best world distance
    float inv_len;        // 1 / |D|
    float omag;           // 1e-4 (max |O_i| + 1): absolute slack of the instance bound
    uint32_t ltri, cur, ref;
    int sp;
    bool in_blas;
    TraceHit best;

    __device__ __forceinline__ bool visit(float t, float limit) const
    {
        const float kInf = __int_as_float(0x7f800000);
        return kOrder == kReferenceOrder ? (t < limit) : (t <= limit && t < kInf);
    }

    __device__ __forceinline__ void start(const SceneView& sc, const float4 o, const float4 d)
    {
        using namespace ex;
        const float kInf = __int_as_float(0x7f800000);
        ox = o.x; oy = o.y; oz = o.z; ow = o.w; dx = d.x; dy = d.y; dz = d.z;
        wix = div(1.0f, d.x); wiy = div(1.0f, d.y); wiz = div(1.0f, d.z);
        inv_len = kOrder == kNearFirst ? rsqrtf(d.x * d.x + d.y * d.y + d.z * d.z) : 0.0f;
        omag = 1e-4f * (fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z)) + 1.0f);
        best.t = kInf; best.rank = kNoHit; best.tri = kNoHit; best.u = 0.0f; best.v = 0.0f;
        lt = kInf; lu = lv = 0.0f; gl = kInf; ltri = kNoHit; cur = 0;
        sp = 0;
        in_blas = false;
        bool h;
        const float tm = slab(sc.tlas_lo[0], sc.tlas_hi[0], sc.tlas_lo[1], sc.tlas_hi[1], sc.tlas_lo[2], sc.tlas_hi[2],
                              ox, oy, oz, wix, wiy, wiz, h);
        ref = (h && tm < kInf) ? sc.tlas_root_ref : PICO_REF_DONE;
    }

    __device__ __forceinline__ float limit() const
    {
        if (!in_blas) return best.t;
        return kOrder == kNearFirst ? fminf(lt, gl) : lt;
    }

    // Returns kTraceOk while the ray continues, kTraceDone when finished, or an error.
    // `stack` is the lane's traversal stack, kept outside the struct so the
    // scalar state stays in registers.
    __device__ __forceinline__ int step(const SceneView& sc, StackEntry* stack, TraceCounters* cnt)
    {
        using namespace ex;
        const float kInf = __int_as_float(0x7f800000);
        const float kNan = __int_as_float(0x7fffffff);
        if (ref == PICO_REF_DONE) {
            // pop the next entry whose box still qualifies against the current best
            while (sp > 0) {
                const StackEntry e = stack[--sp];
                if (e.tmin == -kInf || visit(e.tmin, e.ref == PICO_REF_END_BLAS ? kInf : limit())) {
                    ref = e.ref;
                    break;
                }
            }
            if (ref == PICO_REF_DONE) return kTraceDone;
        }
        if (!pico_is_leaf(ref)) {
            const float4* np = reinterpret_cast<const float4*>(sc.nodes + ref);
            const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
            const uint4 n3 = __ldg(reinterpret_cast<const uint4*>(np) + 3);
            if (kCount) cnt->nodes++;
            const float rx = in_blas ? qox : ox, ry = in_blas ? qoy : oy, rz = in_blas ? qoz : oz;
            const float rix = in_blas ? qix : wix, riy = in_blas ? qiy : wiy, riz = in_blas ? qiz : wiz;
            const float lim = limit();
            bool h0, h1;
            float t0 = slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, rx, ry, rz, rix, riy, riz, h0);
            float t1 = slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, rx, ry, rz, rix, riy, riz, h1);
            t0 = h0 ? t0 : kNan;
            t1 = h1 ? t1 : kNan;
            if (kOrder == kReferenceOrder) {
                // child 1 waits on the stack and is tested when reached
                if (n3.y != PICO_REF_EMPTY) {
                    if (sp >= kTraceStack) return kTraceStackOverflow;
                    stack[sp++] = StackEntry{n3.y, t1};
                }
                ref = (n3.x != PICO_REF_EMPTY && visit(t0, lim)) ? n3.x : PICO_REF_DONE;
            } else {
                const bool v0 = visit(t0, lim), v1 = visit(t1, lim);
                if (v0 && v1) {
                    const bool swap = t1 < t0;
                    if (sp >= kTraceStack) return kTraceStackOverflow;
                    stack[sp++] = swap ? StackEntry{n3.x, t0} : StackEntry{n3.y, t1};
                    ref = swap ? n3.y : n3.x;
                } else {
                    ref = v0 ? n3.x : (v1 ? n3.y : PICO_REF_DONE);
                }
            }
            return kTraceOk;
        }
        if (ref == PICO_REF_END_BLAS) {
            // leave the instance: its candidate is the closest triangle by object-space t
            if (ltri != kNoHit) {
                const float4* tp = reinterpret_cast<const float4*>(sc.tris + ltri);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                const float w = sub(sub(1.0f, lv), lu);
                const float px = add(add(mul(w, a.x), mul(lu, b.x)), mul(lv, c.x));
                const float py = add(add(mul(w, a.y), mul(lu, b.y)), mul(lv, c.y));
                const float pz = add(add(mul(w, a.z), mul(lu, b.z)), mul(lv, c.z));
                const float4* ip = reinterpret_cast<const float4*>(sc.insts + cur);
                const float4 f0 = __ldg(ip + 3), f1 = __ldg(ip + 4), f2 = __ldg(ip + 5), f3 = __ldg(ip + 6);
                const float wx = row4(f0, px, py, pz, 1.0f), wy = row4(f1, px, py, pz, 1.0f);
                const float wz = row4(f2, px, py, pz, 1.0f), ww = row4(f3, px, py, pz, 1.0f);
                const float ex_ = sub(wx, ox), ey = sub(wy, oy), ez = sub(wz, oz), ew = sub(ww, ow);
                const float tw = sqrt_(dot4(ex_, ey, ez, ew, ex_, ey, ez, ew));
                const bool better = kOrder == kReferenceOrder ? tw < best.t
                                                              : (tw < best.t || (tw == best.t && cur < best.rank));
                if (better) {
                    best.t = tw; best.rank = cur; best.tri = ltri; best.u = lu; best.v = lv;
                }
            }
            in_blas = false;
            ref = PICO_REF_DONE;
            return kTraceOk;
        }
        const uint32_t first = pico_leaf_first(ref), count = pico_leaf_count(ref);
        ref = PICO_REF_DONE;
        if (count == 0) return kTraceOk;
        if (in_blas) {
            for (uint32_t k = 0; k < count; ++k) {
                const uint32_t tri = first + k;
                float t, u, v;
                if (kCount) cnt->tris++;
                if (intersect_triangle(sc.tris + tri, qox, qoy, qoz, qdx, qdy, qdz, t, u, v)) {
                    const bool better = kOrder == kReferenceOrder ? t < lt : (t < lt || (t == lt && tri < ltri));
                    if (better) {
                        lt = t; ltri = tri; lu = u; lv = v;
                    }
                }
            }
            return kTraceOk;
        }
        // TLAS leaf: search instance `first`; the rest of the leaf waits on the stack.
        if (count > 1) {
            if (sp >= kTraceStack) return kTraceStackOverflow;
            stack[sp++] = StackEntry{pico_leaf_ref(first + 1, count - 1), -kInf};
        }
        if (kCount) cnt->insts++;
        const float4* ip = reinterpret_cast<const float4*>(sc.insts + first);
        const float4 i0 = __ldg(ip), i1 = __ldg(ip + 1), i2 = __ldg(ip + 2);
        const float4 rl = __ldg(ip + 7), rh = __ldg(ip + 8);
        qox = row4(i0, ox, oy, oz, ow); qoy = row4(i1, ox, oy, oz, ow); qoz = row4(i2, ox, oy, oz, ow);
        qdx = row3(i0, dx, dy, dz); qdy = row3(i1, dx, dy, dz); qdz = row3(i2, dx, dy, dz);
        qix = div(1.0f, qdx); qiy = div(1.0f, qdy); qiz = div(1.0f, qdz);
        // A triangle of this instance at object-space t lies at world distance
        // t * |D| up to float error (relative ~1e-6, absolute ~1e-7 |O|); the bound
        // adds 0.1 % and 1e-4 (|O| + 1), far above that error, so it never cuts a
        // triangle that could beat or tie the best world distance.
        gl = kOrder == kNearFirst ? (best.t * 1.001f + omag) * inv_len : kInf;
        bool h;
        const float tm = slab(rl.x, rh.x, rl.y, rh.y, rl.z, rh.z, qox, qoy, qoz, qix, qiy, qiz, h);
        if (!(h && tm < kInf) || (kOrder == kNearFirst && !(tm <= gl))) return kTraceOk;
        if (sp >= kTraceStack) return kTraceStackOverflow;
        stack[sp++] = StackEntry{PICO_REF_END_BLAS, -kInf};
        in_blas = true;
        cur = first;
        lt = kInf; ltri = kNoHit;
        ref = __float_as_uint(rl.w);
        return kTraceOk;
    }
};

// Runs one ray to completion.
template <bool kCount, int kOrder>
__device__ __forceinline__ int trace_closest(const SceneView& sc, const float4 o, const float4 d, TraceHit& best,
                                             TraceCounters* cnt)
{
    Traversal<kCount, kOrder> tr;
    StackEntry stack[kTraceStack];
    tr.start(sc, o, d);
    for (uint32_t iter = 0; iter < kTraceMaxIter; ++iter) {
        const int s = tr.step(sc, stack, cnt);
        if (s == kTraceDone) {
            best = tr.best;
            return kTraceOk;
        }
        if (s != kTraceOk) {
            best = tr.best;
            return s;
        }
    }
    best = tr.best;
    return kTraceIterLimit;
}

}  // namespace pico
