/*
 * Oracle (test infrastructure only): the reference's acceleration structures.
 *
 *   SAH build      Core/BVH.cpp:73-107 (BVHFactory::split_primitives) and
 *                  Core/BVH.cpp:126-197 (SAH_parition_Scheme::partition),
 *                  max depth 32 (Core/BVH.hpp:125-129)
 *   BLAS input     Core/LowerLevelMeshBVH.cpp:48-64 (per-triangle bounds, value = triangle)
 *   TLAS input     Core/UpperLevelBVH.cpp:27-57 (mesh AABB * transform, value = instance)
 *   traversal      Core/BVH.cpp:16-63 (recursive, children 0 then 1, strict <)
 *   slab test      Core/AABB.cpp:108-147
 *   transform_ray  Core/AABB.cpp:43-52
 *   ray/triangle   Core/LowerLevelMeshBVH.cpp:165-207 (Moeller-Trumbore, eps 1e-7)
 *   interpolation  Core/LowerLevelMeshBVH.cpp:134-163
 *   world space    Core/UpperLevelBVH.cpp:59-80
 *
 * std::partition is restated as the two-ended swap loop that libstdc++ runs
 * for bidirectional/random-access iterators (bits/stl_algo.h __partition),
 * because the leaf order it leaves behind decides the reference's topology.
 */
#include "po_internal.h"

#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ AABB ops */
static po_aabb aabb_empty(void)
{
    po_aabb b;
    b.mn = v4(INFINITY, INFINITY, INFINITY, INFINITY);
    b.mx = v4(-INFINITY, -INFINITY, -INFINITY, -INFINITY);
    return b;
}
static void aabb_union(po_aabb* a, const po_aabb* o)   /* AABB::union_of, AABB.cpp:180-184 */
{
    a->mn = v4_min(a->mn, o->mn);
    a->mx = v4_max(a->mx, o->mx);
}
static void aabb_add_point(po_aabb* a, po_v4 p)         /* AABB::add_point, AABB.cpp:174-178 */
{
    a->mn = v4_min(a->mn, p);
    a->mx = v4_max(a->mx, p);
}
static po_v4 aabb_center(const po_aabb* a)              /* AABB.hpp:122-123 */
{
    return v4_add(a->mn, v4_scale(v4_sub(a->mx, a->mn), 0.5f));
}
static po_v3 aabb_sides(const po_aabb* a)               /* AABB.hpp:125-128 */
{
    po_v4 d = v4_sub(a->mx, a->mn);
    return v3(fabsf(d.x), fabsf(d.y), fabsf(d.z));
}
static float aabb_area(const po_aabb* a)                /* AABB.hpp:130-135 */
{
    po_v3 s = aabb_sides(a);
    return 2.0f * (((s.x * s.y) + (s.x * s.z)) + (s.y * s.z));
}
static po_v3 aabb_offset(const po_aabb* a, po_v4 p)     /* AABB::get_offset, AABB.cpp:194-201 */
{
    po_v3 o = v3(p.x - a->mn.x, p.y - a->mn.y, p.z - a->mn.z);
    if (a->mx.x > a->mn.x) o.x /= a->mx.x - a->mn.x;
    if (a->mx.y > a->mn.y) o.y /= a->mx.y - a->mn.y;
    if (a->mx.z > a->mn.z) o.z /= a->mx.z - a->mn.z;
    return o;
}
static uint32_t max_component(po_v3 v)                  /* AABB.cpp:31-41 */
{
    po_v3 a = v3(fabsf(v.x), fabsf(v.y), fabsf(v.z));
    if ((a.x >= a.y) && (a.x >= a.z)) return 0;
    if ((a.y >= a.x) && (a.y >= a.z)) return 1;
    return 2;
}
static float comp3(po_v3 v, uint32_t i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

/* AABB::operator*(mat4) (AABB.cpp:253-270): transform the 8 corners, divide by w,
 * min/max starting from +-1e7. */
static po_aabb aabb_transform(const po_aabb* a, const po_m4* m)
{
    const po_v4 mn = a->mn, mx = a->mx;
    po_v4 c[8] = {
        mn,
        v4(mn.x, mn.y, mx.z, 1.0f), v4(mx.x, mn.y, mx.z, 1.0f), v4(mx.x, mn.y, mn.z, 1.0f),
        v4(mn.x, mx.y, mn.z, 1.0f), v4(mn.x, mx.y, mx.z, 1.0f), mx, v4(mx.x, mx.y, mn.z, 1.0f)};
    po_v4 lo = v4(10000000.0f, 10000000.0f, 10000000.0f, 10000000.0f);
    po_v4 hi = v4(-10000000.0f, -10000000.0f, -10000000.0f, -10000000.0f);
    for (int i = 0; i < 8; ++i) {
        po_v4 p = m4_mul_v4(m, c[i]);
        const float w = p.w;
        p = v4(p.x / w, p.y / w, p.z / w, p.w / w);
        lo = v4_min(lo, p);
        hi = v4_max(hi, p);
    }
    po_aabb r = {lo, hi};
    return r;
}

/* AABB::intersection_distance (AABB.cpp:108-147) with its exact NaN behaviour:
 * min_max is `a > b ? {b,a} : {a,b}`, then std::max / std::min selects. */
float po_slab(const po_aabb* b, po_v4 o, po_v3 inv)
{
    const float t1 = (b->mn.x - o.x) * inv.x, t2 = (b->mx.x - o.x) * inv.x;
    const float t3 = (b->mn.y - o.y) * inv.y, t4 = (b->mx.y - o.y) * inv.y;
    const float t5 = (b->mn.z - o.z) * inv.z, t6 = (b->mx.z - o.z) * inv.z;
    float a1 = t1, b1 = t2, a2 = t3, b2 = t4, a3 = t5, b3 = t6;
    if (t1 > t2) { a1 = t2; b1 = t1; }
    if (t3 > t4) { a2 = t4; b2 = t3; }
    if (t5 > t6) { a3 = t6; b3 = t5; }
    const float tmin = f_max(f_max(a1, a2), a3);
    const float tmax = f_min(f_min(b1, b2), b3);
    if (tmax < 0 || tmin > tmax) return INFINITY;
    return tmin;
}

/* ----------------------------------------------------------- SAH build */
typedef struct {
    po_node* nodes; uint32_t nnodes, cap;
    uint32_t* leaf_values; uint32_t nvalues, vcap;
} builder;

static uint32_t add_node(builder* bd, const po_node* n)   /* BVH.hpp:157-163 */
{
    if (bd->nnodes == bd->cap) {
        bd->cap = bd->cap ? bd->cap * 2 : 64;
        bd->nodes = (po_node*)realloc(bd->nodes, sizeof(po_node) * bd->cap);
    }
    bd->nodes[bd->nnodes] = *n;
    return bd->nnodes++;
}

static uint32_t bucket_of(const po_aabb* cb, uint32_t axis, const po_bounded* it)
{
    uint32_t b = (uint32_t)(12.0f * comp3(aabb_offset(cb, aabb_center(&it->b)), axis));
    if (b == 12) b = 11;
    return b;
}

/* libstdc++ __partition for bidirectional iterators. */
static po_bounded* partition_by_bucket(po_bounded* first, po_bounded* last,
                                       const po_aabb* cb, uint32_t axis, uint32_t split)
{
    for (;;) {
        for (;;) {
            if (first == last) return first;
            if (bucket_of(cb, axis, first) <= split) ++first; else break;
        }
        --last;
        for (;;) {
            if (first == last) return first;
            if (!(bucket_of(cb, axis, last) <= split)) --last; else break;
        }
        po_bounded tmp = *first; *first = *last; *last = tmp;
        ++first;
    }
}

/* SAH_parition_Scheme::partition (BVH.cpp:126-197). */
static po_bounded* sah_partition(po_bounded* start, po_bounded* end)
{
    if (start == end) return end;
    po_aabb cb = aabb_empty();
    for (po_bounded* it = start; it != end; ++it) aabb_add_point(&cb, aabb_center(&it->b));
    const uint32_t axis = max_component(aabb_sides(&cb));

    uint32_t count[12];
    po_aabb bounds[12];
    for (int i = 0; i < 12; ++i) { count[i] = 0; bounds[i] = aabb_empty(); }
    for (po_bounded* it = start; it < end; ++it) {
        const uint32_t b = bucket_of(&cb, axis, it);
        count[b]++;
        aabb_union(&bounds[b], &it->b);
    }
    const float leaf_cost = (float)(end - start);
    float cost[11];
    for (uint32_t i = 0; i < 11; ++i) {
        po_aabb b0 = aabb_empty(), b1 = aabb_empty();
        uint32_t c0 = 0, c1 = 0;
        for (uint32_t j = 0; j <= i; ++j) { aabb_union(&b0, &bounds[j]); c0 += count[j]; }
        for (uint32_t j = i + 1; j < 12; ++j) { aabb_union(&b1, &bounds[j]); c1 += count[j]; }
        cost[i] = .125f + ((float)c0 * aabb_area(&b0) + (float)c1 * aabb_area(&b1)) /
                              (leaf_cost * aabb_area(&cb));
    }
    uint32_t best = 0;                       /* std::min_element: first strict minimum */
    for (uint32_t i = 1; i < 11; ++i)
        if (cost[i] < cost[best]) best = i;
    const float min_cost = cost[best];
    if (leaf_cost > 2 || min_cost < leaf_cost)
        return partition_by_bucket(start, end, &cb, axis, best);
    return end;
}

/* BVHFactory::split_primitives (BVH.cpp:73-107). */
static uint32_t split_primitives(builder* bd, po_bounded* start, po_bounded* end, uint32_t depth)
{
    if (start == end) return PO_INVALID;
    po_node n;
    memset(&n, 0, sizeof n);
    n.box = aabb_empty();
    for (po_bounded* it = start; it != end; ++it) aabb_union(&n.box, &it->b);

    po_bounded* pivot = sah_partition(start, end);
    if (depth == 0 || pivot == end || (end - start) == 2) {
        n.first = bd->nvalues;
        n.count = (uint32_t)(end - start);
        for (po_bounded* it = start; it != end; ++it) {
            if (bd->nvalues == bd->vcap) {
                bd->vcap = bd->vcap ? bd->vcap * 2 : 64;
                bd->leaf_values = (uint32_t*)realloc(bd->leaf_values, sizeof(uint32_t) * bd->vcap);
            }
            bd->leaf_values[bd->nvalues++] = it->value;
        }
        n.child[0] = n.child[1] = PO_INVALID;
        return add_node(bd, &n);
    }
    n.child[0] = split_primitives(bd, start, pivot, depth - 1);
    n.child[1] = split_primitives(bd, pivot, end, depth - 1);
    return add_node(bd, &n);
}

static void build_bvh(po_bvh* out, po_bounded* items, uint32_t n)
{
    builder bd;
    memset(&bd, 0, sizeof bd);
    out->root = split_primitives(&bd, items, items + n, 32u);
    out->nodes = bd.nodes;
    out->nnodes = bd.nnodes;
    out->values = bd.leaf_values;
    out->nvalues = bd.nvalues;
}

/* glm compute_inverse<4,4> (func_matrix.inl:297-355), same operation order. */
void po_mat4_inverse(const float* mf, float* out)
{
    float m[4][4];
    memcpy(m, mf, sizeof m);
    const float c00 = m[2][2] * m[3][3] - m[3][2] * m[2][3];
    const float c02 = m[1][2] * m[3][3] - m[3][2] * m[1][3];
    const float c03 = m[1][2] * m[2][3] - m[2][2] * m[1][3];
    const float c04 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    const float c06 = m[1][1] * m[3][3] - m[3][1] * m[1][3];
    const float c07 = m[1][1] * m[2][3] - m[2][1] * m[1][3];
    const float c08 = m[2][1] * m[3][2] - m[3][1] * m[2][2];
    const float c10 = m[1][1] * m[3][2] - m[3][1] * m[1][2];
    const float c11 = m[1][1] * m[2][2] - m[2][1] * m[1][2];
    const float c12 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    const float c14 = m[1][0] * m[3][3] - m[3][0] * m[1][3];
    const float c15 = m[1][0] * m[2][3] - m[2][0] * m[1][3];
    const float c16 = m[2][0] * m[3][2] - m[3][0] * m[2][2];
    const float c18 = m[1][0] * m[3][2] - m[3][0] * m[1][2];
    const float c19 = m[1][0] * m[2][2] - m[2][0] * m[1][2];
    const float c20 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    const float c22 = m[1][0] * m[3][1] - m[3][0] * m[1][1];
    const float c23 = m[1][0] * m[2][1] - m[2][0] * m[1][1];
    const float f0[4] = {c00, c00, c02, c03}, f1[4] = {c04, c04, c06, c07};
    const float f2[4] = {c08, c08, c10, c11}, f3[4] = {c12, c12, c14, c15};
    const float f4[4] = {c16, c16, c18, c19}, f5[4] = {c20, c20, c22, c23};
    const float v0[4] = {m[1][0], m[0][0], m[0][0], m[0][0]};
    const float v1[4] = {m[1][1], m[0][1], m[0][1], m[0][1]};
    const float v2[4] = {m[1][2], m[0][2], m[0][2], m[0][2]};
    const float v3_[4] = {m[1][3], m[0][3], m[0][3], m[0][3]};
    const float sa[4] = {1, -1, 1, -1}, sb[4] = {-1, 1, -1, 1};
    float inv[4][4];
    for (int i = 0; i < 4; ++i) {
        inv[0][i] = ((v1[i] * f0[i] - v2[i] * f1[i]) + v3_[i] * f2[i]) * sa[i];
        inv[1][i] = ((v0[i] * f0[i] - v2[i] * f3[i]) + v3_[i] * f4[i]) * sb[i];
        inv[2][i] = ((v0[i] * f1[i] - v1[i] * f3[i]) + v3_[i] * f5[i]) * sa[i];
        inv[3][i] = ((v0[i] * f2[i] - v1[i] * f4[i]) + v2[i] * f5[i]) * sb[i];
    }
    const float d0 = m[0][0] * inv[0][0], d1 = m[0][1] * inv[1][0];
    const float d2 = m[0][2] * inv[2][0], d3 = m[0][3] * inv[3][0];
    const float det = (d0 + d1) + (d2 + d3);
    const float one_over = 1.0f / det;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = inv[c][r] * one_over;
}

/* ------------------------------------------------------------ scene setup */
po_scene* po_scene_create(const po_mesh_desc* meshes, uint32_t nmeshes,
                          const po_instance_desc* instances, uint32_t ninstances,
                          const po_material* materials, uint32_t nmaterials)
{
    po_scene* s = (po_scene*)calloc(1, sizeof(po_scene));
    s->nmeshes = nmeshes;
    s->meshes = (po_mesh*)calloc(nmeshes, sizeof(po_mesh));
    for (uint32_t mi = 0; mi < nmeshes; ++mi) {
        const po_mesh_desc* d = &meshes[mi];
        po_mesh* m = &s->meshes[mi];
        m->desc = *d;
        if (d->shape != PO_SHAPE_TRIANGLES) {
            /* LowerLevelSphereBVH::get_bounds (radius 0.5) and LowerLevelCube's m_box are both
             * [-0.5, 0.5]^3 with w = 1 (LowerLevelImplicitShapesBVH.cpp:54-57, 66-68) */
            m->desc.ntris = 0;
            m->aabb.mn = v4(-0.5f, -0.5f, -0.5f, 1.0f);
            m->aabb.mx = v4(0.5f, 0.5f, 0.5f, 1.0f);
            continue;
        }
        po_bounded* items = (po_bounded*)malloc(sizeof(po_bounded) * (d->ntris ? d->ntris : 1));
        for (uint32_t t = 0; t < d->ntris; ++t) {            /* LowerLevelMeshBVH.cpp:48-64 */
            po_v3 mn = v3(INFINITY, INFINITY, INFINITY), mx = v3(-INFINITY, -INFINITY, -INFINITY);
            for (int k = 0; k < 3; ++k) {
                const float* p = d->positions + 3 * d->indices[3 * t + k];
                mn = v3_min(mn, v3(p[0], p[1], p[2]));
            }
            for (int k = 0; k < 3; ++k) {
                const float* p = d->positions + 3 * d->indices[3 * t + k];
                mx = v3_max(mx, v3(p[0], p[1], p[2]));
            }
            items[t].b.mn = v4_of3(mn, 1.0f);
            items[t].b.mx = v4_of3(mx, 1.0f);
            items[t].value = t;
        }
        build_bvh(&m->bvh, items, d->ntris);
        free(items);
        m->aabb.mn = v4(d->aabb_min[0], d->aabb_min[1], d->aabb_min[2], 1.0f);
        m->aabb.mx = v4(d->aabb_max[0], d->aabb_max[1], d->aabb_max[2], 1.0f);
    }
    s->ninstances = ninstances;
    s->instances = (po_instance*)calloc(ninstances ? ninstances : 1, sizeof(po_instance));
    po_bounded* items = (po_bounded*)malloc(sizeof(po_bounded) * (ninstances ? ninstances : 1));
    s->nlights = 0;
    s->lights = (uint32_t*)calloc(ninstances ? ninstances : 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < ninstances; ++i) {
        po_instance* in = &s->instances[i];
        in->mesh = instances[i].mesh;
        in->bsdf = instances[i].bsdf;
        in->material = instances[i].material;
        memcpy(in->T.m, instances[i].transform, sizeof(float) * 16);
        po_mat4_inverse(instances[i].transform, &in->Tinv.m[0][0]);
        items[i].b = aabb_transform(&s->meshes[in->mesh].aabb, &in->T);   /* UpperLevelBVH.cpp:32-35 */
        items[i].value = i;
        if (in->bsdf == PO_LIGHT) s->lights[s->nlights++] = i;          /* Scene.cpp:406-412 */
    }
    build_bvh(&s->tlas, items, ninstances);
    free(items);
    s->nmaterials = nmaterials;
    s->materials = (po_material*)calloc(nmaterials ? nmaterials : 1, sizeof(po_material));
    if (nmaterials) memcpy(s->materials, materials, sizeof(po_material) * nmaterials);
    po_scene_build_light_tables(s);
    return s;
}

void po_scene_destroy(po_scene* s)
{
    if (!s) return;
    for (uint32_t i = 0; i < s->nmeshes; ++i) {
        free(s->meshes[i].bvh.nodes);
        free(s->meshes[i].bvh.values);
        free(s->meshes[i].alias_weight);
        free(s->meshes[i].alias_index);
    }
    free(s->meshes);
    free(s->sky_pixels);
    free(s->instances);
    free(s->tlas.nodes);
    free(s->tlas.values);
    free(s->lights);
    free(s->materials);
    free(s);
}

static void dump_bvh(const po_bvh* b, float* boxes, uint32_t* links, uint32_t* values)
{
    for (uint32_t i = 0; i < b->nnodes; ++i) {
        const po_node* n = &b->nodes[i];
        if (boxes) {
            float* o = boxes + 6 * i;
            o[0] = n->box.mn.x; o[1] = n->box.mn.y; o[2] = n->box.mn.z;
            o[3] = n->box.mx.x; o[4] = n->box.mx.y; o[5] = n->box.mx.z;
        }
        if (links) {
            uint32_t* l = links + 4 * i;
            l[0] = n->child[0]; l[1] = n->child[1]; l[2] = n->first; l[3] = n->count;
        }
    }
    if (values) memcpy(values, b->values, sizeof(uint32_t) * b->nvalues);
}
uint32_t po_blas_node_count(const po_scene* s, uint32_t mesh) { return s->meshes[mesh].bvh.nnodes; }
uint32_t po_tlas_node_count(const po_scene* s) { return s->tlas.nnodes; }
void po_blas_nodes(const po_scene* s, uint32_t mesh, float* boxes, uint32_t* links, uint32_t* values)
{
    dump_bvh(&s->meshes[mesh].bvh, boxes, links, values);
}
void po_tlas_nodes(const po_scene* s, float* boxes, uint32_t* links, uint32_t* values)
{
    dump_bvh(&s->tlas, boxes, links, values);
}
void po_instance_matrices(const po_scene* s, uint32_t inst, float* transform, float* inverse)
{
    if (transform) memcpy(transform, s->instances[inst].T.m, sizeof(float) * 16);
    if (inverse) memcpy(inverse, s->instances[inst].Tinv.m, sizeof(float) * 16);
}

/* ------------------------------------------------------------ traversal */
typedef struct {
    po_v4 org; po_v3 dir, inv;
} tray;

typedef struct {
    float t; uint32_t prim; float u, v;
} blas_best;

/* Mesh_Intersector::intersects (LowerLevelMeshBVH.cpp:165-207); returns 1 on a hit. */
static int intersect_triangle(const po_mesh_desc* m, uint32_t prim, const tray* r,
                              float* t_out, float* u_out, float* v_out)
{
    const float EPS = 0.0000001f;
    const float* p0 = m->positions + 3 * m->indices[prim * 3];
    const float* p1 = m->positions + 3 * m->indices[prim * 3 + 1];
    const float* p2 = m->positions + 3 * m->indices[prim * 3 + 2];
    const po_v3 v0 = v3(p0[0], p0[1], p0[2]), v1 = v3(p1[0], p1[1], p1[2]), v2 = v3(p2[0], p2[1], p2[2]);
    const po_v3 e1 = v3_sub(v1, v0), e2 = v3_sub(v2, v0);
    const po_v3 h = v3_cross(r->dir, e2);
    const float a = v3_dot(e1, h);
    if (a > -EPS && a < EPS) return 0;
    const float f = (float)(1.0 / (double)a);
    const po_v3 s = v3_sub(v3(r->org.x, r->org.y, r->org.z), v0);
    const float u = f * v3_dot(s, h);
    if (u < 0.0 || u > 1.0) return 0;
    const po_v3 q = v3_cross(s, e1);
    const float v = f * v3_dot(r->dir, q);
    if (v < 0.0 || u + v > 1.0) return 0;
    const float t = f * v3_dot(e2, q);
    if (t > EPS) { *t_out = t; *u_out = u; *v_out = v; return 1; }
    return 0;
}

/* interpolate_fragment (LowerLevelMeshBVH.cpp:134-163). */
void po_interpolate(const po_mesh_desc* m, uint32_t prim, float u, float v,
                    po_v4* pos, po_v3* nrm, po_v2* uv)
{
    const uint32_t i0 = m->indices[prim * 3], i1 = m->indices[prim * 3 + 1], i2 = m->indices[prim * 3 + 2];
    const float w = (1.0f - v) - u;
    const float* a = m->positions + 3 * i0; const float* b = m->positions + 3 * i1;
    const float* c = m->positions + 3 * i2;
    po_v3 P = v3_add(v3_add(v3_scale(v3(a[0], a[1], a[2]), w), v3_scale(v3(b[0], b[1], b[2]), u)),
                     v3_scale(v3(c[0], c[1], c[2]), v));
    *pos = v4_of3(P, 1.0f);
    const float* na = m->normals + 3 * i0; const float* nb = m->normals + 3 * i1;
    const float* nc = m->normals + 3 * i2;
    po_v3 N = v3_add(v3_add(v3_scale(v3(na[0], na[1], na[2]), w), v3_scale(v3(nb[0], nb[1], nb[2]), u)),
                     v3_scale(v3(nc[0], nc[1], nc[2]), v));
    *nrm = v3_normalize(N);
    if (m->uvs) {
        const float* ua = m->uvs + 2 * i0; const float* ub = m->uvs + 2 * i1; const float* uc = m->uvs + 2 * i2;
        uv->x = ((ua[0] * w) + (ub[0] * u)) + (uc[0] * v);
        uv->y = ((ua[1] * w) + (ub[1] * u)) + (uc[1] * v);
    } else {
        uv->x = ((0.0f * w) + (0.0f * u)) + (0.0f * v);
        uv->y = uv->x;
    }
}

typedef struct { uint64_t nodes, tris, insts; } visit_stats;

/* BVH<T,2>::get_closest_intersections over a BLAS (BVH.cpp:27-63). */
static void blas_walk(const po_mesh* m, uint32_t ni, const tray* r, blas_best* best, visit_stats* st)
{
    const po_node* n = &m->bvh.nodes[ni];
    if (st) st->nodes++;
    if (po_slab(&n->box, r->org, r->inv) < best->t) {
        if (n->count) {
            for (uint32_t k = 0; k < n->count; ++k) {
                const uint32_t prim = m->bvh.values[n->first + k];
                float t = INFINITY, u, v;
                if (st) st->tris++;
                if (intersect_triangle(&m->desc, prim, r, &t, &u, &v) && t < best->t) {
                    best->t = t; best->prim = prim; best->u = u; best->v = v;
                }
            }
        } else {
            for (int c = 0; c < 2; ++c)
                if (n->child[c] != PO_INVALID) blas_walk(m, n->child[c], r, best, st);
        }
    }
}

typedef struct {
    float t; uint32_t inst, prim; float u, v; po_v4 pos; po_v3 nrm; po_v2 uv;
} tlas_best;

/* LowerLevelSphereBVH::calculate_intersection (radius 0.5, LowerLevelImplicitShapesBVH.cpp:24-52)
 * and LowerLevelCube::calculate_intersection (:71-91): object-space hit position, normal and uv. */
static int intersect_implicit(uint32_t shape, const tray* r, po_v4* P, po_v3* N, po_v2* uv, float* t_out)
{
    if (shape == PO_SHAPE_SPHERE) {
        const float radius = 0.5f;
        const po_v3 m = v3(r->org.x, r->org.y, r->org.z);
        const float b = v3_dot(m, r->dir);
        const float c = v3_dot(m, m) - radius * radius;
        if (c > 0.0f && b > 0.0f) return 0;
        const float discr = b * b - c;
        if (discr < 0.0f) return 0;
        float t = (float)(-(double)b - sqrt((double)discr));
        if (t < 0.0f) t = 0.0f;
        *P = v4(r->org.x + t * r->dir.x, r->org.y + t * r->dir.y, r->org.z + t * r->dir.z, r->org.w + t * 1.0f);
        P->w = 1.0f;
        *N = v3_normalize(v3(P->x, P->y, P->z));
        uv->x = (float)(atan2((double)N->x, (double)N->z) / (2.0f * 3.14159265358979323846) + 0.5f);
        uv->y = N->y * 0.5f + 0.5f;
        *t_out = t;
        return 1;
    }
    /* the cube: AABB::intersection_distance of [-0.5, 0.5]^3; the normal is the sign of the
     * largest |component| of the hit point (maximum_component_index, AABB.cpp:31-41) */
    po_aabb box;
    box.mn = v4(-0.5f, -0.5f, -0.5f, 1.0f);
    box.mx = v4(0.5f, 0.5f, 0.5f, 1.0f);
    const float t = po_slab(&box, r->org, r->inv);
    if (t == INFINITY) return 0;
    *P = v4(r->org.x + r->dir.x * t, r->org.y + r->dir.y * t, r->org.z + r->dir.z * t, r->org.w + 1.0f);
    P->w = 1.0f;
    uv->x = 0.0f; uv->y = 0.0f;
    const uint32_t k = max_component(v3(P->x, P->y, P->z));
    const float pk = k == 0 ? P->x : (k == 1 ? P->y : P->z);
    const float sgn = (float)((0.0f < pk) - (pk < 0.0f));
    *N = v3(0.0f, 0.0f, 0.0f);
    if (k == 0) N->x = 1.0f * sgn; else if (k == 1) N->y = 1.0f * sgn; else N->z = 1.0f * sgn;
    *t_out = t;
    return 1;
}

/* lower_level_intersector::intersects (UpperLevelBVH.cpp:59-80). */
static int intersect_instance(const po_scene* s, uint32_t inst, const tray* wr, tlas_best* out,
                              visit_stats* st)
{
    const po_instance* in = &s->instances[inst];
    const po_mesh* m = &s->meshes[in->mesh];
    tray r;                                                     /* transform_ray, AABB.cpp:43-52 */
    r.org = m4_mul_v4(&in->Tinv, wr->org);
    r.dir = m4_mul_v3(&in->Tinv, wr->dir);
    r.inv = v3(1.0f / r.dir.x, 1.0f / r.dir.y, 1.0f / r.dir.z);
    if (st) st->insts++;
    if (m->desc.shape != PO_SHAPE_TRIANGLES) {
        po_v4 P; po_v3 N; po_v2 uv; float t;
        if (!intersect_implicit(m->desc.shape, &r, &P, &N, &uv, &t)) return 0;
        out->pos = m4_mul_v4(&in->T, P);
        out->nrm = v3_normalize(m4_mul_v3(&in->T, N));
        out->t = v4_length(v4_sub(out->pos, wr->org));
        out->inst = inst; out->prim = PO_IMPLICIT_PRIM; out->u = t; out->v = 0.0f; out->uv = uv;
        return 1;
    }
    blas_best b = {INFINITY, PO_INVALID, 0, 0};
    if (m->bvh.nnodes) blas_walk(m, m->bvh.root, &r, &b, st);
    if (b.t == INFINITY) return 0;                              /* BVH.cpp:16-25 */
    po_v4 P; po_v3 N; po_v2 uv;
    po_interpolate(&m->desc, b.prim, b.u, b.v, &P, &N, &uv);
    out->pos = m4_mul_v4(&in->T, P);
    out->nrm = v3_normalize(m4_mul_v3(&in->T, N));
    out->t = v4_length(v4_sub(out->pos, wr->org));
    out->inst = inst; out->prim = b.prim; out->u = b.u; out->v = b.v; out->uv = uv;
    return 1;
}

static void tlas_walk(const po_scene* s, uint32_t ni, const tray* r, tlas_best* best, visit_stats* st)
{
    const po_node* n = &s->tlas.nodes[ni];
    if (st) st->nodes++;
    if (po_slab(&n->box, r->org, r->inv) < best->t) {
        if (n->count) {
            for (uint32_t k = 0; k < n->count; ++k) {
                tlas_best cand;
                if (intersect_instance(s, s->tlas.values[n->first + k], r, &cand, st) && cand.t < best->t)
                    *best = cand;
            }
        } else {
            for (int c = 0; c < 2; ++c)
                if (n->child[c] != PO_INVALID) tlas_walk(s, n->child[c], r, best, st);
        }
    }
}

int po_closest_hit(const po_scene* s, po_v4 org, po_v3 dir, po_fragment* out, void* stats)
{
    tray r;
    r.org = org; r.dir = dir;
    r.inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);      /* BVH.cpp:19 */
    tlas_best b;
    memset(&b, 0, sizeof b);
    b.t = INFINITY; b.inst = PO_INVALID; b.prim = PO_INVALID;
    if (s->tlas.nnodes) tlas_walk(s, s->tlas.root, &r, &b, (visit_stats*)stats);
    if (out) {
        out->inst = b.inst; out->prim = b.prim; out->t = b.t; out->u = b.u; out->v = b.v;
        out->position[0] = b.pos.x; out->position[1] = b.pos.y;
        out->position[2] = b.pos.z; out->position[3] = b.pos.w;
        out->normal[0] = b.nrm.x; out->normal[1] = b.nrm.y; out->normal[2] = b.nrm.z;
        out->uv[0] = b.uv.x; out->uv[1] = b.uv.y;
    }
    return b.t != INFINITY;
}

static void trace_range(const po_scene* s, const po_ray* rays, po_hit* hits, size_t lo, size_t hi)
{
    for (size_t i = lo; i < hi; ++i) {
        const po_ray* r = &rays[i];
        po_fragment f;
        po_closest_hit(s, v4(r->org[0], r->org[1], r->org[2], r->org[3]),
                       v3(r->dir[0], r->dir[1], r->dir[2]), &f, NULL);
        hits[i].inst = f.inst; hits[i].prim = f.prim; hits[i].t = f.t;
        hits[i].u = f.u; hits[i].v = f.v;
        if (f.inst == PO_INVALID) { hits[i].t = INFINITY; hits[i].u = hits[i].v = 0.0f; }
    }
}

typedef struct { const po_scene* s; const po_ray* rays; po_hit* hits; size_t lo, hi; } trace_job;
static void trace_job_run(void* p)
{
    trace_job* j = (trace_job*)p;
    trace_range(j->s, j->rays, j->hits, j->lo, j->hi);
}

void po_trace(const po_scene* s, const po_ray* rays, uint32_t n, po_hit* hits, int nthreads)
{
    /* 64x64-ray tasks handed out round-robin, as the reference's Tiler does for pixels. */
    const size_t chunk = 4096;
    const size_t njobs = (n + chunk - 1) / chunk;
    trace_job* jobs = (trace_job*)malloc(sizeof(trace_job) * (njobs ? njobs : 1));
    for (size_t j = 0; j < njobs; ++j) {
        jobs[j].s = s; jobs[j].rays = rays; jobs[j].hits = hits;
        jobs[j].lo = j * chunk; jobs[j].hi = (j + 1) * chunk < n ? (j + 1) * chunk : n;
    }
    po_parallel_for(njobs, jobs, sizeof(trace_job), trace_job_run, nthreads);
    free(jobs);
}

void po_trace_fragments(const po_scene* s, const po_ray* rays, uint32_t n, po_fragment* out)
{
    for (uint32_t i = 0; i < n; ++i) {
        const po_ray* r = &rays[i];
        po_closest_hit(s, v4(r->org[0], r->org[1], r->org[2], r->org[3]),
                       v3(r->dir[0], r->dir[1], r->dir[2]), &out[i], NULL);
    }
}

void po_trace_stats(const po_scene* s, const po_ray* rays, uint32_t n, uint64_t* nodes,
                    uint64_t* tris, uint64_t* insts)
{
    visit_stats st = {0, 0, 0};
    for (uint32_t i = 0; i < n; ++i) {
        const po_ray* r = &rays[i];
        po_closest_hit(s, v4(r->org[0], r->org[1], r->org[2], r->org[3]),
                       v3(r->dir[0], r->dir[1], r->dir[2]), NULL, &st);
    }
    *nodes = st.nodes; *tris = st.tris; *insts = st.insts;
}
