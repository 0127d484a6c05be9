/* Oracle (test infrastructure only): internal types shared by the oracle sources. */
#ifndef PICO_ORACLE_INTERNAL_H
#define PICO_ORACLE_INTERNAL_H

#include "pico_oracle.h"
#include "po_math.h"

#include <stddef.h>

#define PO_INVALID 0xffffffffu

typedef struct { po_v4 mn, mx; } po_aabb;
typedef struct { po_aabb b; uint32_t value; } po_bounded;

/* BVH<T,2>::Node (Core/BVH.hpp:52-66); leaf values live in po_bvh::values. */
typedef struct {
    po_aabb box;
    uint32_t child[2];
    uint32_t first, count;
} po_node;

typedef struct {
    po_node* nodes; uint32_t nnodes;
    uint32_t* values; uint32_t nvalues;
    uint32_t root;
} po_bvh;

typedef struct {
    po_mesh_desc desc;
    po_bvh bvh;
    po_aabb aabb;
    /* light sampling data (LowerLevelMeshBVH.cpp:92-117), built for light meshes */
    float* alias_weight; uint32_t* alias_index; uint32_t alias_n;
} po_mesh;

typedef struct {
    uint32_t mesh, bsdf, material;
    po_m4 T, Tinv;
} po_instance;

struct po_scene {
    po_mesh* meshes; uint32_t nmeshes;
    po_instance* instances; uint32_t ninstances;
    po_bvh tlas;
    po_material* materials; uint32_t nmaterials;
    uint32_t* lights; uint32_t nlights;   /* instance indices, insertion order */
    po_sky sky;                           /* pixels point into sky_pixels (owned) */
    void* sky_pixels;
    float sky_rgb[3];
};

/* ImageCube::sample4 of the scene's sky (Core/Image.cpp:361-397). */
po_v4 po_sky_lookup(const po_scene* s, po_v3 d);

float po_slab(const po_aabb* b, po_v4 o, po_v3 inv);
void po_interpolate(const po_mesh_desc* m, uint32_t prim, float u, float v,
                    po_v4* pos, po_v3* nrm, po_v2* uv);
int po_closest_hit(const po_scene* s, po_v4 org, po_v3 dir, po_fragment* out, void* stats);
void po_scene_build_light_tables(po_scene* s);

/* Runs fn over `count` items of `stride` bytes on up to nthreads threads (<=0: all cores). */
void po_parallel_for(size_t count, void* items, size_t stride, void (*fn)(void*), int nthreads);

#endif
