// Device-resident scene layout shared by the host builder and the kernels.
//
// Everything the traversal touches is read-only after upload and sized to
// stay resident in the 129 MB L2 for the scenes this library targets (a
// 4096-instance field of a 5120-triangle mesh is about 1 MB).
//
//   GpuNode      64 B, one cache-line pair: the two CHILD boxes of a binary
//                node plus the two child references (Aila-Laine layout), in
//                depth-first pre-order so a left child follows its parent.
//   GpuTri       48 B: the three original vertex positions (not edges: the
//                reference's barycentric interpolation of the hit position
//                needs v1 and v2 bit-exactly) and the mesh triangle index.
//   GpuInstance  144 B: inverse and forward transform rows, the BLAS root box
//                and root reference, the original instance index.
//
// A child reference is either an inner node index (bit 31 clear) or a leaf
// (bit 31 set) holding `count` (1..31) consecutive items starting at `first`:
// triangles in a BLAS, instance slots in the TLAS.  Items are stored in the
// reference's depth-first leaf order, so an item's position is its rank in the
// order the reference's recursive walk would meet it; equal-distance hits are
// resolved to the lower rank, which reproduces the reference's first-found rule.
#pragma once

#include <stdint.h>

#define PICO_REF_LEAF 0x80000000u
#define PICO_REF_EMPTY 0x80000000u          // a leaf with no items (absent child)
#define PICO_REF_END_BLAS 0xffffffffu       // stack sentinel: leave object space
#define PICO_REF_DONE 0xfffffffeu           // traversal finished
#define PICO_REF_SPHERE 0xfffffffdu         // BLAS root of the implicit radius-0.5 sphere
#define PICO_REF_CUBE 0xfffffffcu           // BLAS root of the implicit [-0.5, 0.5]^3 cube
#define PICO_LEAF_MAX 31u
#define PICO_FIRST_MAX ((1u << 26) - 2u)

#ifdef __CUDACC__
#define PICO_HD __host__ __device__ __forceinline__
#else
#define PICO_HD inline
#endif

PICO_HD uint32_t pico_leaf_ref(uint32_t first, uint32_t count) { return PICO_REF_LEAF | (first << 5) | count; }
PICO_HD bool pico_is_leaf(uint32_t ref) { return (ref & PICO_REF_LEAF) != 0u; }
PICO_HD uint32_t pico_leaf_first(uint32_t ref) { return (ref & 0x7fffffffu) >> 5; }
PICO_HD uint32_t pico_leaf_count(uint32_t ref) { return ref & 31u; }

struct alignas(16) GpuNode {
    float c0lox, c0hix, c0loy, c0hiy;
    float c1lox, c1hix, c1loy, c1hiy;
    float c0loz, c0hiz, c1loz, c1hiz;
    uint32_t ref0, ref1, pad0, pad1;
};
static_assert(sizeof(GpuNode) == 64, "node is one 64-byte record");

struct alignas(16) GpuTri {
    float v0x, v0y, v0z; uint32_t prim;
    float v1x, v1y, v1z; uint32_t mesh_tri_base;
    float v2x, v2y, v2z; uint32_t pad;
};
static_assert(sizeof(GpuTri) == 48, "triangle is 48 bytes");

// Per-triangle shading data: the three vertex normals.
struct alignas(16) GpuTriShade {
    float n0x, n0y, n0z, pad0;
    float n1x, n1y, n1z, pad1;
    float n2x, n2y, n2z, pad2;
};

struct alignas(16) GpuInstance {
    float inv[3][4];      // rows 0..2 of the inverse transform: inv[r][c] = Inverse[c][r]
    float fwd[4][4];      // rows 0..3 of the transform: fwd[r][c] = Transform[c][r]
    float root_lo[3]; uint32_t root_ref;
    float root_hi[3]; uint32_t inst_id;
};
static_assert(sizeof(GpuInstance) == 144, "instance is 144 bytes");

// Per-instance shading record, indexed by the original instance index.
struct alignas(16) GpuInstanceShade {
    uint32_t bsdf, material, mesh, pad;
};

// Constant material with its reflectance precomputed as
// |specular| / (|specular| + |diffuse|) (Core/MaterialManager.hpp:40-45).
struct alignas(16) GpuMaterial {
    float diffuse[3], reflectance;
    float specular[3], roughness;
    float emissive[3], ior;   // index of refraction of a transparent material
};

// One NEE light: the instance and its triangle alias table, or an implicit shape.
struct alignas(16) GpuLight {
    uint32_t inst;        // original instance index
    uint32_t tri_base;    // first entry in the light-triangle arrays
    uint32_t ntris;
    uint32_t shape;       // pico_shape of the light's mesh
};

// What a kernel needs to walk the scene.
struct SceneView {
    const GpuNode* nodes;
    const GpuTri* tris;
    const GpuTriShade* tri_shade;
    const GpuInstance* insts;          // indexed by TLAS rank
    const uint32_t* tlas_items;         // TLAS leaf item -> instance rank
    const GpuInstanceShade* inst_shade; // indexed by original instance index
    const uint32_t* inst_rank;          // original instance index -> TLAS rank
    const GpuMaterial* materials;
    const GpuLight* lights;
    const float* light_alias_weight;    // per light triangle
    const uint32_t* light_alias_index;  // per light triangle (alias, local index)
    const float* light_positions;       // per light triangle: v0, v1, v2 (9 floats)
    const float* light_tri_geo;         // per light triangle: world unit normal, area pdf (4 floats)
    const uint32_t* light_of_inst;      // original instance index -> light index, or ~0u
    const float* light_pick;            // physical estimator's light pick over nlights + use_sun slots: cdf, then pdf
    uint32_t nlights;
    uint32_t tlas_root_ref;             // the reference's TLAS boxes
    float tlas_lo[3], tlas_hi[3];
    uint32_t tlas_fast_root_ref;        // same topology, boxes refitted to the transformed vertices
    float tlas_fast_lo[3], tlas_fast_hi[3];
    float sky[3];
    uint32_t ninstances;
    uint32_t finite_boxes;              // every non-empty child box and both TLAS root boxes are finite
    uint32_t has_implicit;              // some instance is an implicit sphere or cube
    uint32_t sky_kind, sky_w, sky_h;    // pico_sky_kind; texels per row / column (of a face)
    const void* sky_pixels;             // uchar4 cube faces or float4 equirectangular texels
    uint32_t use_sun;
    float sun_dir[3], sun_col[3];
    // traversal bounds of the launching context (pico_gpu_set_traversal_limits):
    // iterations of one walk, and entries of its stack in use (at most the 96 it has)
    uint32_t max_iterations;
    uint32_t stack_entries;
    uint32_t watertight;                // the launching context's triangle test is the watertight one
    // per NEE light its widened world box (lo x, y, z, 0, hi x, y, z, 0): no hit on
    // the light lies outside it.  light_bounds: every light has one (else none is used).
    const float* light_boxes;
    uint32_t light_bounds;
};
