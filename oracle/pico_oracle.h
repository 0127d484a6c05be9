/*
 * pico_oracle — CPU restatement of the Pico reference's rendering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300
 * kernels: tests, the smoke entry and the CPU-baseline leg of the benchmark
 * call it; the product library never links or loads it.
 *
 * Each function restates the reference routine it names (file:line paths are
 * relative to the Pico source tree) with the same float operation order, so
 * that its results are bit-identical to the reference compiled with
 * -ffp-contract=off on the same machine.  That claim is pinned by golden
 * vectors produced by the reference itself (tests/golden).
 */
#ifndef PICO_ORACLE_H
#define PICO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BSRDF kinds: 0-4 numbered like Render::BSRDF_Type (Render/BSRDF.hpp:32-39), where
 * kBTDF is Transparent_BTDF; 5 Fresnel_BTDF (also kBTDF), 6 Specular_Delta_BRDF
 * (type kSpecular_BRDF). */
enum { PO_DIFFUSE = 0, PO_SPECULAR = 1, PO_DIELECTRIC = 2, PO_BTDF = 3, PO_LIGHT = 4, PO_FRESNEL = 5, PO_DELTA = 6 };
/* Mesh shapes: a triangle mesh, or the implicit "Sphere" (LowerLevelSphereBVH(0.5)) and
 * "Cube" (LowerLevelCube) assets every scene starts with (Core/Scene.cpp:49-57). */
enum { PO_SHAPE_TRIANGLES = 0, PO_SHAPE_SPHERE = 1, PO_SHAPE_CUBE = 2 };

typedef struct {
    uint32_t nverts, ntris;
    const float* positions;   /* nverts * 3 */
    const float* normals;     /* nverts * 3 */
    const float* uvs;         /* nverts * 2, or NULL (interpolates to 0) */
    const uint32_t* indices;  /* ntris * 3 */
    float aabb_min[3], aabb_max[3]; /* aiMesh::mAABB: min/max over the positions */
    uint32_t shape;                 /* PO_SHAPE_*; the other fields are ignored for implicit shapes */
} po_mesh_desc;

typedef struct {
    uint32_t mesh, bsdf, material, reserved;
    float transform[16];      /* column-major object->world matrix */
} po_instance_desc;

/* Core::EvaluatedMaterial for constant materials (Core/MaterialManager.hpp:17-46). */
typedef struct {
    float diffuse[3], specular[3], roughness, emissive[3];
    float index_of_refraction;      /* ConstantTransparentMaterial's IoR (Transparent / Fresnel lobes) */
} po_material;

/* Core::Ray (Core/AABB.hpp:24-42): origin is a vec4, dir[3] carries mLenght. */
typedef struct { float org[4]; float dir[4]; } po_ray;

/* A hit on an implicit shape reports prim = PO_IMPLICIT_PRIM and u = its object-space t. */
#define PO_IMPLICIT_PRIM 0xfffffffeu
typedef struct { uint32_t inst, prim; float t, u, v; } po_hit;

/* Full closest-hit record: the reference's InterpolatedVertex plus IDs. */
typedef struct {
    uint32_t inst, prim; float t, u, v;
    float position[4], normal[3], uv[2];
} po_fragment;

/* Scene::Camera members (Core/Camera.hpp:98-107). */
typedef struct {
    float position[3], direction[3], up[3];
    uint32_t resolution[2];
    float aspect, near_plane, far_plane, fov;
} po_camera;

typedef struct po_scene po_scene;

/* The sky of Scene::process_globals (Core/Scene.cpp:639-700) and its sun; the
 * same layout as pico_sky of the product's header. */
enum { PO_SKY_CONSTANT = 0, PO_SKY_CUBE_RGBA8 = 1, PO_SKY_EQUIRECT_RGBAF = 2 };
typedef struct {
    uint32_t kind, width, height;
    const void* pixels;       /* CUBE_RGBA8: 6 faces of W*H RGBA bytes; EQUIRECT_RGBAF: W*H RGBA floats */
    int32_t use_sun;
    float sun_direction[3], sun_colour[3];
} po_sky;

po_scene* po_scene_create(const po_mesh_desc* meshes, uint32_t nmeshes,
                          const po_instance_desc* instances, uint32_t ninstances,
                          const po_material* materials, uint32_t nmaterials);
void po_scene_destroy(po_scene* s);
/* Copies the sky into the scene (sky NULL or kind CONSTANT: the constant rgb, no
 * sun unless sky says so).  A scene without this call has a black sky, no sun. */
void po_scene_set_sky(po_scene* s, const po_sky* sky, const float* rgb);
/* ImageCube::sample4 (Core/Image.cpp:361-397): RGBA of n directions (dirs n*3). */
void po_sky_sample(const po_sky* sky, const float* dirs, uint32_t n, float* rgba);

/* BVH introspection (node arrays in the reference's post-order). */
uint32_t po_blas_node_count(const po_scene* s, uint32_t mesh);
uint32_t po_tlas_node_count(const po_scene* s);
/* per node: box min xyz, max xyz (6 floats); child0, child1, first, count (4 u32);
 * leaf values (triangle / instance indices) in leaf order. */
void po_blas_nodes(const po_scene* s, uint32_t mesh, float* boxes, uint32_t* links, uint32_t* values);
void po_tlas_nodes(const po_scene* s, float* boxes, uint32_t* links, uint32_t* values);
void po_instance_matrices(const po_scene* s, uint32_t inst, float* transform, float* inverse);

/* glm::inverse(mat4) (glm/detail/func_matrix.inl:297-355). */
void po_mat4_inverse(const float* m, float* out);

/* UpperLevelBVH::get_closest_intersection over a batch (Core/UpperLevelBVH.cpp:12-20).
 * Misses report inst = prim = 0xffffffff and t = +inf.  nthreads <= 0 uses all cores. */
void po_trace(const po_scene* s, const po_ray* rays, uint32_t n, po_hit* hits, int nthreads);
void po_trace_fragments(const po_scene* s, const po_ray* rays, uint32_t n, po_fragment* out);
/* Visit statistics of the reference traversal (nodes, triangle tests, instance entries). */
void po_trace_stats(const po_scene* s, const po_ray* rays, uint32_t n, uint64_t* nodes,
                    uint64_t* tris, uint64_t* instances);

/* Camera::generate_ray (Core/Camera.cpp:11-28). */
void po_generate_ray(const po_camera* cam, float xi_x, float xi_y, uint32_t px, uint32_t py, po_ray* out);

/* ---------------- sampling building blocks (known-answer tests) ---------------- */
uint32_t po_xorshift_next(uint32_t state[4]);                 /* Core/RandUtils.cpp:65-81 */
void po_xorshift_seed(uint32_t seed, uint32_t state[4]);      /* Core/RandUtils.cpp:57-63 */
float po_radical_inverse(uint32_t bits);                      /* Core/RandUtils.cpp:13-21 */
void po_hammersley_next(uint32_t state[4], float* xi);        /* Core/RandUtils.cpp:87-90 */
void po_uniform_sample_triangle(const float* xi, float* out); /* Core/RandUtils.cpp:29-33 */
void po_mt64_seed(uint64_t* state /* 313 words */, uint64_t seed);
float po_mt64_uniform(uint64_t* state);                        /* uniform_real_distribution<float> */

void po_tangent_frame(const float* V, const float* N, float* m3);          /* Core/vectorUtils.cpp:9-35 */
void po_cos_sample(const float* xi, float* H);                               /* Render/Distributions.cpp:14-24 */
float po_cos_pdf(const float* H);                                            /* Render/Distributions.cpp:25-29 */
void po_beckmann_sample(const float* xi, const float* V, float R, float* H); /* Render/Distributions.cpp:31-48 */
float po_beckmann_pdf(const float* H, float R);                              /* Render/Distributions.cpp:50-56 */
float po_bsdf_pdf(int bsdf, const float* wo, const float* H, float roughness, float reflectance);
/* BSRDF::sample for Diffuse/Specular/Dielectric/Light (Render/BSRDF.cpp:11-202);
 * `xi` holds the Hammersley points the lobe consumes (2 for Diffuse/Specular/Light, 4 for Dielectric). */
void po_bsdf_sample(int bsdf, const po_material* mat, const float* V, const float* N,
                    const float* xi, float* L, float* P, float* energy);
float po_direct_lighting_pdf(int bsdf, const po_material* mat, const float* N,
                             const float* wi, const float* wo);   /* Render/Integrators.cpp:13-22 */
/* AliasTable::build_table / sample (Util/AliasTable.cpp:12-104). */
void po_alias_build(const float* weights, uint32_t n, float* bucket_weight, uint32_t* bucket_alias);
/* LowerLevelMeshBVH::generate_sampling_data triangle weights (Core/LowerLevelMeshBVH.cpp:92-117). */
void po_triangle_weights(const po_mesh_desc* mesh, float* weights);

/* Monte_Carlo_Integrator::integrate_ray (Render/Integrators.cpp:130-154) with the
 * reference's own random streams (xorshift Hammersley + mt19937_64), seeded
 * like the Integrator constructor (Render/Integrators.cpp:36-44). */
void po_integrate_ray(const po_scene* s, const po_camera* cam, uint32_t px, uint32_t py,
                      uint32_t max_depth, uint64_t seed, uint32_t nsamples, float* out_rgb);
/* The per-pixel sample loop of Scene::render_scene_to_memory (Core/Scene.cpp:164-198):
 * one integrator per pixel seeded with seeds[i], running mean / variance, early exit. */
void po_render_pixels(const po_scene* s, const po_camera* cam, uint32_t max_depth,
                      uint32_t max_samples, float max_variance,
                      const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels,
                      float* pixels, uint32_t* sample_count, float* variance, int nthreads);
/* The physical estimator (no reference counterpart; po_physical.c): the BSDF at
 * unit V, N, L (double), a sample from three uniforms (returns 0 when it leaves
 * below the surface), and the plain FP64 mean and sample variance of `spp` paths
 * per listed pixel with both light strategies (0), light sampling alone (1) or
 * BSDF sampling alone (2). */
void po_phys_bsdf_eval(int bsdf, const po_material* m, const double* V, const double* N, const double* L,
                       double* f_rgb, double* pdf);
int po_phys_bsdf_sample(int bsdf, const po_material* m, const double* V, const double* N, const double* u3,
                        double* L, double* pdf, double* weight_rgb);
void po_phys_render_mean(const po_scene* s, const po_camera* cam, uint32_t max_depth, uint32_t spp,
                         const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels, int strategy,
                         double* mean_rgb, double* var_rgb, int nthreads);
/* The radiance-cache form of the physical estimator with a cache answering the
 * constant cache_rgb: paths end after one bounce (two behind a first vertex of
 * roughness < 0.1) with throughput * cache_rgb. */
void po_phys_render_mean_cached(const po_scene* s, const po_camera* cam, uint32_t max_depth, uint32_t spp,
                                const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels,
                                const double* cache_rgb, double* mean_rgb, double* var_rgb, int nthreads);
/* Mean/variance recurrence alone, applied to a given sample sequence per pixel. */
void po_accumulate(const float* samples /* n * 3 */, uint32_t n, uint32_t max_samples,
                   float max_variance, float* pixel, uint32_t* count, float* variance);

/* Scene::generate_denoiser_inputs (Core/Scene.cpp:248-294) and
 * Util::atrous_denoise (Util/Denoisers.cpp:18-126). */
void po_denoiser_inputs(const po_scene* s, const po_camera* cam, uint32_t W, uint32_t H,
                        float* normals, float* positions, float* diffuse);
void po_view_matrix(const po_camera* cam, float* m4);          /* Camera::getViewMatrix */
void po_atrous_denoise(const float* pixels, const float* normals, const float* positions,
                       const float* diffuse, uint32_t W, uint32_t H, float* out);
/* Util::reinhard_tone_mapping (Util/ToneMappers.cpp:12-44), in place. */
void po_reinhard(float* pixels, uint32_t W, uint32_t H);
/* render_scene_to_file's output step (Core/Scene.cpp:238-246): std::reverse of
 * the pixels, then stbi_write_hdr's Radiance RGBE file (returns its length). */
void po_reverse_pixels(float* pixels, uint32_t n);
void po_rgbe(const float* rgb, unsigned char* out);
size_t po_encode_hdr(const float* pixels, uint32_t W, uint32_t H, unsigned char* out, size_t cap);

#ifdef __cplusplus
}
#endif
#endif
