/*
 * pico_gpu — GB300 (sm_103a) implementation of the Pico path tracer's
 * rendering hot path behind a plain C ABI.
 *
 * The entry points replace these reference interfaces (paths relative to the
 * Pico source tree):
 *
 *   pico_gpu_scene_upload      Scene's BLAS/TLAS construction: LowerLevelMeshBVH's
 *                              constructor (Core/LowerLevelMeshBVH.cpp:11-79),
 *                              UpperLevelBVH::add_lower_level_bvh / build
 *                              (Core/UpperLevelBVH.cpp:22-57), the light list of
 *                              Scene::add_mesh_instance (Core/Scene.cpp:406-412)
 *   pico_gpu_trace_closest     UpperLevelBVH::get_closest_intersection
 *                              (Core/UpperLevelBVH.hpp:36, Core/UpperLevelBVH.cpp:12-20)
 *   pico_gpu_render            Scene::render_scene_to_memory
 *                              (Core/Scene.hpp:68, Core/Scene.cpp:143-235) with the
 *                              Monte_Carlo_Integrator it runs per pixel
 *                              (Render/Integrators.hpp:33-57)
 *   pico_gpu_denoiser_inputs   Scene::generate_denoiser_inputs (Core/Scene.cpp:248-294)
 *   pico_gpu_atrous            Util::atrous_denoise (Util/Denoisers.hpp:9)
 *   pico_gpu_tonemap           Util::reinhard_tone_mapping (Util/ToneMappers.hpp, ToneMappers.cpp:12-44)
 *   pico_gpu_render_to_file    Scene::render_scene_to_file (Core/Scene.hpp:69, Core/Scene.cpp:238-246)
 *
 * Conventions: every function returns PICO_OK (0) or a negative PICO_ERR_*
 * code; host buffers are caller-owned and the call returns when they hold
 * the result (synchronous semantics); a context belongs to one host thread.
 * Matrices are column-major 4x4 (glm layout).
 */
#ifndef PICO_GPU_H
#define PICO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum pico_status {
    PICO_OK = 0,
    PICO_ERR_INVALID_ARG = -1,
    PICO_ERR_CUDA = -2,
    PICO_ERR_OUT_OF_MEMORY = -3,
    PICO_ERR_STACK_OVERFLOW = -4,   /* a ray needed a deeper traversal stack than the kernel has */
    PICO_ERR_TIMEOUT = -5,          /* a bounded device loop gave up */
    PICO_ERR_CANCELLED = -6,        /* *should_quit became non-zero */
    PICO_ERR_NO_DEVICE = -7,
    PICO_ERR_UNSUPPORTED = -8
};

/* BSRDF kinds, numbered like Render::BSRDF_Type (Render/BSRDF.hpp:32-39). */
enum pico_bsdf {
    PICO_BSDF_DIFFUSE = 0,          /* Diffuse_BRDF */
    PICO_BSDF_SPECULAR = 1,         /* Specular_BRDF */
    PICO_BSDF_DIELECTRIC = 2,       /* Dielectric_BRDF */
    PICO_BSDF_BTDF = 3,             /* Transparent_BTDF (type kBTDF) */
    PICO_BSDF_LIGHT = 4,            /* Light_BRDF */
    PICO_BSDF_FRESNEL = 5,          /* Fresnel_BTDF (type kBTDF) */
    PICO_BSDF_DELTA = 6             /* Specular_Delta_BRDF (type kSpecular_BRDF) */
};

/* Mesh shapes: triangles, or the implicit assets every reference scene holds
 * (Core/Scene.cpp:49-57): "Sphere", LowerLevelSphereBVH(0.5), and "Cube",
 * LowerLevelCube over [-0.5, 0.5]^3 (Core/LowerLevelImplicitShapesBVH.cpp). */
enum pico_shape { PICO_SHAPE_TRIANGLES = 0, PICO_SHAPE_SPHERE = 1, PICO_SHAPE_CUBE = 2 };

typedef struct pico_gpu_ctx pico_gpu_ctx;
typedef struct pico_gpu_scene pico_gpu_scene;

/* An indexed triangle mesh, as LowerLevelMeshBVH copies it out of an aiMesh. */
typedef struct {
    uint32_t nverts, ntris;
    const float* positions;         /* nverts * 3 */
    const float* normals;           /* nverts * 3 */
    const float* uvs;               /* nverts * 2, or NULL */
    const uint32_t* indices;        /* ntris * 3 */
    float aabb_min[3], aabb_max[3]; /* aiMesh::mAABB */
    uint32_t shape;                 /* pico_shape; implicit shapes ignore the fields above */
} pico_mesh;

/* One UpperLevelBVH::Entry: mesh, object->world transform, BSRDF and material. */
typedef struct {
    uint32_t mesh, bsdf, material, reserved;
    float transform[16];
} pico_instance;

/* Core::EvaluatedMaterial of a constant material (Core/MaterialManager.hpp:17-46). */
typedef struct {
    float diffuse[3], specular[3], roughness, emissive[3];
    float index_of_refraction;      /* of a ConstantTransparentMaterial (Render/BasicMaterials.hpp:41-66) */
} pico_material;

/* The sky and sun of Scene::process_globals (Core/Scene.cpp:639-700): the
 * radiance of rays that leave the scene is ImageCube::sample4 of their
 * direction (Core/Image.cpp:361-397, nearest texel; a 6-face cube of RGBA8
 * images, or one RGBA float equirectangular image), and with use_sun the light
 * pick of sample_direct_lighting includes a directional sun
 * (Render/Integrators.cpp:54-76). */
enum pico_sky_kind {
    PICO_SKY_CONSTANT = 0,          /* pico_scene_desc::sky_rgb everywhere */
    PICO_SKY_CUBE_RGBA8 = 1,        /* 6 faces of width*height RGBA bytes: +x, -x, +y, -y, +z, -z */
    PICO_SKY_EQUIRECT_RGBAF = 2     /* width*height RGBA floats, row 0 at the top */
};
typedef struct {
    uint32_t kind;
    uint32_t width, height;         /* of one face for the cube */
    const void* pixels;
    int32_t use_sun;
    float sun_direction[3];         /* the direction sunlight travels, normalised */
    float sun_colour[3];
} pico_sky;

typedef struct {
    const pico_mesh* meshes; uint32_t nmeshes;
    const pico_instance* instances; uint32_t ninstances;
    const pico_material* materials; uint32_t nmaterials;
    float sky_rgb[3];               /* constant sky radiance (the black 1x1 sky of Scene.cpp:683-690) */
    const pico_sky* sky;            /* NULL: the constant sky_rgb and no sun */
} pico_scene_desc;

/* Core::Ray's origin (vec4) and direction; dir[3] carries mLenght (the far distance). */
typedef struct { float org[4]; float dir[4]; } pico_ray;

/* Closest hit: instance (insertion index), triangle (mesh index), world distance
 * |T * P(u,v) - O| exactly as lower_level_intersector::intersects computes it,
 * and the barycentrics.  A miss has inst = prim = 0xffffffff and t = +inf; a hit
 * on an implicit sphere or cube has prim = 0xfffffffe and its object-space ray
 * parameter in u. */
typedef struct { uint32_t inst, prim; float t, u, v; } pico_hit;

/* Scene::Camera members (Core/Camera.hpp:98-107); the FOV is carried but, as in
 * the reference, rays use an image plane at distance 1 with half-height 0.5. */
typedef struct {
    float position[3], direction[3], up[3];
    uint32_t resolution[2];
    float aspect, near_plane, far_plane, fov;
} pico_camera;

/* Scene::RenderParams (Core/Scene.hpp:30-43) without the buffers, plus the seed
 * that replaces the reference's std::random_device draw and the estimator.
 *
 * PICO_ESTIMATOR_REFERENCE (0) is Monte_Carlo_Integrator (Render/Integrators.cpp:
 * 46-209) with the render loop of Scene.cpp:164-198, quirks included.
 * PICO_ESTIMATOR_PHYSICAL (1) has no counterpart in the reference: Lambert plus
 * GGX microfacet reflection (alpha = roughness^2, Smith height-correlated
 * masking, Schlick Fresnel with F0 = specular) sampled through the GGX
 * visible-normal distribution, next-event estimation on the triangle lights and
 * the sun combined with BSDF sampling by the power heuristic, Russian roulette
 * from the fourth vertex, a jitter over the whole pixel and a plain running mean
 * (every sample counts; max_variance is ignored and no pixel stops early).
 * Diffuse, Specular, Dielectric, Light and Specular_Delta (a mirror with Schlick
 * reflectance) instances are supported, and Transparent and Fresnel ones as a
 * rough dielectric interface between air and the material's
 * index_of_refraction (GGX with alpha = roughness^2, Walter et al. 2007): the
 * Fresnel kind reflects with the exact dielectric Fresnel probability and
 * refracts otherwise, the Transparent kind only refracts (it reflects under
 * total internal reflection), refraction tinted by the diffuse colour; these
 * vertices take no next-event estimation.  The radiance cache estimator returns
 * PICO_ERR_UNSUPPORTED for Transparent and Fresnel instances.  Emitters are
 * two-sided; the sun is a directional light whose colour is its irradiance. */
enum pico_estimator {
    PICO_ESTIMATOR_REFERENCE = 0,
    PICO_ESTIMATOR_PHYSICAL = 1,
    /* No counterpart in the reference: the physical estimator whose camera paths
     * end after one bounce (two when the first vertex has roughness < 0.1) in the
     * context's neural radiance cache (pico_gpu_set_radiance_cache), which every
     * sample pass first trains on full-depth physical paths.  See the radiance
     * cache section below. */
    PICO_ESTIMATOR_RADIANCE_CACHE = 2
};
typedef struct {
    uint32_t max_ray_depth;
    uint32_t max_samples;
    float max_variance;
    uint32_t height, width;
    int32_t tonemap, denoise;
    uint32_t estimator;       /* pico_estimator */
    uint64_t seed;
} pico_render_config;

/* ---- context ------------------------------------------------------------ */
int pico_gpu_init(int device, pico_gpu_ctx** out);
void pico_gpu_shutdown(pico_gpu_ctx* ctx);
const char* pico_gpu_status_string(int status);
const char* pico_gpu_last_error(const pico_gpu_ctx* ctx);

/* Traversal order of every closest-hit query in a context.  NEAR_FIRST (the
 * default) enters the nearer child first and breaks equal distances by the
 * reference's depth-first rank; REFERENCE walks children 0 then 1 with strict
 * comparisons exactly like BVH::get_closest_intersections (Core/BVH.cpp:27-63).
 * They differ only where the reference's float slab test prunes a box whose
 * triangle is a few ulp nearer than the best so far (near-ties at shared
 * edges); REFERENCE reproduces the reference's choice there too.  Scenes with
 * implicit sphere instances are always walked in the REFERENCE order: the
 * reference's sphere test reports points off a scaled sphere, and which of them
 * it returns depends on its own visit order. */
enum pico_traversal_order { PICO_ORDER_NEAR_FIRST = 0, PICO_ORDER_REFERENCE = 1 };
int pico_gpu_set_traversal_order(pico_gpu_ctx* ctx, int order);
/* The bounds every traversal of this context's calls runs under (the reference
 * recurses without bounds, Core/BVH.cpp:27-63, depth limited to 32 only at build
 * time, Core/BVH.hpp:129): at most max_iterations steps per ray walk (0: the
 * default 2^24) and at most stack_entries entries of the 96-entry traversal stack
 * (0: all 96).  A walk that needs more stops, and the call returns
 * PICO_ERR_TIMEOUT or PICO_ERR_STACK_OVERFLOW; nothing waits or faults.  Smaller
 * bounds are a debugging aid and for tests of those error paths; the defaults
 * never bind on scenes of the reference's depth limit. */
int pico_gpu_set_traversal_limits(pico_gpu_ctx* ctx, uint32_t max_iterations, uint32_t stack_entries);
/* The ray / triangle test of every closest-hit query in a context.
 * MOLLER_TRUMBORE (the default) is the reference's Mesh_Intersector::intersects
 * (Core/LowerLevelMeshBVH.cpp:165-207, epsilon 1e-7) in its float operation order,
 * which gives the reference's hits bit for bit.  WATERTIGHT has no counterpart in
 * the reference: the test of Woop, Benthin and Wald (JCGT 2013), under which a ray
 * through an edge or vertex shared by two triangles always hits one of them
 * (Moeller-Trumbore can let such rays through the crack); away from edges it finds
 * the same triangles, with t, u, v equal up to rounding. */
enum pico_triangle_test { PICO_TRIANGLE_MOLLER_TRUMBORE = 0, PICO_TRIANGLE_WATERTIGHT = 1 };
int pico_gpu_set_triangle_test(pico_gpu_ctx* ctx, int test);

/* ---- scene -------------------------------------------------------------- */
int pico_gpu_scene_upload(pico_gpu_ctx* ctx, const pico_scene_desc* desc, pico_gpu_scene** out);
void pico_gpu_scene_free(pico_gpu_scene* scene);
/* Sizes of the flattened scene: [0] TLAS nodes, [1] BLAS nodes, [2] triangles,
 * [3] instances, [4] device bytes, [5] lights. */
int pico_gpu_scene_info(const pico_gpu_scene* scene, uint64_t* out6);
/* The binary BVH pico_gpu_scene_upload builds before flattening it (host only, no
 * device needed), in the layout of the reference's BVH<T,2>::m_nodes
 * (Core/BVH.hpp:52-81, built by Core/BVH.cpp:73-197): which = -1 the TLAS over
 * instances, else the BLAS of mesh `which`.  Per node, in the order the builder
 * pushes them (children before their parent): boxes[6] (min xyz, max xyz),
 * links[4] (child 0, child 1, 0xffffffff for none; first, count of its leaf items
 * in `values`); values lists every leaf's items (triangle or instance indices) in
 * node order.  *nnodes and *nvalues receive the sizes; NULL arrays are skipped, so
 * a first call with NULL arrays sizes the second. */
int pico_gpu_reference_bvh(const pico_scene_desc* desc, int32_t which, float* boxes, uint32_t* links,
                           uint32_t* values, uint32_t* nnodes, uint32_t* nvalues);

/* ---- closest hit (UpperLevelBVH::get_closest_intersection) --------------- */
/* rays / hits are host buffers.  When each lies inside one page-locked, mapped
 * allocation (cudaHostAlloc, or one cudaHostRegister under unified addressing)
 * the kernel reads and writes them in place (over NVLink-C2C on a Grace host),
 * with no staging copies; other buffers are staged through device memory in
 * chunks, and a buffer only partly inside page-locked memory through
 * page-locked bounce buffers of the context (slower, chunk by chunk). */
int pico_gpu_trace_closest(pico_gpu_ctx* ctx, const pico_gpu_scene* scene,
                           const pico_ray* rays, uint64_t n, pico_hit* hits);
/* No counterpart in the reference: whether pico_gpu_trace_closest reads or
 * writes the host range [p, p + bytes) in place (*in_place = 1) or stages it
 * through device memory (0).  In place needs the whole range inside ONE
 * page-locked allocation or registration that is mapped for the context's
 * device; a range spanning several pinned regions is staged, since pageable
 * memory may lie between them. */
int pico_gpu_host_buffer_in_place(pico_gpu_ctx* ctx, const void* p, uint64_t bytes, int32_t* in_place);
/* Device-pointer variant on a caller stream (cudaStream_t, NULL = legacy default). */
int pico_gpu_trace_closest_device(pico_gpu_ctx* ctx, const pico_gpu_scene* scene,
                                  const pico_ray* d_rays, uint64_t n, pico_hit* d_hits,
                                  void* stream);
/* Waits for `stream` and returns the status the device-pointer calls latched
 * since the last check (traversal stack overflow, loop bound), clearing it. */
int pico_gpu_check(pico_gpu_ctx* ctx, void* stream);
/* Counts, over a ray batch, the nodes visited, triangles tested and instance
 * entries transformed by this library's traversal (out3 = {nodes, tris, instances}). */
int pico_gpu_trace_stats(pico_gpu_ctx* ctx, const pico_gpu_scene* scene,
                         const pico_ray* d_rays, uint64_t n, uint64_t* out3, void* stream);

/* ---- rendering (Scene::render_scene_to_memory) --------------------------- */
/* No counterpart in the reference.  The most paths (pixels x samples) a batch of
 * this context's renders holds: 0 for the default, 2^26, else 64 .. 2^26.  A
 * smaller limit holds less path state on the device (208 bytes per path) for more
 * launches; an image of more pixels than the limit is rendered in pixel chunks.
 * The images are the same whatever the limit: a path depends only on its pixel and
 * sample index, and each pixel takes its samples in order. */
int pico_gpu_set_path_limit(pico_gpu_ctx* ctx, uint32_t max_paths);
/* The render runs in batches of up to 2^26 paths (pixels x samples; 208 bytes of
 * path state each, 14 GB at the limit).  Where the reference's early exit can
 * stop pixels (reference estimator, max_variance >= 0) the first batch takes 6
 * samples per pixel and later batches only the pixels still sampling, as many
 * samples each as fill the path state; otherwise every batch covers all pixels.
 * With a cancel flag (should_quit not NULL) it polls *should_quit before every
 * batch and a batch takes at most 16 samples per pixel: about 30-40 ms each for a
 * 1080p render on a GB300, which bounds how soon a cancel is seen. */
int pico_gpu_render(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                    const pico_render_config* config, float* pixels_rgb, uint32_t* sample_count,
                    float* variance_rgb, const volatile int32_t* should_quit);
/* Work of the context's last pico_gpu_render call: [0] samples added to the
 * image (the growth of sample_count), [1] camera paths traced (pixels past their
 * early exit trace none), [2] bounce rays, [3] next-event shadow rays,
 * [4] G-buffer primary rays (W*H when denoising, else 0).  After
 * pico_gpu_render_device it first waits for that render's stream. */
int pico_gpu_render_stats(const pico_gpu_ctx* ctx, uint64_t* out5);
/* No counterpart in the reference, whose RenderParams buffers are host memory:
 * pico_gpu_render on device buffers (d_pixels and d_variance W*H*3 floats,
 * d_count W*H), enqueued on `stream` (cudaStream_t, NULL = legacy default)
 * without waiting for it and without host copies: the same samples, denoise
 * and tone map, so the same images as pico_gpu_render gives for the same
 * inputs.  There is no cancel flag; the reference and physical estimators only.
 * Traversal errors are latched like the other device-pointer calls and
 * returned by pico_gpu_check(ctx, stream); pico_gpu_render_stats reports this
 * render's work.  The buffers must not be touched until the stream reaches the
 * end of the render. */
int pico_gpu_render_device(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                           const pico_render_config* config, float* d_pixels, uint32_t* d_count,
                           float* d_variance, void* stream);

/* ---- measurement ---------------------------------------------------------------
 * No counterpart in the reference, whose only profiler is a stub (Core/Profiler.hpp).
 * pico_gpu_set_render_probe switches the hooks on the closest-hit launches of this
 * context's renders (both off by default) and clears their totals: time_extend
 * brackets every such launch with CUDA events on its stream; count_work runs a
 * counting variant of the launches (the same traversal, 128-thread CTAs) that
 * tallies the nodes visited, triangles tested and instance entries transformed.
 * pico_gpu_render_probe_read waits for the device and returns the totals since:
 * out4 = {launches timed, nodes, triangles, instance entries}, *extend_ms = the
 * timed launches' summed duration. */
int pico_gpu_set_render_probe(pico_gpu_ctx* ctx, int32_t time_extend, int32_t count_work);
int pico_gpu_render_probe_read(pico_gpu_ctx* ctx, uint64_t* out4, double* extend_ms);
/* With time_extend on, the shade launches (one per bounce depth) are bracketed too:
 * their count and summed duration since the probe was set. */
int pico_gpu_render_probe_read_shade(pico_gpu_ctx* ctx, uint64_t* launches, double* shade_ms);
/* The read bandwidth of the L2 cache (GB/s), the roof of the closest-hit kernels
 * whose scene data stays in L2: one launch reads a device buffer of `bytes` bytes
 * (0: 32 MiB, which the GB300's L2 holds) `passes` times (0: 100) with 16-byte
 * loads cached in L2 only, after a warm-up pass; the best of five launches. */
int pico_gpu_l2_read_bandwidth(pico_gpu_ctx* ctx, uint64_t bytes, uint32_t passes, double* gbs);

/* ---- denoiser ------------------------------------------------------------ */
int pico_gpu_denoiser_inputs(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                             float* normals, float* positions, float* diffuse);
int pico_gpu_atrous(pico_gpu_ctx* ctx, const float* pixels, const float* normals, const float* positions,
                    const float* diffuse, uint32_t width, uint32_t height, float* out);
/* Device-pointer variant; all buffers are W*H*3 floats. */
int pico_gpu_atrous_device(pico_gpu_ctx* ctx, const float* d_pixels, const float* d_normals,
                           const float* d_positions, const float* d_diffuse, uint32_t width,
                           uint32_t height, float* d_out, void* stream);
/* No counterpart in the reference.  pico_gpu_atrous_device for callers that
 * must not allocate device memory during their denoise step: a frame loop that
 * overlaps streams (cudaFree, and often cudaMalloc, synchronises the whole
 * device) or a process whose device memory belongs to another allocator.  On
 * success it allocates nothing: its scratch is a fixed 48 MiB + 5.5 MiB device
 * array per device, so images are limited to 2,097,152 pixels (1920 x 1080
 * fits) and 65,535 rows; larger ones return PICO_ERR_INVALID_ARG with a
 * message, and so does an output that overlaps an input.  The caller's current
 * device is left as it was.  All calls on a device share that array: calls that overlap on the
 * GPU race, so order them on one stream.  Nothing in it has to start at zero.
 * The first call on a device looks up the array's address (set-up); make that
 * first call before any stream capture. */
int pico_gpu_atrous_device_noalloc(pico_gpu_ctx* ctx, const float* d_pixels, const float* d_normals,
                                   const float* d_positions, const float* d_diffuse, uint32_t width,
                                   uint32_t height, float* d_out, void* stream);

/* Util::reinhard_tone_mapping (Util/ToneMappers.cpp:12-44) in place on W*H*3 floats. */
int pico_gpu_tonemap(pico_gpu_ctx* ctx, float* pixels, uint32_t width, uint32_t height);
int pico_gpu_tonemap_device(pico_gpu_ctx* ctx, float* d_pixels, uint32_t width, uint32_t height, void* stream);

/* ---- image output --------------------------------------------------------
 * Scene::render_scene_to_file (Core/Scene.hpp:69, Core/Scene.cpp:238-246):
 * render, reverse the flat pixel array in the caller's buffer (a 180-degree
 * rotation, as the reference does) and write a Radiance .hdr file with the same
 * bytes stbi_write_hdr produces.  pico_gpu_encode_hdr is the writer alone
 * (no reversal): it stores the file image in `out` (pico_gpu_hdr_bound bytes
 * always suffice) and its size in *length. */
int pico_gpu_render_to_file(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                            const pico_render_config* config, float* pixels_rgb, uint32_t* sample_count,
                            float* variance_rgb, const char* path);
size_t pico_gpu_hdr_bound(uint32_t width, uint32_t height);
int pico_gpu_encode_hdr(pico_gpu_ctx* ctx, const float* pixels, uint32_t width, uint32_t height,
                        unsigned char* out, size_t capacity, size_t* length);

/* ---- shading routines on caller inputs ---------------------------------------
 * BSRDF::pdf and BSRDF::sample (Render/BSRDF.hpp:50-52) and direct_lighting_pdf
 * (Render/Integrators.cpp:13-22) as the device integrator evaluates them, for n
 * tuples: kinds[n], mats[n], V/N/H[n*3], xi[n*4] (the Hammersley points the lobe
 * consumes, in order).  Outputs: pdf(V, H) [n], L [n*3], P [n], energy [n*3] and
 * the direct-lighting pdf towards L [n]. */
int pico_gpu_bsdf_eval(pico_gpu_ctx* ctx, uint64_t n, const uint32_t* kinds, const pico_material* mats,
                       const float* V, const float* N, const float* H, const float* xi, float* pdf,
                       float* L, float* P, float* energy, float* direct_pdf);
/* No counterpart in the reference: the physical estimator's BSDF (see
 * pico_render_config) for n tuples of a Diffuse, Specular or Dielectric kind,
 * unit V, N, L [n*3] and uniforms u [n*3]: f(V, L) [n*3] and the sampling
 * density of L [n], and one sample from u: its direction [n*3], density [n],
 * throughput weight f (N.L) / pdf [n*3] and whether it stays above the surface
 * [n].  Other kinds return PICO_ERR_INVALID_ARG. */
int pico_gpu_phys_bsdf_eval(pico_gpu_ctx* ctx, uint64_t n, const uint32_t* kinds, const pico_material* mats,
                            const float* V, const float* N, const float* L, const float* u, float* f, float* pdf,
                            float* sample_L, float* sample_pdf, float* sample_weight, uint32_t* sample_ok);

/* ---- batched rendering ------------------------------------------------------
 * No counterpart in the reference, which renders one scene at a time.  Many
 * independent renders, each what pico_gpu_render does for one (scene, camera,
 * config, progressive buffers) with the REFERENCE or PHYSICAL estimator and
 * no denoise / tone map, run as one CUDA graph: the renders (or their pieces)
 * are spread over graph branches (streams) by estimated cost (pixels x samples
 * x (1 + min(depth, 4))) so that the branches end together, each branch runs
 * its work cheapest first, and the cheaper a piece the higher the scheduling
 * priority of its kernels; the graph is instantiated and launched once, and the
 * branches share the GPU.  The cancel flag is not polled.  Each render keeps
 * its own path state (at most `wavefront` paths), so device memory grows with
 * the number of renders. */
typedef struct {
    const pico_gpu_scene* scene;
    pico_camera camera;
    pico_render_config config;
    float* pixels_rgb;              /* W*H*3, in/out, as pico_gpu_render */
    uint32_t* sample_count;         /* W*H, in/out */
    float* variance_rgb;            /* W*H*3, in/out */
} pico_render_item;

typedef struct {
    uint32_t wavefront;             /* paths per batch of one render; 0: 2^20 */
    uint32_t extend_ctas_per_sm;    /* persistent CTAs per SM of each closest-hit launch; 0: as many as fit */
    uint32_t branches;              /* graph branches the pieces are spread over; 0: one per piece; at
                                     * most the device's work queues (CUDA_DEVICE_MAX_CONNECTIONS, 8 by
                                     * default), past which branches would share queues */
    uint32_t piece_paths;           /* a render of more paths (pixels x samples) than this is split into
                                     * pieces of disjoint pixel ranges, each its own branch work; 0: none */
    uint32_t extend_threads;        /* threads per CTA of each closest-hit launch: 64, 128 or 256; 0: 128 */
    uint32_t reserved;
} pico_launch_params;

typedef struct {
    double build_ms;                /* capture and instantiation of the graph */
    double run_ms;                  /* graph launch to completion (host clock) */
    uint64_t graph_nodes;
    uint64_t samples;               /* samples added over all renders */
    uint64_t rays;                  /* camera, bounce and shadow rays over all renders */
} pico_batch_report;

/* completion_ms (n entries, may be NULL): each render's finish time after the
 * graph started, from device timestamps. */
int pico_gpu_render_many(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items,
                         const pico_launch_params* params, double* completion_ms, pico_batch_report* report);
/* Chooses launch parameters for a set of renders by timing short renders of the
 * same items into scratch buffers (the items' buffers are not touched): the item
 * with the most samples per pixel takes trial_samples of them, every other item
 * the same fraction of its own, rounded, at least 1.  Tuned, each by the highest
 * samples per second: the wavefront size, then the closest-hit block shape
 * (threads per CTA), then the closest-hit CTAs per SM, then the piece size
 * (relative to the items' total paths), then the number of branches (2, 4, or
 * as many as the device has work queues).
 * trials_out / trial_msamples_per_s (may be NULL) receive up to max_trials tried
 * settings and their millions of samples per second; *ntrials the count. */
int pico_gpu_autotune_batch(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items, uint32_t trial_samples,
                            pico_launch_params* best, pico_launch_params* trials_out, double* trial_msamples_per_s,
                            uint32_t max_trials, uint32_t* ntrials);

/* ---- neural radiance cache ------------------------------------------------
 * No counterpart in the reference (Mueller et al. 2021, "Real-time neural
 * radiance caching for path tracing").  A cache maps a surface point to the
 * radiance it reflects towards a direction (its own emission excluded):
 *
 *   inputs   position in the cache's box through a 16-level multiresolution
 *            hash grid (Mueller et al. 2022; 2 fp16 features per level,
 *            2^log2_table_size entries per level, resolutions from
 *            base_resolution to max_resolution in geometric steps, dense
 *            indexing where a level fits its table), the direction through
 *            real spherical harmonics of degrees 0-3 (16 values), the normal,
 *            roughness and albedo (diffuse + specular colour), a constant 1
 *            and zero padding: 64 values;
 *   network  5 hidden layers of 64 ReLU units and 3 linear outputs, bf16
 *            weights and activations, fp32 accumulation on the tensor cores;
 *   training relative L2 loss sum_c (y_c - t_c)^2 / (y_c^2 + 0.01), the
 *            denominator held constant, averaged over the batch and channels;
 *            Adam over the fp32 master weights and grid features.
 *
 * Parameters for pico_gpu_nrc_get_params / set_params: the network as
 * 6 x 64 x 64 floats (layer, output, input; layer 5 uses outputs 0-2, the
 * other rows are ignored and kept 0) and the grid as levels x entries x 2
 * floats (16 x 2^log2_table_size x 2). */
typedef struct pico_gpu_nrc pico_gpu_nrc;

typedef struct {
    float position[3];
    float direction[3];             /* unit, towards the viewer */
    float normal[3];
    float roughness;
    float albedo[3];
    uint32_t payload;               /* carried through, unused by the network */
    uint32_t pad[2];
} pico_nrc_query;                   /* 64 bytes */

typedef struct {
    uint32_t log2_table_size;       /* [10, 22]; 19 */
    float base_resolution, max_resolution;   /* 16, 4096 */
    float aabb_min[3], aabb_max[3]; /* the box the grid covers; a render with an empty box uses the scene's bounds */
    float learning_rate, beta1, beta2, epsilon;   /* 1e-2, 0.9, 0.99, 1e-15 */
    uint32_t train_paths;           /* training paths per sample pass of a render: 65536 */
    uint32_t train_batch;           /* records per optimiser step: 65536, at most 2^20 */
    uint32_t max_train_steps;       /* optimiser steps per sample pass: 4 */
    uint32_t warmup_frames;         /* training-only passes before a render's first sample: 0 */
    uint64_t seed;                  /* initial weights and training-path streams */
    uint32_t bounces;               /* camera paths query the cache after this many bounces, one more
                                     * behind a vertex of roughness < 0.1 (a mirror counts as 0): 1 */
    uint32_t infer_groups;          /* 128-query tiles each inference CTA keeps in flight: 1, 2 or 4; 0: 4 */
} pico_nrc_config;

int pico_gpu_nrc_default_config(pico_nrc_config* out);
/* A cache lives on its context's device and must be freed before the context is
 * shut down.  An empty box (aabb_max not above aabb_min on any axis) is set from
 * the bounds of the first scene rendered with the cache; set_bounds changes it. */
int pico_gpu_nrc_create(pico_gpu_ctx* ctx, const pico_nrc_config* config, pico_gpu_nrc** out);
void pico_gpu_nrc_free(pico_gpu_nrc* cache);
int pico_gpu_nrc_get_params(pico_gpu_nrc* cache, float* mlp, float* grid);
/* Replaces the parameters and resets the optimiser state. */
int pico_gpu_nrc_set_params(pico_gpu_nrc* cache, const float* mlp, const float* grid);
int pico_gpu_nrc_set_bounds(pico_gpu_nrc* cache, const float* aabb_min, const float* aabb_max);
/* [0] optimiser steps, [1] grid entries, [2] network parameters (incl. padding), [3] frames rendered. */
int pico_gpu_nrc_info(const pico_gpu_nrc* cache, uint64_t* out4);
/* Render work with this cache since its creation: [0] training paths traced,
 * [1] training records, [2] optimiser steps, [3] cache queries of camera paths. */
int pico_gpu_nrc_stats(const pico_gpu_nrc* cache, uint64_t* out4);
/* The 64 network inputs of n queries (n * 64 floats, before their bf16 rounding). */
int pico_gpu_nrc_encode(pico_gpu_nrc* cache, const pico_nrc_query* queries, uint64_t n, float* out);
/* Network outputs (n * 3 floats) of n <= 2^26 queries. */
int pico_gpu_nrc_infer(pico_gpu_nrc* cache, const pico_nrc_query* queries, uint64_t n, float* rgb);
int pico_gpu_nrc_infer_device(pico_gpu_nrc* cache, const pico_nrc_query* d_queries, uint64_t n, float* d_rgb,
                              void* stream);
/* One optimiser step on n <= 2^20 records (targets: n * 3 floats; the device
 * variant takes n * 4 floats, the fourth unused); with apply = 0 only the
 * gradients are computed (pico_gpu_nrc_gradients reads them).  *loss receives
 * the batch's mean loss. */
int pico_gpu_nrc_train(pico_gpu_nrc* cache, const pico_nrc_query* queries, const float* targets, uint64_t n,
                       int apply, float* loss);
int pico_gpu_nrc_train_device(pico_gpu_nrc* cache, const pico_nrc_query* d_queries, const float* d_targets,
                              uint64_t n, int apply, void* stream);
/* Gradients of the last training call: network (6 x 64 x 64) and grid (levels x entries x 2). */
int pico_gpu_nrc_gradients(pico_gpu_nrc* cache, float* mlp_grad, float* grid_grad);
/* The cache's kernels wait on mbarriers for their bulk copies and tensor-core
 * commits; each wait gives up after limit_ns nanoseconds of the device's global
 * timer (1e9 by default), the kernel frees its tensor memory and returns, and the
 * call that launched it (or the render using the cache) returns PICO_ERR_TIMEOUT
 * with the context still usable.  withheld_bytes > 0 (at most 1024, a multiple of
 * 16) makes the inference kernel's weight-load barrier expect that many bytes more
 * than its copy delivers, so that this wait runs out: a test of the timeout path,
 * nothing else; 0 (the default) for every other use. */
int pico_gpu_nrc_set_wait_limit(pico_gpu_nrc* cache, uint64_t limit_ns, uint32_t withheld_bytes);
/* The cache PICO_ESTIMATOR_RADIANCE_CACHE renders of this context use (NULL: none). */
int pico_gpu_set_radiance_cache(pico_gpu_ctx* ctx, pico_gpu_nrc* cache);

#ifdef __cplusplus
}
#endif
#endif
