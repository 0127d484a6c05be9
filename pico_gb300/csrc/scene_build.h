// Host-side scene construction: the reference's SAH builder and the
// flattening of its binary BVHs into the device layout of layout.h.
#pragma once

#include "layout.h"
#include "pico_gpu.h"

#include <string>
#include <vector>

namespace pico {

// A binary BVH in the reference's own layout (BVH<T,2>::m_nodes, Core/BVH.hpp:52-81):
// nodes in the order the builder pushed them (children before their parent), per
// node its box (lo xyz, hi xyz), its two child indices (0xffffffff: none) and its
// leaf items as (first, count) into `values`, which lists every leaf's items in
// node order.
struct TreeDump {
    std::vector<float> boxes;
    std::vector<uint32_t> links;   // child 0, child 1, first, count per node
    std::vector<uint32_t> values;
};

// The most NEE lights whose boxes a shadow ray scans for its early exit.
constexpr size_t kMaxBoundedLights = 64;

// Host image of everything pico_gpu_scene_upload copies to the device.
struct FlatScene {
    // kept only when keep_trees is set before build_flat_scene: the reference-layout
    // trees the device nodes are flattened from (one per mesh, then the TLAS)
    bool keep_trees = false;
    std::vector<TreeDump> blas_trees;
    TreeDump tlas_tree;
    std::vector<GpuNode> nodes;           // TLAS nodes first, then every BLAS
    std::vector<GpuTri> tris;
    std::vector<GpuTriShade> tri_shade;
    std::vector<GpuInstance> insts;       // TLAS rank order
    std::vector<uint32_t> tlas_items;     // TLAS leaf items -> instance rank (identity for the reference tree)
    std::vector<GpuInstanceShade> inst_shade;
    std::vector<uint32_t> inst_rank;      // original index -> rank
    std::vector<GpuMaterial> materials;
    std::vector<GpuLight> lights;
    std::vector<float> light_alias_weight;
    std::vector<uint32_t> light_alias_index;
    std::vector<float> light_positions;
    std::vector<float> light_tri_geo;     // per light triangle: world unit normal, area pdf (4 floats)
    std::vector<uint32_t> light_of_inst;  // original instance index -> NEE light index, or ~0u
    // The physical estimator's next-event light pick over the slots lights[0 .. n-1]
    // and, with use_sun, the sun (slot n): cdf[n + sun] then pdf[n + sun].  The sun
    // keeps a uniform share 1 / (n + 1); triangle lights share the rest in proportion
    // to their power (sum of emitted radiance channels x world area), implicit
    // lights get 0 (the physical estimator reaches them by BSDF sampling only).
    std::vector<float> light_pick;
    // Per NEE light, its widened world box (lo x, y, z, 0, hi x, y, z, 0): no hit on
    // the light lies outside it.  light_bounds: the boxes exist for every light
    // (none may be missing for the shadow rays' early exit to hold).
    std::vector<float> light_boxes;
    bool light_bounds = false;
    uint32_t tlas_root_ref = PICO_REF_EMPTY;
    float tlas_lo[3] = {0, 0, 0}, tlas_hi[3] = {0, 0, 0};
    uint32_t tlas_fast_root_ref = PICO_REF_EMPTY;   // refitted TLAS for the near-first walk
    float tlas_fast_lo[3] = {0, 0, 0}, tlas_fast_hi[3] = {0, 0, 0};
    float sky[3] = {0, 0, 0};
    uint32_t sky_kind = PICO_SKY_CONSTANT, sky_w = 0, sky_h = 0, use_sun = 0;
    std::vector<unsigned char> sky_pixels;   // RGBA8 cube faces or RGBA float texels, as given
    float sun_dir[3] = {0, -1, 0}, sun_col[3] = {1, 1, 1};
    uint32_t tlas_nodes = 0, blas_nodes = 0;
};

// Builds the flat scene; returns an empty string on success, else the reason.
std::string build_flat_scene(const pico_scene_desc& desc, FlatScene& out);

// glm::inverse of a column-major 4x4 in glm's operation order.
void mat4_inverse(const float* m, float* out);

}  // namespace pico
