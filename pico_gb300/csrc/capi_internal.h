// Internal definitions behind the C ABI.
#pragma once

#include "kernels.h"
#include "pico_gpu.h"
#include "scene_build.h"
#include "traverse_status.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

struct RenderBuffers;
struct BatchState;
struct pico_gpu_nrc;
namespace pico {
struct LaunchTimer;
}

namespace pico {

// Makes a device current for the length of an entry point and gives the caller's
// current device back when the entry point returns (device < 0: leaves it alone).
struct DeviceScope {
    int prev = -1;
    cudaError_t status = cudaSuccess;
    explicit DeviceScope(int device)
    {
        if (device < 0) return;
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != device) status = cudaSetDevice(device);
        else prev = -1;   // already current: nothing to restore
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

// Whether two buffers of n floats share an element (compared as addresses).
inline bool ranges_overlap(const float* a, const float* b, size_t n)
{
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    const uintptr_t bytes = (uintptr_t)n * sizeof(float);
    return n != 0 && x < y + bytes && y < x + bytes;
}

// Whether an a-trous output of W*H*3 floats overlaps any of its four inputs: the
// last level writes the output while it still reads the colour and the G-buffer.
inline bool atrous_output_aliases(const float* out, const float* pixels, const float* normals,
                                  const float* positions, const float* diffuse, size_t n3)
{
    return ranges_overlap(out, pixels, n3) || ranges_overlap(out, normals, n3) ||
           ranges_overlap(out, positions, n3) || ranges_overlap(out, diffuse, n3);
}

// A device allocation reused across calls, grown on demand.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t bytes);
    void release();
};

}  // namespace pico

struct pico_gpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;
    pico::DeviceStatus* status = nullptr;   // two status blocks, one per stream
    std::string last_error;
    pico::DeviceBuffer buf_a, buf_b, buf_c, buf_d, buf_e;
    // page-locked bounce buffers for host ranges that are only partly page-locked
    void* bounce_in = nullptr;
    void* bounce_out = nullptr;
    size_t bounce_rays = 0;
    RenderBuffers* render = nullptr;            // wavefront path state and image buffers
    int order = PICO_ORDER_NEAR_FIRST;          // traversal order of every trace in this context
    uint32_t max_iterations = pico::kTraceMaxIter;   // pico_gpu_set_traversal_limits
    uint32_t stack_entries = pico::kTraceStack;
    int triangle_test = PICO_TRIANGLE_MOLLER_TRUMBORE;   // pico_gpu_set_triangle_test
    uint32_t max_paths = 0;   // pico_gpu_set_path_limit; 0: the default (kMaxPaths)
    uint64_t render_stats[5] = {0, 0, 0, 0, 0}; // tallies of the last pico_gpu_render call
    // the last render was pico_gpu_render_device: its tallies are read from the
    // device (after its stream) when asked for
    bool stats_on_device = false;
    cudaStream_t stats_stream = nullptr;
    uint64_t stats_gbuffer_rays = 0;
    pico_gpu_nrc* cache = nullptr;              // radiance cache of PICO_ESTIMATOR_RADIANCE_CACHE renders
    BatchState* batch = nullptr;                // per-render state and streams of pico_gpu_render_many
    pico::LaunchTimer* extend_timer = nullptr;  // pico_gpu_set_render_probe: events around closest-hit launches
    pico::LaunchTimer* shade_timer = nullptr;   // ... and around the shade launches
    bool count_work = false;                    // pico_gpu_set_render_probe: counting closest-hit variant
    pico::DeviceStatus* status2() { return status + 1; }
};

struct pico_gpu_scene {
    pico_gpu_ctx* ctx = nullptr;
    SceneView view{};
    std::vector<void*> allocations;
    std::vector<uint32_t> inst_rank_host;
    std::vector<uint32_t> light_inst_host;
    uint32_t nlights = 0, ninstances = 0;
    // The reference's sphere intersector solves its quadratic as if the object-space
    // direction had unit length, so through a scaled instance it reports points off the
    // sphere, even for rays that miss it (Core/LowerLevelImplicitShapesBVH.cpp:24-52).
    // Which of those the reference returns depends on its own visit order and pruning,
    // so scenes with sphere instances are always traversed in the reference's order.
    bool needs_reference_order = false;
    bool has_btdf = false;   // Transparent or Fresnel instances: the radiance cache has no such lobes
    uint64_t info[6] = {0, 0, 0, 0, 0, 0};
};

namespace pico {
// The traversal order a context uses on a scene.
inline int scene_order(const pico_gpu_ctx* ctx, const pico_gpu_scene* scene)
{
    return scene->needs_reference_order ? PICO_ORDER_REFERENCE : ctx->order;
}
// The scene's view with the context's traversal bounds, as every launch takes it.
inline SceneView traversal_view(const pico_gpu_ctx* ctx, const pico_gpu_scene* scene)
{
    SceneView v = scene->view;
    v.max_iterations = ctx->max_iterations;
    v.stack_entries = ctx->stack_entries;
    v.watertight = ctx->triangle_test == PICO_TRIANGLE_WATERTIGHT ? 1u : 0u;
    return v;
}
int set_error(pico_gpu_ctx* ctx, int code, const std::string& msg);
int cuda_error(pico_gpu_ctx* ctx, cudaError_t e, const char* what);
int take_device_status(pico_gpu_ctx* ctx, cudaStream_t stream);
RenderBuffers* render_buffers(pico_gpu_ctx* ctx);
void free_render_buffers(pico_gpu_ctx* ctx);   // also the render probe's timer
void free_batch_state(pico_gpu_ctx* ctx);
}  // namespace pico
