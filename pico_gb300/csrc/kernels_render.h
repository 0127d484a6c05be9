// Host-visible state and launchers of the wavefront renderer and denoiser.
#pragma once

#include "kernels.h"
#include "layout.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pico {

// Camera::generate_ray inputs plus host-precomputed glm quantities.
struct CameraView {
    float pos[3], dir[3], up[3];
    float res_x, res_y, aspect, far_plane;
    float right[3];                    // cross(normalize(dir), up), glm operation order
    float view[16];                    // glm::lookAt(pos, pos + dir, up), column-major
};

// Structure-of-arrays path state of one batch (capacity >= n) and the
// per-pixel accumulation buffers of the whole image.
struct PathBatch {
    uint32_t n, npix, width, pad;
    const uint32_t* pix_list;          // npix pixel indices
    float4* org; float4* dir; float4* thr; float4* pay;
    float4* hit; uint32_t* hit_tri;
    unsigned long long* rng;
    uint32_t* depth;
    uint32_t* ior_n; float4* ior_lo; float4* ior_hi;   // index-of-refraction stack: size, entries 0-3, 4-7
    float4* sorg; float4* sdir; float4* scontrib; float4* senergy;
    uint32_t* queue[2];
    uint32_t* shadow_queue;
    uint32_t* counters;                // [0], [1]: path queues, [2]: shadow queue
    float4* samples;                   // per path: final radiance
    // image state (W*H entries)
    float* pixels; float* variance; uint32_t* count; uint32_t* taken; uint32_t* done;
};

cudaError_t launch_render_batch(const SceneView& sc, PathBatch& b, const CameraView& cam, unsigned long long seed,
                                uint32_t spb, uint32_t max_depth, uint32_t max_samples, float max_variance,
                                int estimator, DeviceStatus* status, int order, cudaStream_t st);
cudaError_t launch_gbuffer(const SceneView& sc, const CameraView& cam, uint32_t W, uint32_t H, float* normals,
                           float* positions, float* diffuse, DeviceStatus* status, int order, cudaStream_t st);
// Floats of a-trous scratch per 64 x 64 tile: four partial statistics records
// (white point, min |position|, max |position|, unused) per level.
constexpr size_t kAtrousStatsFloatsPerTile = 16;
cudaError_t launch_atrous(const float* pixels, const float* normals, const float* positions, const float* diffuse,
                          uint32_t W, uint32_t H, float* scratch_a, float* scratch_b, float* tile_stats, float* out,
                          cudaStream_t st);
cudaError_t launch_reinhard(float* pixels, uint32_t W, uint32_t H, unsigned* scratch, cudaStream_t st);

}  // namespace pico
