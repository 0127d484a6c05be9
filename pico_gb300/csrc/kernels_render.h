// Host-visible state and launchers of the wavefront renderer and denoiser.
#pragma once

#include "kernels.h"
#include "layout.h"
#include "nrc.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace pico {

// Camera::generate_ray inputs plus host-precomputed glm quantities.
struct CameraView {
    float pos[3], dir[3], up[3];
    float res_x, res_y, aspect, far_plane;
    float right[3];                    // cross(normalize(dir), up), glm operation order
    float view[16];                    // glm::lookAt(pos, pos + dir, up), column-major
};

// The device-side plan of one sample round of a render with the early exit on
// (launch_plan_round, launch_compact_pixels): a batch with a plan reads the round's
// pixel count and samples per pixel from it instead of PathBatch::n / npix and the
// spb argument, so that the host enqueues rounds without knowing how many pixels
// are still sampling.
struct RoundPlan {
    uint32_t npix;        // pixels listed for this round (all still sampling)
    uint32_t spb;         // samples per pixel this round (0: the round does nothing)
    uint32_t n;           // paths of the round: npix * spb
    uint32_t scheduled;   // samples per pixel the rounds so far took
    uint32_t next_npix;   // pixels the compaction kept for the next round
    uint32_t pad[3];
};

// Structure-of-arrays path state of one batch (capacity >= n) and the
// per-pixel accumulation buffers of the whole image.
struct PathBatch {
    uint32_t n, npix, width;
    uint32_t extend_ctas;              // closest-hit launches: persistent CTAs per SM (0: as many as fit)
    uint32_t extend_threads;           // closest-hit launches: threads per CTA, 64, 128 or 256 (other: 128)
    uint32_t pad;
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
    // image state (W*H entries)
    float* pixels; float* variance; uint32_t* count; uint32_t* taken; uint32_t* done;
    unsigned long long* sample_tally;  // samples added to the image (set by launch_render_batch)
    const RoundPlan* plan;             // null, or the round's n / npix / spb (n and npix above are then bounds)
};

// Measurement hooks of a render's closest-hit launches: CUDA events recorded on
// the launching stream before and after each one (timer), or work counters
// (count: the counting kernel variant adds nodes, triangles, instance entries
// and nodes inside instances to `counters`).  Both are off in ordinary renders.
struct LaunchTimer {
    std::vector<cudaEvent_t> events;   // before / after pairs, reused across renders
    size_t used = 0;
    cudaError_t record(cudaStream_t st);
    // Sum of the recorded launches' durations (ms) and their number; the events
    // must have completed.
    cudaError_t total(double& ms, uint64_t& launches) const;
    void reset() { used = 0; }
    ~LaunchTimer();
};
struct RenderProbe {
    LaunchTimer* timer;
    unsigned long long* counters;      // 4 counters, or null
    LaunchTimer* shade_timer;          // events around the shade launches, or null
};

// What the physical shade step does for the radiance cache.
//   kNrcRecord     every shaded vertex of a training path appends a record: the
//                  cache query (4 float4), then the path throughput and payload
//                  on arrival (2 float4 in rec_tp), from which the radiance the
//                  rest of the path reflects there is (final payload - payload)
//                  / throughput;
//   kNrcTerminate  a camera path stops at its vertex after one bounce (after two
//                  when the first vertex has roughness < 0.1) and appends that
//                  vertex's query; the cache's answer times the throughput is
//                  added to the payload after the depth loop.
enum NrcMode { kNrcOff = 0, kNrcRecord = 1, kNrcTerminate = 2 };
struct NrcShadeArgs {
    int mode;
    uint32_t capacity;        // entries of queries / rec_tp
    uint32_t bounces;         // kNrcTerminate: bounces before the cache answers (one more behind a glossy vertex)
    float4* queries;          // 4 float4 per entry (pico_nrc_query)
    float4* rec_tp;           // kNrcRecord: 2 float4 per entry
    uint32_t* count;          // entries appended
    float* prev_rough;        // kNrcTerminate: per path, roughness of its previous vertex
    // the cache the terminating paths query
    nrc::GridGeometry geo;
    const __half2* table;
    const uint8_t* weights;
    int* err;
    int infer_groups;
    nrc::WaitPolicy wait;
};

cudaError_t launch_render_batch(const SceneView& sc, PathBatch& b, const CameraView& cam, unsigned long long seed,
                                uint32_t spb, uint32_t max_depth, uint32_t max_samples, float max_variance,
                                int estimator, DeviceStatus* status, int order, cudaStream_t st,
                                const NrcShadeArgs* nrc = nullptr, const RenderProbe* probe = nullptr);
// Exit-aware rounds: plan_init lists npix pixels for the first round; plan_round
// sets the next round from the pixels the compaction kept: samples per pixel
// min(max_samples - scheduled, max_paths / pixels, cap), at most first_cap in the
// first round; compact_pixels keeps the pixels of `in` (plan->npix of them) that
// are not done, in `out`, counting them in plan->next_npix.
cudaError_t launch_plan_init(RoundPlan* plan, uint32_t npix, cudaStream_t st);
cudaError_t launch_plan_round(RoundPlan* plan, uint32_t max_samples, uint32_t first_cap, uint32_t cap,
                              uint32_t max_paths, cudaStream_t st);
cudaError_t launch_compact_pixels(RoundPlan* plan, const uint32_t* in, const uint32_t* done, uint32_t* out,
                                  uint32_t npix_bound, cudaStream_t st);
// The image state of a render into caller device buffers: every pixel listed in
// order, done where count >= max_samples, nothing taken yet.
cudaError_t launch_prepare_image(const uint32_t* count, uint32_t npx, uint32_t max_samples, uint32_t* pix_list,
                                 uint32_t* done, uint32_t* taken, cudaStream_t st);
// The radiance cache's training paths of one sample pass: n full-depth physical
// paths from pseudo-random pixels of the W x H image (path slots 0 .. n-1 of b),
// recording every shaded vertex (kNrcRecord), then the records' targets
// (4 floats each) in `targets`.
cudaError_t launch_training_paths(const SceneView& sc, PathBatch& b, const CameraView& cam, unsigned long long seed,
                                  uint32_t frame, uint32_t n, uint32_t W, uint32_t H, uint32_t max_depth,
                                  const NrcShadeArgs& nrc, float4* targets, DeviceStatus* status, int order,
                                  cudaStream_t st);
// Writes the device's global nanosecond timer to *dst when the stream reaches it.
cudaError_t launch_stamp(unsigned long long* dst, cudaStream_t st);
cudaError_t launch_gbuffer(const SceneView& sc, const CameraView& cam, uint32_t W, uint32_t H, float* normals,
                           float* positions, float* diffuse, DeviceStatus* status, int order, cudaStream_t st);
// Floats of a-trous statistics scratch for a W x H image (beyond its two ping-pong
// images): per 64 x 64 tile four partial white points (one per CTA of a level's
// statistics launch) and the five levels' (min, max) |position| ranges, then per
// image row and tile column the five levels' (min, max) row ranges.
inline size_t atrous_stats_floats(uint32_t W, uint32_t H)
{
    const size_t tx = (W + 63) / 64, ty = (H + 63) / 64;
    return tx * ty * (4 + 5 * 2) + (size_t)5 * 2 * H * tx;
}
cudaError_t launch_atrous(const float* pixels, const float* normals, const float* positions, const float* diffuse,
                          uint32_t W, uint32_t H, float* scratch_a, float* scratch_b, float* tile_stats, float* out,
                          cudaStream_t st);
cudaError_t launch_reinhard(float* pixels, uint32_t W, uint32_t H, unsigned* scratch, cudaStream_t st);

}  // namespace pico
