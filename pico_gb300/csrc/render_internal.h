// Render state shared by the single-render and batched-render entry points.
#pragma once

#include "capi_internal.h"
#include "kernels_render.h"

// Path state and image buffers of one render, grown on demand.
struct RenderBuffers {
    pico::DeviceBuffer org, dir, thr, pay, hit, hit_tri, rng, depth, ior_n, ior_lo, ior_hi, sorg, sdir, scontrib,
        senergy, q0, q1, sq, counters;
    pico::DeviceBuffer pixels, variance, count, taken, done, pix_list;
    pico::DeviceBuffer pix_list2, plan;   // exit-aware rounds: the compacted pixel list, the round plan
    pico::DeviceBuffer gn, gp, gd, ga, gb, stats, out, tonemap;
    // radiance cache: terminal queries / training records, record throughput and
    // payload, targets, previous roughness per path, entry counters
    pico::DeviceBuffer nrc_q, nrc_tp, nrc_tgt, nrc_prev, nrc_count;
    ~RenderBuffers()
    {
        for (pico::DeviceBuffer* b : {&org, &dir, &thr, &pay, &hit, &hit_tri, &rng, &depth, &ior_n, &ior_lo, &ior_hi,
                                      &sorg, &sdir, &scontrib, &senergy, &q0, &q1, &sq, &counters, &pixels,
                                      &variance, &count, &taken, &done, &pix_list, &pix_list2, &plan, &gn, &gp, &gd,
                                      &ga, &gb, &stats,
                                      &out, &tonemap, &nrc_q, &nrc_tp, &nrc_tgt, &nrc_prev, &nrc_count})
            b->release();
    }
};

namespace pico {

// Paths of one batch of a single render (pixels x samples; 208 B of path state
// each, 14 GB at the limit).  Larger batches amortise each launch and its
// tail: a 1080p render at 64 spp measured 159 / 206 / 267 / 279 / 286 Msamples/s
// with batches of 2^19 / 2^20 / 2^22 / 2^23 / 2^24 paths (physical estimator),
// and 2^25 / 2^26 took the 1080p renders 1.4 / 2.5 % (reference estimator) and
// 1.4 / 2.0 % (physical) below 2^24's time.
constexpr uint32_t kMaxPaths = 1u << 26;
// Device bytes of path state per path that reserve_paths allocates: eleven float4
// arrays, six uint32 arrays and the 64-bit random state.
constexpr size_t kPathStateBytes = 11 * 16 + 6 * 4 + 8;

template <class T>
T* as(DeviceBuffer& b) { return static_cast<T*>(b.ptr); }

// Camera::getRight (Core/Camera.hpp:64-65) and Camera::getViewMatrix (glm::lookAtRH).
CameraView make_camera_view(const pico_camera& c);
cudaError_t reserve_paths(RenderBuffers& r, size_t n);
// The path state of a batch of n paths over npix listed pixels, in r's buffers.
PathBatch make_batch(RenderBuffers& r, uint32_t n, uint32_t npix, uint32_t W, const uint32_t* pix_list);

}  // namespace pico
