// Host-side state and launchers of the neural radiance cache.
#pragma once

#include "pico_gpu.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nrc_layout.h"

namespace pico {
namespace nrc {

constexpr uint32_t kMlpParams = kLayers * kWidth * kWidth;   // (layer, out, in); layer 5 uses out rows 0-2

struct AdamStep {
    float lr, beta1, beta2, eps;
    float c1, c2;          // 1 / (1 - beta1^t), 1 / (1 - beta2^t)
};

// One training batch: record j is queries[4 * (offset + j * stride)] with target targets[offset + j * stride].
struct TrainBatch {
    const float4* queries;
    const float4* targets;
    uint32_t n, offset, stride;
};

cudaError_t launch_encode(const GridGeometry& g, const __half2* table, const float4* queries, uint32_t n, float* out,
                          cudaStream_t st);
// How the kernels wait on their mbarriers (bulk copies, tensor-core commits): each
// wait gives up after limit_ns nanoseconds of the device's global timer and the
// kernel reports kErrTimeout.  withheld_bytes > 0 makes the inference kernel's
// weight-load barrier expect that many bytes more than its copy delivers, so that
// its wait runs out (a test of the timeout path; 0 otherwise).
struct WaitPolicy {
    uint64_t limit_ns = 1000000000ull;
    uint32_t withheld_bytes = 0;
};
// Network output for n queries: RGB into out_rgb (n * 3), or, when pay is given,
// pay[q.pad] += thr[q.pad] * max(rgb, 0) for every query q (render mode).  With
// n_dev the count is min(*n_dev, n), read on the device.  `groups` (1, 2 or 4)
// is the number of 128-row tiles each CTA keeps in flight.
cudaError_t launch_infer(const GridGeometry& g, const __half2* table, const uint8_t* weights, const float4* queries,
                         uint32_t n, float* out_rgb, const float4* thr, float4* pay, int* err, cudaStream_t st,
                         const uint32_t* n_dev = nullptr, int groups = 4, const WaitPolicy& wait = WaitPolicy{});
// Gradients of the relative L2 loss over one batch: per-CTA weight-gradient
// partials (kMlpParams floats each, returned count in *parts) and the hash-grid
// gradient (accumulated into grid_grad, which the caller zeroes); adds the mean
// loss to *loss.
cudaError_t launch_train(const GridGeometry& g, const __half2* table, const uint8_t* weights, const TrainBatch& b,
                         float2* grid_grad, float* partial, uint32_t max_parts, uint32_t* parts, float* loss,
                         int* err, cudaStream_t st, const WaitPolicy& wait = WaitPolicy{});
// Sums the partials into grad; with apply, one Adam step on the master weights,
// which are then written as the swizzled bf16 image.
cudaError_t launch_adam_mlp(const float* partial, uint32_t parts, float* master, float* m, float* v, float* grad,
                            uint8_t* image, const AdamStep& s, bool apply, cudaStream_t st);
cudaError_t launch_adam_grid(const float* grad, float* master, float* m, float* v, __half2* table, size_t nfloats,
                             const AdamStep& s, cudaStream_t st);
cudaError_t launch_write_image(const float* master, uint8_t* image, cudaStream_t st);
cudaError_t launch_write_table(const float* master, __half2* table, size_t nfloats, cudaStream_t st);
uint32_t train_grid_size(uint32_t n);

}  // namespace nrc
}  // namespace pico
