// The radiance cache object behind the C ABI.
#pragma once

#include "capi_internal.h"
#include "nrc.h"

#include <vector>

struct pico_gpu_nrc {
    pico_gpu_ctx* ctx = nullptr;
    pico_nrc_config cfg{};
    pico::nrc::GridGeometry geo{};
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    size_t grid_floats = 0;            // levels x entries x 2 features
    uint32_t max_parts = 0;            // weight-gradient partials (one per training CTA)
    uint64_t step = 0;                 // optimiser steps taken
    uint64_t frames = 0;               // frames rendered with the cache
    uint64_t train_passes = 0;         // training-path passes traced (selects their random streams)
    // network: fp32 master weights (layer, out, in), Adam moments, last gradient,
    // per-CTA gradient partials, swizzled bf16 image the kernels load
    float *master = nullptr, *adam_m = nullptr, *adam_v = nullptr, *grad = nullptr, *partial = nullptr;
    uint8_t* image = nullptr;
    // hash grid: fp32 master features, Adam moments, gradient, fp16 table
    float *grid_master = nullptr, *grid_m = nullptr, *grid_v = nullptr, *grid_grad = nullptr;
    __half2* table = nullptr;
    float* loss = nullptr;
    int* err = nullptr;
    pico::nrc::WaitPolicy wait{};      // pico_gpu_nrc_set_wait_limit
    std::vector<void*> allocations;
    // cumulative render work: training paths, training records, optimiser steps, cache queries
    uint64_t render_stats[4] = {0, 0, 0, 0};
};

namespace pico {
namespace nrc {

constexpr uint64_t kMaxQueries = 1ull << 26;
constexpr uint64_t kMaxTrainBatch = 1ull << 20;

void set_geometry(pico_gpu_nrc* c, const float lo[3], const float hi[3]);
AdamStep next_adam_step(pico_gpu_nrc* c);
int train_step(pico_gpu_nrc* c, const TrainBatch& b, bool apply, cudaStream_t st);
int take_status(pico_gpu_nrc* c, cudaStream_t st);

}  // namespace nrc
}  // namespace pico
