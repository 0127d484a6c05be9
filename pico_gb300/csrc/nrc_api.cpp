// The C ABI of the neural radiance cache (no counterpart in the reference):
// parameters and optimiser state in device memory, inference and training
// entry points on host or device buffers.
#include "capi_internal.h"
#include "nrc.h"
#include "nrc_internal.h"

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace pico;
using namespace pico::nrc;

namespace {

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

float uniform01(uint64_t& s) { return (float)((splitmix64(s) >> 40) * (1.0 / 16777216.0)); }

bool valid_config(const pico_nrc_config& c, std::string& why)
{
    if (c.log2_table_size < 10 || c.log2_table_size > 22) { why = "log2_table_size must lie in [10, 22]"; return false; }
    if (!(c.base_resolution >= 1.0f) || !(c.max_resolution >= c.base_resolution)) {
        why = "resolutions must satisfy 1 <= base_resolution <= max_resolution";
        return false;
    }
    if (!(c.learning_rate > 0.0f) || !(c.beta1 >= 0.0f && c.beta1 < 1.0f) || !(c.beta2 >= 0.0f && c.beta2 < 1.0f) ||
        !(c.epsilon > 0.0f)) {
        why = "invalid optimiser settings";
        return false;
    }
    if (c.train_batch == 0 || c.train_batch > kMaxTrainBatch) { why = "train_batch must lie in [1, 2^20]"; return false; }
    if (c.bounces < 1 || c.bounces > 8) { why = "bounces must lie in [1, 8]"; return false; }
    if (c.infer_groups != 0 && c.infer_groups != 1 && c.infer_groups != 2 && c.infer_groups != 4) {
        why = "infer_groups must be 0, 1, 2 or 4";
        return false;
    }
    return true;
}

}  // namespace

namespace pico {
namespace nrc {

void set_geometry(pico_gpu_nrc* c, const float lo[3], const float hi[3])
{
    GridGeometry& g = c->geo;
    const pico_nrc_config& cfg = c->cfg;
    const uint32_t T = 1u << cfg.log2_table_size;
    const double b = kLevels > 1 ? std::exp((std::log((double)cfg.max_resolution) -
                                             std::log((double)cfg.base_resolution)) / (kLevels - 1))
                                 : 1.0;
    for (int l = 0; l < kLevels; ++l) {
        const float s = (float)((double)cfg.base_resolution * std::pow(b, (double)l));
        g.scale[l] = s;
        const uint64_t r1 = (uint64_t)std::floor(s) + 2;
        g.res1[l] = (r1 * r1 * r1 <= T) ? (uint32_t)r1 : 0u;
    }
    g.table_mask = T - 1;
    g.log2_table = cfg.log2_table_size;
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = lo[a];
        const float ext = hi[a] - lo[a];
        g.inv_extent[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
        c->lo[a] = lo[a];
        c->hi[a] = hi[a];
    }
}

AdamStep next_adam_step(pico_gpu_nrc* c)
{
    ++c->step;
    AdamStep s;
    s.lr = c->cfg.learning_rate;
    s.beta1 = c->cfg.beta1;
    s.beta2 = c->cfg.beta2;
    s.eps = c->cfg.epsilon;
    s.c1 = (float)(1.0 / (1.0 - std::pow((double)c->cfg.beta1, (double)c->step)));
    s.c2 = (float)(1.0 / (1.0 - std::pow((double)c->cfg.beta2, (double)c->step)));
    return s;
}

// One optimiser step (apply) or only the gradients on a device batch, on `st`.
int train_step(pico_gpu_nrc* c, const TrainBatch& b, bool apply, cudaStream_t st)
{
    pico_gpu_ctx* ctx = c->ctx;
    cudaError_t e = cudaMemsetAsync(c->grid_grad, 0, c->grid_floats * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->loss, 0, sizeof(float), st);
    uint32_t parts = 0;
    if (e == cudaSuccess)
        e = launch_train(c->geo, c->table, c->image, b, reinterpret_cast<float2*>(c->grid_grad), c->partial,
                         c->max_parts, &parts, c->loss, c->err, st, c->wait);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache training");
    const AdamStep s = apply ? next_adam_step(c) : AdamStep{};
    if (parts > 0) e = launch_adam_mlp(c->partial, parts, c->master, c->adam_m, c->adam_v, c->grad, c->image, s, apply, st);
    else e = cudaMemsetAsync(c->grad, 0, kMlpParams * sizeof(float), st);
    if (e == cudaSuccess && apply)
        e = launch_adam_grid(c->grid_grad, c->grid_master, c->grid_m, c->grid_v, c->table, c->grid_floats, s, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache optimiser");
    return PICO_OK;
}

int take_status(pico_gpu_nrc* c, cudaStream_t st)
{
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, c->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(c->ctx, e, "radiance cache status");
    if (err) {
        cudaMemsetAsync(c->err, 0, sizeof(int), st);
        cudaStreamSynchronize(st);
        return set_error(c->ctx, PICO_ERR_TIMEOUT, "a radiance cache kernel timed out waiting for its tensor cores");
    }
    return PICO_OK;
}

}  // namespace nrc
}  // namespace pico

extern "C" {

int pico_gpu_nrc_default_config(pico_nrc_config* out)
{
    if (!out) return PICO_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof *out);
    out->log2_table_size = 19;
    out->base_resolution = 16.0f;
    out->max_resolution = 4096.0f;
    out->learning_rate = 1e-2f;
    out->beta1 = 0.9f;
    out->beta2 = 0.99f;
    out->epsilon = 1e-15f;
    out->train_paths = 1u << 16;
    out->train_batch = 1u << 16;
    out->max_train_steps = 4;
    out->warmup_frames = 0;
    out->seed = 1;
    out->bounces = 1;
    return PICO_OK;
}

int pico_gpu_nrc_create(pico_gpu_ctx* ctx, const pico_nrc_config* cfg, pico_gpu_nrc** out)
{
    if (!ctx || !cfg || !out) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::string why;
    if (!valid_config(*cfg, why)) return set_error(ctx, PICO_ERR_INVALID_ARG, why);
    const DeviceScope device_scope(ctx->device);
    auto* c = new (std::nothrow) pico_gpu_nrc();
    if (!c) return set_error(ctx, PICO_ERR_OUT_OF_MEMORY, "host allocation");
    c->ctx = ctx;
    c->cfg = *cfg;
    c->grid_floats = (size_t)kLevels * ((size_t)1 << cfg->log2_table_size) * 2;
    c->max_parts = (uint32_t)sm_count();
    set_geometry(c, cfg->aabb_min, cfg->aabb_max);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto*& p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p), bytes);
        if (e == cudaSuccess) c->allocations.push_back(p);
    };
    alloc(c->master, kMlpParams * sizeof(float));
    alloc(c->adam_m, kMlpParams * sizeof(float));
    alloc(c->adam_v, kMlpParams * sizeof(float));
    alloc(c->grad, kMlpParams * sizeof(float));
    alloc(c->partial, (size_t)c->max_parts * kMlpParams * sizeof(float));
    alloc(c->image, kWeightBytes);
    alloc(c->grid_master, c->grid_floats * sizeof(float));
    alloc(c->grid_m, c->grid_floats * sizeof(float));
    alloc(c->grid_v, c->grid_floats * sizeof(float));
    alloc(c->grid_grad, c->grid_floats * sizeof(float));
    alloc(c->table, c->grid_floats * sizeof(__half));
    alloc(c->loss, sizeof(float));
    alloc(c->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->err, 0, sizeof(int));
    if (e != cudaSuccess) {
        pico_gpu_nrc_free(c);
        return cuda_error(ctx, e, "radiance cache allocation");
    }
    // seeded initial parameters: Xavier-uniform weights, grid features uniform in [-1e-4, 1e-4]
    uint64_t s = cfg->seed;
    std::vector<float> mlp(kMlpParams, 0.0f);
    for (int l = 0; l < kLayers; ++l) {
        const int outs = l < kHidden ? kWidth : kOutputs;
        const float a = std::sqrt(6.0f / (float)(kWidth + outs));
        for (int o = 0; o < outs; ++o)
            for (int i = 0; i < kWidth; ++i)
                mlp[((size_t)l * kWidth + o) * kWidth + i] = (2.0f * uniform01(s) - 1.0f) * a;
    }
    std::vector<float> grid(c->grid_floats);
    for (float& x : grid) x = (2.0f * uniform01(s) - 1.0f) * 1e-4f;
    const int st = pico_gpu_nrc_set_params(c, mlp.data(), grid.data());
    if (st != PICO_OK) {
        pico_gpu_nrc_free(c);
        return st;
    }
    *out = c;
    return PICO_OK;
}

void pico_gpu_nrc_free(pico_gpu_nrc* c)
{
    if (!c) return;
    const DeviceScope device_scope(c->ctx->device);
    if (c->ctx->cache == c) c->ctx->cache = nullptr;
    for (void* p : c->allocations) cudaFree(p);
    delete c;
}

int pico_gpu_nrc_set_params(pico_gpu_nrc* c, const float* mlp, const float* grid)
{
    if (!c || !mlp || !grid) return PICO_ERR_INVALID_ARG;
    pico_gpu_ctx* ctx = c->ctx;
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    std::vector<float> w(mlp, mlp + kMlpParams);
    for (int o = kOutputs; o < kWidth; ++o)
        for (int i = 0; i < kWidth; ++i) w[((size_t)kHidden * kWidth + o) * kWidth + i] = 0.0f;
    cudaError_t e = cudaMemcpyAsync(c->master, w.data(), kMlpParams * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->grid_master, grid, c->grid_floats * sizeof(float),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->adam_m, 0, kMlpParams * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->adam_v, 0, kMlpParams * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->grad, 0, kMlpParams * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->grid_m, 0, c->grid_floats * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->grid_v, 0, c->grid_floats * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->grid_grad, 0, c->grid_floats * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->image, 0, kWeightBytes, st);
    if (e == cudaSuccess) e = launch_write_image(c->master, c->image, st);
    if (e == cudaSuccess) e = launch_write_table(c->grid_master, c->table, c->grid_floats, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache parameters");
    c->step = 0;
    return PICO_OK;
}

int pico_gpu_nrc_get_params(pico_gpu_nrc* c, float* mlp, float* grid)
{
    if (!c) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(c->ctx->device);
    cudaStream_t st = c->ctx->stream;
    cudaError_t e = cudaSuccess;
    if (mlp) e = cudaMemcpyAsync(mlp, c->master, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && grid)
        e = cudaMemcpyAsync(grid, c->grid_master, c->grid_floats * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(c->ctx, e, "radiance cache parameters");
    return PICO_OK;
}

int pico_gpu_nrc_set_bounds(pico_gpu_nrc* c, const float* aabb_min, const float* aabb_max)
{
    if (!c || !aabb_min || !aabb_max) return PICO_ERR_INVALID_ARG;
    set_geometry(c, aabb_min, aabb_max);
    return PICO_OK;
}

int pico_gpu_nrc_info(const pico_gpu_nrc* c, uint64_t* out4)
{
    if (!c || !out4) return PICO_ERR_INVALID_ARG;
    out4[0] = c->step;
    out4[1] = (uint64_t)c->grid_floats / 2;
    out4[2] = kMlpParams;
    out4[3] = c->frames;
    return PICO_OK;
}

int pico_gpu_nrc_stats(const pico_gpu_nrc* c, uint64_t* out4)
{
    if (!c || !out4) return PICO_ERR_INVALID_ARG;
    for (int k = 0; k < 4; ++k) out4[k] = c->render_stats[k];
    return PICO_OK;
}

int pico_gpu_nrc_encode(pico_gpu_nrc* c, const pico_nrc_query* q, uint64_t n, float* out)
{
    if (!c || (n && (!q || !out))) return PICO_ERR_INVALID_ARG;
    if (n > kMaxQueries) return set_error(c->ctx, PICO_ERR_INVALID_ARG, "too many queries");
    pico_gpu_ctx* ctx = c->ctx;
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    cudaError_t e = ctx->buf_a.reserve(n * sizeof(pico_nrc_query) + 16);
    if (e == cudaSuccess) e = ctx->buf_b.reserve(n * kWidth * sizeof(float) + 16);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(ctx->buf_a.ptr, q, n * sizeof(pico_nrc_query), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_encode(c->geo, c->table, static_cast<const float4*>(ctx->buf_a.ptr), (uint32_t)n,
                                            static_cast<float*>(ctx->buf_b.ptr), st);
    if (e == cudaSuccess && n)
        e = cudaMemcpyAsync(out, ctx->buf_b.ptr, n * kWidth * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache encoding");
    return PICO_OK;
}

int pico_gpu_nrc_infer_device(pico_gpu_nrc* c, const pico_nrc_query* d_q, uint64_t n, float* d_rgb, void* stream)
{
    if (!c || (n && (!d_q || !d_rgb))) return PICO_ERR_INVALID_ARG;
    if (n > kMaxQueries) return set_error(c->ctx, PICO_ERR_INVALID_ARG, "too many queries");
    const DeviceScope device_scope(c->ctx->device);
    cudaError_t e = launch_infer(c->geo, c->table, c->image, reinterpret_cast<const float4*>(d_q), (uint32_t)n, d_rgb,
                                 nullptr, nullptr, c->err, static_cast<cudaStream_t>(stream), nullptr,
                                 (int)c->cfg.infer_groups, c->wait);
    if (e != cudaSuccess) return cuda_error(c->ctx, e, "radiance cache inference");
    return PICO_OK;
}

int pico_gpu_nrc_set_wait_limit(pico_gpu_nrc* c, uint64_t limit_ns, uint32_t withheld_bytes)
{
    if (!c) return PICO_ERR_INVALID_ARG;
    if (limit_ns == 0 || withheld_bytes > 1024 || withheld_bytes % 16)
        return set_error(c->ctx, PICO_ERR_INVALID_ARG,
                         "wait limit: a positive time, and at most 1024 withheld bytes in multiples of 16");
    c->wait.limit_ns = limit_ns;
    c->wait.withheld_bytes = withheld_bytes;
    return PICO_OK;
}

int pico_gpu_nrc_infer(pico_gpu_nrc* c, const pico_nrc_query* q, uint64_t n, float* rgb)
{
    if (!c || (n && (!q || !rgb))) return PICO_ERR_INVALID_ARG;
    if (n > kMaxQueries) return set_error(c->ctx, PICO_ERR_INVALID_ARG, "too many queries");
    pico_gpu_ctx* ctx = c->ctx;
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    cudaError_t e = ctx->buf_a.reserve(n * sizeof(pico_nrc_query) + 16);
    if (e == cudaSuccess) e = ctx->buf_b.reserve(n * 3 * sizeof(float) + 16);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(ctx->buf_a.ptr, q, n * sizeof(pico_nrc_query), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache upload");
    int status = pico_gpu_nrc_infer_device(c, static_cast<const pico_nrc_query*>(ctx->buf_a.ptr), n,
                                           static_cast<float*>(ctx->buf_b.ptr), st);
    if (status != PICO_OK) return status;
    if (n) e = cudaMemcpyAsync(rgb, ctx->buf_b.ptr, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache download");
    return take_status(c, st);
}

int pico_gpu_nrc_train_device(pico_gpu_nrc* c, const pico_nrc_query* d_q, const float* d_targets, uint64_t n,
                              int apply, void* stream)
{
    if (!c || (n && (!d_q || !d_targets))) return PICO_ERR_INVALID_ARG;
    if (n > kMaxTrainBatch) return set_error(c->ctx, PICO_ERR_INVALID_ARG, "a training batch holds at most 2^20 records");
    const DeviceScope device_scope(c->ctx->device);
    TrainBatch b{reinterpret_cast<const float4*>(d_q), reinterpret_cast<const float4*>(d_targets), (uint32_t)n, 0, 1};
    return train_step(c, b, apply != 0, static_cast<cudaStream_t>(stream));
}

int pico_gpu_nrc_train(pico_gpu_nrc* c, const pico_nrc_query* q, const float* targets, uint64_t n, int apply,
                       float* loss)
{
    if (!c || (n && (!q || !targets))) return PICO_ERR_INVALID_ARG;
    if (n > kMaxTrainBatch) return set_error(c->ctx, PICO_ERR_INVALID_ARG, "a training batch holds at most 2^20 records");
    pico_gpu_ctx* ctx = c->ctx;
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    std::vector<float> t4(n * 4, 0.0f);
    for (uint64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) t4[4 * i + k] = targets[3 * i + k];
    cudaError_t e = ctx->buf_a.reserve(n * sizeof(pico_nrc_query) + 16);
    if (e == cudaSuccess) e = ctx->buf_b.reserve(n * 4 * sizeof(float) + 16);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(ctx->buf_a.ptr, q, n * sizeof(pico_nrc_query), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(ctx->buf_b.ptr, t4.data(), n * 4 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache upload");
    int status = pico_gpu_nrc_train_device(c, static_cast<const pico_nrc_query*>(ctx->buf_a.ptr),
                                           static_cast<const float*>(ctx->buf_b.ptr), n, apply, st);
    if (status != PICO_OK) return status;
    float l = 0.0f;
    e = cudaMemcpyAsync(&l, c->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache training");
    if (loss) *loss = l;
    return take_status(c, st);
}

int pico_gpu_nrc_gradients(pico_gpu_nrc* c, float* mlp_grad, float* grid_grad)
{
    if (!c) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(c->ctx->device);
    cudaStream_t st = c->ctx->stream;
    cudaError_t e = cudaSuccess;
    if (mlp_grad) e = cudaMemcpyAsync(mlp_grad, c->grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && grid_grad)
        e = cudaMemcpyAsync(grid_grad, c->grid_grad, c->grid_floats * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(c->ctx, e, "radiance cache gradients");
    return PICO_OK;
}

int pico_gpu_set_radiance_cache(pico_gpu_ctx* ctx, pico_gpu_nrc* cache)
{
    if (!ctx) return PICO_ERR_INVALID_ARG;
    if (cache && cache->ctx != ctx) return set_error(ctx, PICO_ERR_INVALID_ARG, "the cache belongs to another context");
    ctx->cache = cache;
    return PICO_OK;
}

}  // extern "C"
