// Scene::render_scene_to_memory (Core/Scene.cpp:143-235) on the device, plus the
// denoiser entry points.
//
// The caller's progressive buffers (mean, sample count, variance per pixel) are
// copied in, advanced by up to max_samples samples per pixel with the
// reference's running mean / variance and early-exit rule, and copied back.
// Pixels whose count already reaches max_samples are skipped, as the
// reference's tile loop skips them.  Samples run as batches of at most 16M
// paths (pixels x samples), each pixel's samples in order across batches; the
// cancel flag is polled between batches.  When requested, the a-trous pass
// then runs on the result and replaces it (Scene.cpp:212-234).
// pico_gpu_render_device does the same on caller device buffers, asynchronously
// on the caller's stream (no host copies, no cancel flag).
#include "nrc_internal.h"
#include "render_internal.h"

#include <cmath>
#include <cstring>

using namespace pico;

namespace {

// glm-order float helpers for the host-side camera quantities.
float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
void cross3(const float* a, const float* b, float* o)
{
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}
void normalize3(const float* a, float* o)
{
    const float s = 1.0f / std::sqrt(dot3(a, a));
    o[0] = a[0] * s; o[1] = a[1] * s; o[2] = a[2] * s;
}

}  // namespace

namespace pico {

CameraView make_camera_view(const pico_camera& c)
{
    CameraView v{};
    for (int a = 0; a < 3; ++a) { v.pos[a] = c.position[a]; v.dir[a] = c.direction[a]; v.up[a] = c.up[a]; }
    v.res_x = (float)c.resolution[0];
    v.res_y = (float)c.resolution[1];
    v.aspect = c.aspect;
    v.far_plane = c.far_plane;
    float nd[3];
    normalize3(c.direction, nd);
    cross3(nd, c.up, v.right);
    const float center[3] = {c.position[0] + c.direction[0], c.position[1] + c.direction[1],
                             c.position[2] + c.direction[2]};
    const float fd[3] = {center[0] - c.position[0], center[1] - c.position[1], center[2] - c.position[2]};
    float f[3], s[3], u[3], sc[3];
    normalize3(fd, f);
    cross3(f, c.up, sc);
    normalize3(sc, s);
    cross3(s, f, u);
    float m[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    m[0][0] = s[0]; m[1][0] = s[1]; m[2][0] = s[2];
    m[0][1] = u[0]; m[1][1] = u[1]; m[2][1] = u[2];
    m[0][2] = -f[0]; m[1][2] = -f[1]; m[2][2] = -f[2];
    m[3][0] = -dot3(s, c.position); m[3][1] = -dot3(u, c.position); m[3][2] = dot3(f, c.position);
    std::memcpy(v.view, m, sizeof m);
    return v;
}

RenderBuffers* render_buffers(pico_gpu_ctx* ctx)
{
    if (!ctx->render) ctx->render = new RenderBuffers();
    return ctx->render;
}
void free_render_buffers(pico_gpu_ctx* ctx)
{
    delete ctx->render;
    ctx->render = nullptr;
    delete ctx->extend_timer;
    ctx->extend_timer = nullptr;
    delete ctx->shade_timer;
    ctx->shade_timer = nullptr;
}

cudaError_t reserve_paths(RenderBuffers& r, size_t n)
{
    cudaError_t e = cudaSuccess;
    for (DeviceBuffer* b : {&r.org, &r.dir, &r.thr, &r.pay, &r.hit, &r.sorg, &r.sdir, &r.scontrib, &r.senergy,
                            &r.ior_lo, &r.ior_hi})
        if (e == cudaSuccess) e = b->reserve(n * sizeof(float4));
    for (DeviceBuffer* b : {&r.hit_tri, &r.depth, &r.ior_n, &r.q0, &r.q1, &r.sq})
        if (e == cudaSuccess) e = b->reserve(n * sizeof(uint32_t));
    if (e == cudaSuccess) e = r.rng.reserve(n * sizeof(unsigned long long));
    if (e == cudaSuccess) e = r.counters.reserve(4 * sizeof(uint32_t));
    return e;
}

PathBatch make_batch(RenderBuffers& r, uint32_t n, uint32_t npix, uint32_t W, const uint32_t* pix_list)
{
    PathBatch b{};
    b.n = n; b.npix = npix; b.width = W;
    b.pix_list = pix_list;
    b.org = as<float4>(r.org); b.dir = as<float4>(r.dir); b.thr = as<float4>(r.thr);
    b.pay = as<float4>(r.pay); b.hit = as<float4>(r.hit); b.hit_tri = as<uint32_t>(r.hit_tri);
    b.rng = as<unsigned long long>(r.rng); b.depth = as<uint32_t>(r.depth);
    b.ior_n = as<uint32_t>(r.ior_n); b.ior_lo = as<float4>(r.ior_lo); b.ior_hi = as<float4>(r.ior_hi);
    b.sorg = as<float4>(r.sorg); b.sdir = as<float4>(r.sdir); b.scontrib = as<float4>(r.scontrib);
    b.senergy = as<float4>(r.senergy); b.queue[0] = as<uint32_t>(r.q0); b.queue[1] = as<uint32_t>(r.q1);
    b.shadow_queue = as<uint32_t>(r.sq); b.counters = as<uint32_t>(r.counters);
    b.pixels = as<float>(r.pixels); b.variance = as<float>(r.variance); b.count = as<uint32_t>(r.count);
    b.taken = as<uint32_t>(r.taken); b.done = as<uint32_t>(r.done);
    return b;
}

}  // namespace pico

namespace {

int run_atrous(pico_gpu_ctx* ctx, RenderBuffers& r, const float* d_pix, const float* d_n, const float* d_p,
               const float* d_d, uint32_t W, uint32_t H, float* d_out, cudaStream_t st)
{
    const size_t n = (size_t)W * H * 3;
    cudaError_t e = r.ga.reserve(n * sizeof(float));
    if (e == cudaSuccess) e = r.gb.reserve(n * sizeof(float));
    if (e == cudaSuccess) e = r.stats.reserve(atrous_stats_floats(W, H) * sizeof(float));
    if (e == cudaSuccess)
        e = launch_atrous(d_pix, d_n, d_p, d_d, W, H, as<float>(r.ga), as<float>(r.gb), as<float>(r.stats), d_out, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "a-trous");
    return PICO_OK;
}

bool valid_camera(const pico_camera* c) { return c && c->resolution[0] > 0 && c->resolution[1] > 0; }

// PICO_ESTIMATOR_RADIANCE_CACHE: warmup_frames training-only passes, then per
// sample pass the cache trains on train_paths full-depth physical paths (at most
// max_train_steps optimiser steps of at most train_batch records, spread over all
// records of the pass) and every active pixel takes one sample whose path ends
// in the cache.  The pixel list is on the device already.
// Paths a render's batch may hold: the context's limit, else kMaxPaths.
static uint32_t path_limit(const pico_gpu_ctx* ctx) { return ctx->max_paths ? ctx->max_paths : kMaxPaths; }

int render_with_cache(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, pico_gpu_nrc* c, const pico_render_config* cfg,
                      const CameraView& cam, RenderBuffers& r, size_t nactive, const volatile int32_t* should_quit,
                      bool& cancelled)
{
    cudaStream_t st = ctx->stream;
    const uint32_t W = cfg->width, H = cfg->height;
    const uint32_t chunk_pix = (uint32_t)std::min<size_t>(nactive, path_limit(ctx));
    const uint32_t ntrain = std::min<uint32_t>(c->cfg.train_paths, path_limit(ctx));
    const uint32_t max_depth = cfg->max_ray_depth;
    const size_t rec_cap = (size_t)ntrain * std::max(max_depth, 1u);
    const size_t q_cap = std::max<size_t>(chunk_pix, rec_cap);
    const size_t slots = std::max<size_t>(chunk_pix, ntrain);
    cudaError_t e = reserve_paths(r, slots);
    if (e == cudaSuccess) e = r.nrc_q.reserve(q_cap * sizeof(pico_nrc_query));
    if (e == cudaSuccess) e = r.nrc_tp.reserve(rec_cap * 2 * sizeof(float4));
    if (e == cudaSuccess) e = r.nrc_tgt.reserve(rec_cap * sizeof(float4));
    if (e == cudaSuccess) e = r.nrc_prev.reserve(slots * sizeof(float));
    if (e == cudaSuccess) e = r.nrc_count.reserve(4 * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache render buffers");
    if (!(c->hi[0] > c->lo[0] || c->hi[1] > c->lo[1] || c->hi[2] > c->lo[2]))
        nrc::set_geometry(c, scene->view.tlas_fast_lo, scene->view.tlas_fast_hi);

    NrcShadeArgs na{};
    na.queries = as<float4>(r.nrc_q);
    na.rec_tp = as<float4>(r.nrc_tp);
    na.count = as<uint32_t>(r.nrc_count);
    na.prev_rough = as<float>(r.nrc_prev);
    na.geo = c->geo;
    na.table = c->table;
    na.weights = c->image;
    na.err = c->err;
    na.bounces = c->cfg.bounces;
    na.infer_groups = (int)c->cfg.infer_groups;
    na.wait = c->wait;
    const unsigned long long train_seed = c->cfg.seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    const int order = scene_order(ctx, scene);
    const bool training = ntrain > 0 && c->cfg.max_train_steps > 0;
    // training paths of one pass, then at most max_train_steps optimiser steps over their records
    auto train_pass = [&]() -> int {
        na.mode = kNrcRecord;
        na.capacity = (uint32_t)rec_cap;
        PathBatch tb = make_batch(r, ntrain, 0, W, nullptr);
        cudaError_t te = launch_training_paths(traversal_view(ctx, scene), tb, cam, train_seed, (uint32_t)c->train_passes, ntrain,
                                               W, H, max_depth, na, as<float4>(r.nrc_tgt), ctx->status, order, st);
        uint32_t nrec = 0;
        if (te == cudaSuccess) te = cudaMemcpyAsync(&nrec, na.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (te == cudaSuccess) te = cudaStreamSynchronize(st);
        if (te != cudaSuccess) return cuda_error(ctx, te, "radiance cache training paths");
        nrec = std::min<uint32_t>(nrec, (uint32_t)rec_cap);
        ++c->train_passes;
        c->render_stats[0] += ntrain;
        c->render_stats[1] += nrec;
        if (nrec == 0) return PICO_OK;
        const uint32_t batch = c->cfg.train_batch;
        const uint32_t steps =
            std::max<uint32_t>(1u, std::min<uint32_t>(c->cfg.max_train_steps, (nrec + batch - 1) / batch));
        const uint32_t per = steps * ((nrec + steps * batch - 1) / (steps * batch));   // record stride
        for (uint32_t s = 0; s < steps && s < nrec; ++s) {
            const nrc::TrainBatch b{na.queries, as<float4>(r.nrc_tgt), (nrec - s + per - 1) / per, s, per};
            const int status = nrc::train_step(c, b, true, st);
            if (status != PICO_OK) return status;
            c->render_stats[2] += 1;
        }
        return PICO_OK;
    };
    const uint32_t passes = c->cfg.warmup_frames + cfg->max_samples;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        if (should_quit && *should_quit) { cancelled = true; break; }
        if (training) {
            const int status = train_pass();
            if (status != PICO_OK) return status;
        }
        if (pass < c->cfg.warmup_frames) continue;
        // one sample per active pixel, ending in the cache
        na.mode = kNrcTerminate;
        na.capacity = chunk_pix;
        for (size_t p0 = 0; p0 < nactive; p0 += chunk_pix) {
            const uint32_t npix = (uint32_t)std::min<size_t>(chunk_pix, nactive - p0);
            PathBatch b = make_batch(r, npix, npix, W, as<uint32_t>(r.pix_list) + p0);
            e = launch_render_batch(traversal_view(ctx, scene), b, cam, cfg->seed, 1, max_depth, cfg->max_samples,
                                    cfg->max_variance, PICO_ESTIMATOR_RADIANCE_CACHE, ctx->status, order, st, &na);
            uint32_t nq = 0;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&nq, na.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return cuda_error(ctx, e, "radiance cache render batch");
            c->render_stats[3] += nq;
        }
        ++c->frames;
    }
    return nrc::take_status(c, st);
}

// Checks shared by the render entry points.
int validate_render(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                    const pico_render_config* cfg)
{
    if (!ctx || !scene || !cfg || !valid_camera(camera)) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (cfg->width != camera->resolution[0] || cfg->height != camera->resolution[1])
        return set_error(ctx, PICO_ERR_INVALID_ARG, "render size differs from the camera resolution");
    if (cfg->estimator != PICO_ESTIMATOR_REFERENCE && cfg->estimator != PICO_ESTIMATOR_PHYSICAL &&
        cfg->estimator != PICO_ESTIMATOR_RADIANCE_CACHE)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "unknown estimator");
    if (cfg->estimator == PICO_ESTIMATOR_RADIANCE_CACHE && scene->has_btdf)
        return set_error(ctx, PICO_ERR_UNSUPPORTED, "the radiance cache has no Transparent or Fresnel lobes");
    if (cfg->estimator == PICO_ESTIMATOR_RADIANCE_CACHE && !ctx->cache)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "no radiance cache attached (pico_gpu_set_radiance_cache)");
    return PICO_OK;
}

// With a cancel flag, a render's batches take at most this many samples per pixel,
// so that a cancel is seen after at most one such batch (on small images a batch
// could otherwise hold hundreds of samples per pixel).
constexpr uint32_t kCancelSamplesPerBatch = 16;
// The reference's early exit can first stop a fresh pixel at its sixth sample
// (Scene.cpp:193-197: after a sample taken with more than 4 before it), so the
// first round of an exit-aware render takes six.
constexpr uint32_t kFirstExitSamples = 6;

// Whether the reference's early exit can stop pixels of this render: the reference
// estimator with a variance bound that a variance can meet.
static bool early_exit_on(const pico_render_config* cfg)
{
    return cfg->estimator == PICO_ESTIMATOR_REFERENCE && cfg->max_variance >= 0.0f;
}

// Exit-aware rounds over the first `nactive` pixels of r.pix_list (at most
// the path limit of them): the first round takes kFirstExitSamples samples per pixel;
// after every round a compaction keeps the pixels still sampling and the next round
// takes as many samples per pixel as fill the path state (the path limit), so that
// rounds after the exits are dense.  Both are decided on the device (RoundPlan), so
// nothing here waits for it: the host enqueues as many rounds as a render with no
// exit needs, and rounds with nothing left to do launch empty kernels.  Images are
// the same as with fixed batches: a path's random stream depends on its pixel and
// sample index only, and every pixel takes its samples in order.
static int run_exit_aware_rounds(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_render_config* cfg,
                                 const CameraView& cam, RenderBuffers& r, uint32_t nactive, float* pixels,
                                 float* variance, uint32_t* count, const volatile int32_t* should_quit,
                                 cudaStream_t st, bool& cancelled)
{
    const uint32_t cap = should_quit ? kCancelSamplesPerBatch : cfg->max_samples;
    const uint32_t paths = (uint32_t)std::min<uint64_t>(path_limit(ctx), (uint64_t)nactive * cfg->max_samples);
    cudaError_t e = reserve_paths(r, paths);
    if (e == cudaSuccess) e = r.pix_list2.reserve((size_t)nactive * sizeof(uint32_t));
    if (e == cudaSuccess) e = r.plan.reserve(sizeof(RoundPlan));
    if (e != cudaSuccess) return cuda_error(ctx, e, "path state");
    // rounds a render with no exit needs: the first (as plan_round sizes it for all nactive
    // pixels: at most kFirstExitSamples, and no more than the path state holds), then rounds of
    // the smallest later size (every pixel still sampling)
    const uint32_t later = std::max(1u, std::min(paths / nactive, cap));
    const uint32_t first = std::min({kFirstExitSamples, cfg->max_samples, later});
    const uint32_t rounds = 1 + (cfg->max_samples - first + later - 1) / later;
    RoundPlan* plan = as<RoundPlan>(r.plan);
    uint32_t* lists[2] = {as<uint32_t>(r.pix_list), as<uint32_t>(r.pix_list2)};
    const RenderProbe probe{ctx->extend_timer, ctx->count_work ? ctx->status->counters : nullptr, ctx->shade_timer};
    const RenderProbe* pp = (probe.timer || probe.counters) ? &probe : nullptr;
    e = launch_plan_init(plan, nactive, st);
    for (uint32_t k = 0; k < rounds && e == cudaSuccess; ++k) {
        if (should_quit && *should_quit) { cancelled = true; break; }
        e = launch_plan_round(plan, cfg->max_samples, first, cap, paths, st);
        if (e != cudaSuccess) break;
        PathBatch b = make_batch(r, paths, nactive, cfg->width, lists[k & 1]);
        b.plan = plan;
        b.pixels = pixels;
        b.variance = variance;
        b.count = count;
        e = launch_render_batch(traversal_view(ctx, scene), b, cam, cfg->seed, 0, cfg->max_ray_depth, cfg->max_samples,
                                cfg->max_variance, (int)cfg->estimator, ctx->status, scene_order(ctx, scene), st,
                                nullptr, pp);
        if (e == cudaSuccess && k + 1 < rounds)
            e = launch_compact_pixels(plan, lists[k & 1], as<uint32_t>(r.done), lists[(k + 1) & 1], nactive, st);
        if (e == cudaSuccess && should_quit) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "render round");
    return PICO_OK;
}

// The sample batches of a reference or physical render over the first `nactive`
// pixels of r.pix_list, advancing the image buffers (pixels, variance, count) and
// r's taken / done state on st.  With a cancel flag the host polls it before each
// batch (and waits for the previous one); without one nothing waits for the device.
int run_sample_batches(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_render_config* cfg,
                       const CameraView& cam, RenderBuffers& r, size_t nactive, float* pixels, float* variance,
                       uint32_t* count, const volatile int32_t* should_quit, cudaStream_t st, bool& cancelled)
{
    if (early_exit_on(cfg) && nactive <= path_limit(ctx))
        return run_exit_aware_rounds(ctx, scene, cfg, cam, r, (uint32_t)nactive, pixels, variance, count, should_quit,
                                     st, cancelled);
    const uint32_t chunk_pix = (uint32_t)std::min<size_t>(nactive, path_limit(ctx));
    uint32_t spb_cap = path_limit(ctx) / chunk_pix;
    if (should_quit) spb_cap = std::min(spb_cap, kCancelSamplesPerBatch);
    const uint32_t spb_max = std::max<uint32_t>(1u, std::min<uint32_t>(cfg->max_samples, spb_cap));
    cudaError_t e = reserve_paths(r, (size_t)chunk_pix * spb_max);
    if (e != cudaSuccess) return cuda_error(ctx, e, "path state");
    const RenderProbe probe{ctx->extend_timer, ctx->count_work ? ctx->status->counters : nullptr, ctx->shade_timer};
    const RenderProbe* pp = (probe.timer || probe.counters) ? &probe : nullptr;
    for (size_t p0 = 0; p0 < nactive && !cancelled; p0 += chunk_pix) {
        const uint32_t npix = (uint32_t)std::min<size_t>(chunk_pix, nactive - p0);
        for (uint32_t s0 = 0; s0 < cfg->max_samples; s0 += spb_max) {
            if (should_quit && *should_quit) { cancelled = true; break; }
            const uint32_t spb = std::min(spb_max, cfg->max_samples - s0);
            PathBatch b = make_batch(r, npix * spb, npix, cfg->width, as<uint32_t>(r.pix_list) + p0);
            b.pixels = pixels;
            b.variance = variance;
            b.count = count;
            e = launch_render_batch(traversal_view(ctx, scene), b, cam, cfg->seed, spb, cfg->max_ray_depth, cfg->max_samples,
                                    cfg->max_variance, (int)cfg->estimator, ctx->status, scene_order(ctx, scene), st,
                                    nullptr, pp);
            if (e == cudaSuccess && should_quit) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return cuda_error(ctx, e, "render batch");
        }
    }
    return PICO_OK;
}

// Scene.cpp:212-234 after the samples: the a-trous pass on the G-buffer replaces
// the image, then the tone map runs in place.
int finish_image(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const CameraView& cam, const pico_render_config* cfg,
                 RenderBuffers& r, float* pixels, cudaStream_t st)
{
    const uint32_t W = cfg->width, H = cfg->height;
    const size_t n3 = (size_t)W * H * 3;
    cudaError_t e = cudaSuccess;
    if (cfg->denoise) {
        for (DeviceBuffer* b : {&r.gn, &r.gp, &r.gd, &r.out})
            if (e == cudaSuccess) e = b->reserve(n3 * sizeof(float));
        if (e == cudaSuccess)
            e = launch_gbuffer(traversal_view(ctx, scene), cam, W, H, as<float>(r.gn), as<float>(r.gp), as<float>(r.gd), ctx->status,
                               scene_order(ctx, scene), st);
        if (e != cudaSuccess) return cuda_error(ctx, e, "denoiser inputs");
        const int status = run_atrous(ctx, r, pixels, as<float>(r.gn), as<float>(r.gp), as<float>(r.gd), W, H,
                                      as<float>(r.out), st);
        if (status != PICO_OK) return status;
        e = cudaMemcpyAsync(pixels, r.out.ptr, n3 * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_error(ctx, e, "denoise copy");
    }
    if (cfg->tonemap) {
        // in place on the (denoised) buffer, which then replaces the caller's pixels (Scene.cpp:225-234)
        e = r.tonemap.reserve(sizeof(unsigned));
        if (e == cudaSuccess) e = launch_reinhard(pixels, W, H, as<unsigned>(r.tonemap), st);
        if (e != cudaSuccess) return cuda_error(ctx, e, "tone mapping");
    }
    return PICO_OK;
}

}  // namespace

extern "C" {

int pico_gpu_render(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                    const pico_render_config* cfg, float* pixels, uint32_t* sample_count, float* variance,
                    const volatile int32_t* should_quit)
{
    int status = validate_render(ctx, scene, camera, cfg);
    if (status != PICO_OK) return status;
    if (!pixels || !sample_count || !variance) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if ((size_t)cfg->width * cfg->height > 0xffffffffull)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "image larger than 2^32 pixels");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    RenderBuffers& r = *render_buffers(ctx);
    const uint32_t W = cfg->width, H = cfg->height;
    const size_t npx = (size_t)W * H;
    ctx->stats_on_device = false;

    cudaError_t e = r.pixels.reserve(npx * 3 * sizeof(float));
    if (e == cudaSuccess) e = r.variance.reserve(npx * 3 * sizeof(float));
    for (DeviceBuffer* b : {&r.count, &r.taken, &r.done, &r.pix_list})
        if (e == cudaSuccess) e = b->reserve(npx * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_error(ctx, e, "image buffers");

    // The radiance cache's passes take the pixels still sampling as a compacted list built
    // here; the other estimators list every pixel on the device (prepare_image_kernel) and
    // skip the finished ones there, with no host pass over the image.
    const bool host_list = cfg->estimator == PICO_ESTIMATOR_RADIANCE_CACHE;
    std::vector<uint32_t> active, done;
    uint64_t samples_before = 0;
    if (host_list) {
        done.assign(npx, 0u);
        active.reserve(npx);
        for (size_t p = 0; p < npx; ++p) {
            samples_before += sample_count[p];
            if (sample_count[p] >= cfg->max_samples) done[p] = 1;
            else active.push_back((uint32_t)p);
        }
    }
    for (uint64_t& v : ctx->render_stats) v = 0;
    e = cudaMemcpyAsync(r.pixels.ptr, pixels, npx * 3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.variance.ptr, variance, npx * 3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.count.ptr, sample_count, npx * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status->rays, 0, sizeof(ctx->status->rays), st);
    if (host_list) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(r.done.ptr, done.data(), npx * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(r.taken.ptr, 0, npx * sizeof(uint32_t), st);
        if (e == cudaSuccess && !active.empty())
            e = cudaMemcpyAsync(r.pix_list.ptr, active.data(), active.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // the host vectors end with this call
    } else if (e == cudaSuccess) {
        e = launch_prepare_image(as<uint32_t>(r.count), (uint32_t)npx, cfg->max_samples, as<uint32_t>(r.pix_list),
                                 as<uint32_t>(r.done), as<uint32_t>(r.taken), st);
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "render upload");

    const CameraView cam = make_camera_view(*camera);
    bool cancelled = false;
    const size_t nactive = host_list ? active.size() : npx;
    if (nactive > 0 && cfg->max_samples > 0) {
        status = host_list
                     ? render_with_cache(ctx, scene, ctx->cache, cfg, cam, r, nactive, should_quit, cancelled)
                     : run_sample_batches(ctx, scene, cfg, cam, r, nactive, as<float>(r.pixels),
                                          as<float>(r.variance), as<uint32_t>(r.count), should_quit, st, cancelled);
        if (status != PICO_OK) return status;
    }
    status = take_device_status(ctx, st);
    if (status != PICO_OK) return status;
    status = finish_image(ctx, scene, cam, cfg, r, as<float>(r.pixels), st);
    if (status != PICO_OK) return status;

    e = cudaMemcpyAsync(pixels, r.pixels.ptr, npx * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(variance, r.variance.ptr, npx * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sample_count, r.count.ptr, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    unsigned long long rays[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(rays, ctx->status->rays, sizeof(rays), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "render download");
    if (host_list) {
        uint64_t samples_after = 0;
        for (size_t p = 0; p < npx; ++p) samples_after += sample_count[p];
        ctx->render_stats[0] = samples_after - samples_before;
    } else {
        ctx->render_stats[0] = rays[3];   // the samples accumulate added, tallied on the device
    }
    ctx->render_stats[1] = rays[0];
    ctx->render_stats[2] = rays[1];
    ctx->render_stats[3] = rays[2];
    ctx->render_stats[4] = cfg->denoise ? npx : 0;
    status = take_device_status(ctx, st);
    if (status != PICO_OK) return status;
    return cancelled ? set_error(ctx, PICO_ERR_CANCELLED, "render cancelled") : PICO_OK;
}

int pico_gpu_render_device(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                           const pico_render_config* cfg, float* d_pixels, uint32_t* d_count, float* d_variance,
                           void* stream)
{
    int status = validate_render(ctx, scene, camera, cfg);
    if (status != PICO_OK) return status;
    if (!d_pixels || !d_count || !d_variance) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (cfg->estimator == PICO_ESTIMATOR_RADIANCE_CACHE)
        return set_error(ctx, PICO_ERR_UNSUPPORTED, "device-buffer renders take the reference or physical estimator");
    const size_t npx = (size_t)cfg->width * cfg->height;
    if (npx > 0xffffffffull) return set_error(ctx, PICO_ERR_INVALID_ARG, "image larger than 2^32 pixels");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RenderBuffers& r = *render_buffers(ctx);
    cudaError_t e = cudaSuccess;
    for (DeviceBuffer* b : {&r.taken, &r.done, &r.pix_list})
        if (e == cudaSuccess) e = b->reserve(npx * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_error(ctx, e, "image state");
    e = launch_prepare_image(d_count, (uint32_t)npx, cfg->max_samples, as<uint32_t>(r.pix_list), as<uint32_t>(r.done),
                             as<uint32_t>(r.taken), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status->rays, 0, sizeof(ctx->status->rays), st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "render set-up");
    const CameraView cam = make_camera_view(*camera);
    bool cancelled = false;
    if (npx > 0 && cfg->max_samples > 0) {
        status = run_sample_batches(ctx, scene, cfg, cam, r, npx, d_pixels, d_variance, d_count, nullptr, st,
                                    cancelled);
        if (status != PICO_OK) return status;
    }
    status = finish_image(ctx, scene, cam, cfg, r, d_pixels, st);
    if (status != PICO_OK) return status;
    ctx->stats_on_device = true;
    ctx->stats_stream = st;
    ctx->stats_gbuffer_rays = cfg->denoise ? npx : 0;
    return PICO_OK;
}

int pico_gpu_render_stats(const pico_gpu_ctx* cctx, uint64_t* out5)
{
    if (!cctx || !out5) return PICO_ERR_INVALID_ARG;
    pico_gpu_ctx* ctx = const_cast<pico_gpu_ctx*>(cctx);
    if (ctx->stats_on_device) {
        // the tallies of the last pico_gpu_render_device call, once its stream has them
        const DeviceScope device_scope(ctx->device);
        unsigned long long rays[4] = {0, 0, 0, 0};
        cudaError_t e = cudaStreamSynchronize(ctx->stats_stream);
        if (e == cudaSuccess) e = cudaMemcpy(rays, ctx->status->rays, sizeof(rays), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_error(ctx, e, "render stats");
        ctx->render_stats[0] = rays[3];
        ctx->render_stats[1] = rays[0];
        ctx->render_stats[2] = rays[1];
        ctx->render_stats[3] = rays[2];
        ctx->render_stats[4] = ctx->stats_gbuffer_rays;
        ctx->stats_on_device = false;
    }
    for (int k = 0; k < 5; ++k) out5[k] = ctx->render_stats[k];
    return PICO_OK;
}

int pico_gpu_set_path_limit(pico_gpu_ctx* ctx, uint32_t max_paths)
{
    if (!ctx) return PICO_ERR_INVALID_ARG;
    if (max_paths != 0 && (max_paths < 64 || max_paths > kMaxPaths))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "path limit: 0 (the default, 2^26) or 64 .. 2^26");
    ctx->max_paths = max_paths;
    return PICO_OK;
}

int pico_gpu_set_render_probe(pico_gpu_ctx* ctx, int32_t time_extend, int32_t count_work)
{
    if (!ctx) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_error(ctx, e, "render probe");
    if (time_extend) {
        if (!ctx->extend_timer) ctx->extend_timer = new LaunchTimer();
        if (!ctx->shade_timer) ctx->shade_timer = new LaunchTimer();
        ctx->extend_timer->reset();
        ctx->shade_timer->reset();
    } else {
        delete ctx->extend_timer;
        ctx->extend_timer = nullptr;
        delete ctx->shade_timer;
        ctx->shade_timer = nullptr;
    }
    ctx->count_work = count_work != 0;
    e = cudaMemset(ctx->status->counters, 0, sizeof(ctx->status->counters));
    if (e != cudaSuccess) return cuda_error(ctx, e, "render probe");
    return PICO_OK;
}

int pico_gpu_render_probe_read(pico_gpu_ctx* ctx, uint64_t* out4, double* extend_ms)
{
    if (!ctx || !out4 || !extend_ms) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long c[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(c, ctx->status->counters, sizeof c, cudaMemcpyDeviceToHost);
    double ms = 0.0;
    uint64_t launches = 0;
    if (e == cudaSuccess && ctx->extend_timer) e = ctx->extend_timer->total(ms, launches);
    if (e != cudaSuccess) return cuda_error(ctx, e, "render probe");
    out4[0] = launches;
    out4[1] = c[0];
    out4[2] = c[1];
    out4[3] = c[2];
    *extend_ms = ms;
    return PICO_OK;
}

int pico_gpu_render_probe_read_shade(pico_gpu_ctx* ctx, uint64_t* launches, double* shade_ms)
{
    if (!ctx || !launches || !shade_ms) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    double ms = 0.0;
    uint64_t n = 0;
    if (e == cudaSuccess && ctx->shade_timer) e = ctx->shade_timer->total(ms, n);
    if (e != cudaSuccess) return cuda_error(ctx, e, "render probe");
    *launches = n;
    *shade_ms = ms;
    return PICO_OK;
}

int pico_gpu_denoiser_inputs(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                             float* normals, float* positions, float* diffuse)
{
    if (!ctx || !scene || !valid_camera(camera) || !normals || !positions || !diffuse)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    RenderBuffers& r = *render_buffers(ctx);
    const uint32_t W = camera->resolution[0], H = camera->resolution[1];
    const size_t n3 = (size_t)W * H * 3;
    cudaError_t e = cudaSuccess;
    for (DeviceBuffer* b : {&r.gn, &r.gp, &r.gd})
        if (e == cudaSuccess) e = b->reserve(n3 * sizeof(float));
    if (e == cudaSuccess)
        e = launch_gbuffer(traversal_view(ctx, scene), make_camera_view(*camera), W, H, as<float>(r.gn), as<float>(r.gp),
                           as<float>(r.gd), ctx->status, scene_order(ctx, scene), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(normals, r.gn.ptr, n3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(positions, r.gp.ptr, n3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(diffuse, r.gd.ptr, n3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "denoiser inputs");
    return take_device_status(ctx, st);
}

int pico_gpu_atrous_device(pico_gpu_ctx* ctx, const float* d_pixels, const float* d_normals, const float* d_positions,
                           const float* d_diffuse, uint32_t width, uint32_t height, float* d_out, void* stream)
{
    if (!ctx || !d_pixels || !d_normals || !d_positions || !d_diffuse || !d_out)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (atrous_output_aliases(d_out, d_pixels, d_normals, d_positions, d_diffuse, (size_t)width * height * 3))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "the output must not overlap an input");
    const DeviceScope device_scope(ctx->device);
    return run_atrous(ctx, *render_buffers(ctx), d_pixels, d_normals, d_positions, d_diffuse, width, height, d_out,
                      static_cast<cudaStream_t>(stream));
}

int pico_gpu_atrous(pico_gpu_ctx* ctx, const float* pixels, const float* normals, const float* positions,
                    const float* diffuse, uint32_t W, uint32_t H, float* out)
{
    if (!ctx || !pixels || !normals || !positions || !diffuse || !out)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    RenderBuffers& r = *render_buffers(ctx);
    const size_t n3 = (size_t)W * H * 3;
    cudaError_t e = cudaSuccess;
    for (DeviceBuffer* b : {&r.pixels, &r.gn, &r.gp, &r.gd, &r.out})
        if (e == cudaSuccess) e = b->reserve(n3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.pixels.ptr, pixels, n3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.gn.ptr, normals, n3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.gp.ptr, positions, n3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.gd.ptr, diffuse, n3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "a-trous upload");
    int status = run_atrous(ctx, r, as<float>(r.pixels), as<float>(r.gn), as<float>(r.gp), as<float>(r.gd), W, H,
                            as<float>(r.out), st);
    if (status != PICO_OK) return status;
    e = cudaMemcpyAsync(out, r.out.ptr, n3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "a-trous download");
    return PICO_OK;
}

int pico_gpu_tonemap_device(pico_gpu_ctx* ctx, float* d_pixels, uint32_t width, uint32_t height, void* stream)
{
    if (!ctx || !d_pixels) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    RenderBuffers& r = *render_buffers(ctx);
    cudaError_t e = r.tonemap.reserve(sizeof(unsigned));
    if (e == cudaSuccess)
        e = launch_reinhard(d_pixels, width, height, as<unsigned>(r.tonemap), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error(ctx, e, "tone mapping");
    return PICO_OK;
}

int pico_gpu_tonemap(pico_gpu_ctx* ctx, float* pixels, uint32_t width, uint32_t height)
{
    if (!ctx || !pixels) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    RenderBuffers& r = *render_buffers(ctx);
    const size_t n3 = (size_t)width * height * 3;
    cudaError_t e = r.out.reserve(n3 * sizeof(float));
    if (e == cudaSuccess) e = r.tonemap.reserve(sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.out.ptr, pixels, n3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_reinhard(as<float>(r.out), width, height, as<unsigned>(r.tonemap), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pixels, r.out.ptr, n3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "tone mapping");
    return PICO_OK;
}

}  // extern "C"
