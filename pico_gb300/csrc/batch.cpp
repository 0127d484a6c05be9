// Batched rendering (pico_gpu_render_many) and its autotuner: no counterpart in
// the reference, which renders one scene at a time.
//
// Every render gets a slot of its own (path state, image buffers, device status
// block) and its batches are captured, without host synchronisation, on one of
// `branches` streams forked from the context's stream; the captured graph
// (one branch per stream, renders on a branch in sequence) is instantiated and
// launched once.  Small renders cannot fill 152 SMs on their own; side by side
// their persistent closest-hit grids and shade kernels share the GPU.  A 1-thread
// kernel at the graph's start and at the end of each render stores the device's
// nanosecond timer, from which the per-render completion times are read.
#include "render_internal.h"

#include <algorithm>
#include <chrono>
#include <memory>
#include <vector>

using namespace pico;

struct BatchSlot {
    RenderBuffers r;
    DeviceStatus* status = nullptr;
    ~BatchSlot()
    {
        if (status) cudaFree(status);
    }
};

struct BatchState {
    std::vector<std::unique_ptr<BatchSlot>> slots;
    std::vector<cudaStream_t> streams;
    unsigned long long* stamps = nullptr;   // [0] graph start, [1 + r] end of render r
    size_t stamp_cap = 0;
    ~BatchState()
    {
        slots.clear();
        for (cudaStream_t s : streams) cudaStreamDestroy(s);
        if (stamps) cudaFree(stamps);
    }
};

namespace pico {
void free_batch_state(pico_gpu_ctx* ctx)
{
    delete ctx->batch;
    ctx->batch = nullptr;
}
}  // namespace pico

namespace {

struct Params {
    uint32_t wavefront, extend_ctas, branches;
};

// Host-side state of one render between its upload and its download.
struct Prepared {
    uint32_t W = 0, H = 0;
    size_t npx = 0;
    size_t nactive = 0;
    uint64_t samples_before = 0;
    uint32_t chunk_pix = 0, spb_max = 0;
    CameraView cam{};
};

Params resolve(const pico_launch_params* lp, uint32_t n)
{
    Params p{1u << 20, 0u, n};
    if (lp) {
        if (lp->wavefront) p.wavefront = std::min<uint32_t>(std::max<uint32_t>(lp->wavefront, 1u << 12), kMaxPaths);
        p.extend_ctas = lp->extend_ctas_per_sm;
        if (lp->branches) p.branches = std::min(lp->branches, n);
    }
    if (p.branches == 0) p.branches = 1;
    return p;
}

int validate(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items)
{
    if (!ctx || (n && !items)) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    for (uint32_t r = 0; r < n; ++r) {
        const pico_render_item& it = items[r];
        const pico_render_config& c = it.config;
        if (!it.scene || !it.pixels_rgb || !it.sample_count || !it.variance_rgb)
            return set_error(ctx, PICO_ERR_INVALID_ARG, "render " + std::to_string(r) + ": null argument");
        if (it.camera.resolution[0] == 0 || it.camera.resolution[1] == 0 || c.width != it.camera.resolution[0] ||
            c.height != it.camera.resolution[1])
            return set_error(ctx, PICO_ERR_INVALID_ARG, "render " + std::to_string(r) + ": bad image size");
        if (c.estimator != PICO_ESTIMATOR_REFERENCE && c.estimator != PICO_ESTIMATOR_PHYSICAL)
            return set_error(ctx, PICO_ERR_INVALID_ARG,
                             "render " + std::to_string(r) + ": batches take the reference or physical estimator");
        if (c.estimator == PICO_ESTIMATOR_PHYSICAL && it.scene->has_btdf)
            return set_error(ctx, PICO_ERR_UNSUPPORTED,
                             "render " + std::to_string(r) + ": the physical estimator has no Transparent or Fresnel lobes");
        if (c.denoise || c.tonemap)
            return set_error(ctx, PICO_ERR_INVALID_ARG,
                             "render " + std::to_string(r) + ": batches do not denoise or tone map");
        if (it.scene->ctx != ctx)
            return set_error(ctx, PICO_ERR_INVALID_ARG, "render " + std::to_string(r) + ": scene of another context");
    }
    return PICO_OK;
}

cudaError_t ensure_state(pico_gpu_ctx* ctx, uint32_t n, uint32_t branches)
{
    if (!ctx->batch) ctx->batch = new BatchState();
    BatchState& bs = *ctx->batch;
    while (bs.slots.size() < n) {
        auto s = std::make_unique<BatchSlot>();
        cudaError_t e = cudaMalloc(&s->status, sizeof(DeviceStatus));
        if (e == cudaSuccess) e = cudaMemset(s->status, 0, sizeof(DeviceStatus));
        if (e != cudaSuccess) return e;
        bs.slots.push_back(std::move(s));
    }
    while (bs.streams.size() < branches) {
        cudaStream_t s = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        bs.streams.push_back(s);
    }
    if (bs.stamp_cap < (size_t)n + 1) {
        if (bs.stamps) cudaFree(bs.stamps);
        bs.stamps = nullptr;
        bs.stamp_cap = 0;
        cudaError_t e = cudaMalloc(&bs.stamps, ((size_t)n + 1) * sizeof(unsigned long long));
        if (e != cudaSuccess) return e;
        bs.stamp_cap = (size_t)n + 1;
    }
    return cudaSuccess;
}

// Uploads one render's progressive buffers and active-pixel list and reserves its path state.
cudaError_t prepare(const pico_render_item& it, BatchSlot& s, const Params& p, Prepared& pr, cudaStream_t st,
                    std::vector<uint32_t>& active, std::vector<uint32_t>& done)
{
    const pico_render_config& cfg = it.config;
    RenderBuffers& r = s.r;
    pr.W = cfg.width;
    pr.H = cfg.height;
    pr.npx = (size_t)pr.W * pr.H;
    active.clear();
    done.assign(pr.npx, 0u);
    pr.samples_before = 0;
    for (size_t px = 0; px < pr.npx; ++px) {
        pr.samples_before += it.sample_count[px];
        if (it.sample_count[px] >= cfg.max_samples) done[px] = 1;
        else active.push_back((uint32_t)px);
    }
    pr.nactive = active.size();
    pr.cam = make_camera_view(it.camera);
    cudaError_t e = r.pixels.reserve(pr.npx * 3 * sizeof(float));
    if (e == cudaSuccess) e = r.variance.reserve(pr.npx * 3 * sizeof(float));
    for (DeviceBuffer* b : {&r.count, &r.taken, &r.done, &r.pix_list})
        if (e == cudaSuccess) e = b->reserve(pr.npx * sizeof(uint32_t));
    pr.chunk_pix = (uint32_t)std::min<size_t>(std::max<size_t>(pr.nactive, 1), p.wavefront);
    pr.spb_max = std::max<uint32_t>(1u, std::min<uint32_t>(std::max(cfg.max_samples, 1u), p.wavefront / pr.chunk_pix));
    if (e == cudaSuccess && pr.nactive && cfg.max_samples) e = reserve_paths(r, (size_t)pr.chunk_pix * pr.spb_max);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.pixels.ptr, it.pixels_rgb, pr.npx * 3 * sizeof(float),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.variance.ptr, it.variance_rgb, pr.npx * 3 * sizeof(float),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.count.ptr, it.sample_count, pr.npx * sizeof(uint32_t),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.done.ptr, done.data(), pr.npx * sizeof(uint32_t),
                                              cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r.taken.ptr, 0, pr.npx * sizeof(uint32_t), st);
    if (e == cudaSuccess && pr.nactive)
        e = cudaMemcpyAsync(r.pix_list.ptr, active.data(), pr.nactive * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.status, 0, sizeof(DeviceStatus), st);
    // the pageable sources above must stay alive until the copies finish
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// The render's batches on stream st, without synchronisation (they are captured).
cudaError_t enqueue(pico_gpu_ctx* ctx, const pico_render_item& it, BatchSlot& s, const Params& p,
                    const Prepared& pr, cudaStream_t st)
{
    const pico_render_config& cfg = it.config;
    const int order = scene_order(ctx, it.scene);
    cudaError_t e = cudaSuccess;
    if (!pr.nactive || !cfg.max_samples) return e;
    for (size_t p0 = 0; p0 < pr.nactive && e == cudaSuccess; p0 += pr.chunk_pix) {
        const uint32_t npix = (uint32_t)std::min<size_t>(pr.chunk_pix, pr.nactive - p0);
        for (uint32_t s0 = 0; s0 < cfg.max_samples && e == cudaSuccess; s0 += pr.spb_max) {
            const uint32_t spb = std::min(pr.spb_max, cfg.max_samples - s0);
            PathBatch b = make_batch(s.r, npix * spb, npix, pr.W, as<uint32_t>(s.r.pix_list) + p0);
            b.extend_ctas = p.extend_ctas;
            e = launch_render_batch(it.scene->view, b, pr.cam, cfg.seed, spb, cfg.max_ray_depth, cfg.max_samples,
                                    cfg.max_variance, (int)cfg.estimator, s.status, order, st);
        }
    }
    return e;
}

int run_batch(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items, const Params& p, double* completion_ms,
              pico_batch_report* rep)
{
    using clock = std::chrono::steady_clock;
    cudaStream_t st = ctx->stream;
    cudaError_t e = ensure_state(ctx, n, p.branches);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch state");
    BatchState& bs = *ctx->batch;
    std::vector<Prepared> prep(n);
    std::vector<uint32_t> active, done;
    for (uint32_t r = 0; r < n && e == cudaSuccess; ++r) e = prepare(items[r], *bs.slots[r], p, prep[r], st, active, done);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch upload");

    const auto t_build = clock::now();
    std::vector<cudaEvent_t> events(1 + p.branches, nullptr);
    for (cudaEvent_t& ev : events)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (cudaEvent_t ev : events)
            if (ev) cudaEventDestroy(ev);
    };
    // relaxed: the launchers' one-time occupancy queries may run inside the capture
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_error(ctx, e, "batch capture");
    }
    cudaError_t ce = launch_stamp(bs.stamps, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(events[0], st);
    for (uint32_t k = 0; k < p.branches && ce == cudaSuccess; ++k) ce = cudaStreamWaitEvent(bs.streams[k], events[0], 0);
    for (uint32_t r = 0; r < n && ce == cudaSuccess; ++r) {
        cudaStream_t bst = bs.streams[r % p.branches];
        ce = enqueue(ctx, items[r], *bs.slots[r], p, prep[r], bst);
        if (ce == cudaSuccess) ce = launch_stamp(bs.stamps + 1 + r, bst);
    }
    for (uint32_t k = 0; k < p.branches && ce == cudaSuccess; ++k) {
        ce = cudaEventRecord(events[1 + k], bs.streams[k]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(st, events[1 + k], 0);
    }
    e = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) e = ce;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    size_t nodes = 0;
    if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nullptr, &nodes);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_error(ctx, e, "batch graph");
    }
    const auto t_run = clock::now();
    e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    const auto t_end = clock::now();
    cleanup();
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch launch");

    std::vector<unsigned long long> stamps((size_t)n + 1);
    e = cudaMemcpy(stamps.data(), bs.stamps, stamps.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    uint64_t samples = 0, rays = 0;
    int status = PICO_OK;
    for (uint32_t r = 0; r < n && e == cudaSuccess; ++r) {
        const pico_render_item& it = items[r];
        BatchSlot& s = *bs.slots[r];
        const Prepared& pr = prep[r];
        e = cudaMemcpyAsync(it.pixels_rgb, s.r.pixels.ptr, pr.npx * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it.variance_rgb, s.r.variance.ptr, pr.npx * 3 * sizeof(float),
                                                  cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it.sample_count, s.r.count.ptr, pr.npx * sizeof(uint32_t),
                                                  cudaMemcpyDeviceToHost, st);
        DeviceStatus ds{};
        if (e == cudaSuccess) e = cudaMemcpyAsync(&ds, s.status, sizeof ds, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        uint64_t after = 0;
        for (size_t px = 0; px < pr.npx; ++px) after += it.sample_count[px];
        samples += after - pr.samples_before;
        rays += ds.rays[0] + ds.rays[1] + ds.rays[2];
        if (ds.trace_error && status == PICO_OK)
            status = set_error(ctx, (ds.trace_error & kTraceStackOverflow) ? PICO_ERR_STACK_OVERFLOW : PICO_ERR_TIMEOUT,
                               "render " + std::to_string(r) + ": a traversal failed");
        if (completion_ms) completion_ms[r] = (double)(stamps[1 + r] - stamps[0]) * 1e-6;
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch download");
    if (rep) {
        rep->build_ms = std::chrono::duration<double, std::milli>(t_run - t_build).count();
        rep->run_ms = std::chrono::duration<double, std::milli>(t_end - t_run).count();
        rep->graph_nodes = nodes;
        rep->samples = samples;
        rep->rays = rays;
    }
    return status;
}

}  // namespace

extern "C" {

int pico_gpu_render_many(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items,
                         const pico_launch_params* params, double* completion_ms, pico_batch_report* report)
{
    int status = validate(ctx, n, items);
    if (status != PICO_OK) return status;
    if (report) *report = pico_batch_report{};
    if (n == 0) return PICO_OK;
    cudaSetDevice(ctx->device);
    return run_batch(ctx, n, items, resolve(params, n), completion_ms, report);
}

int pico_gpu_autotune_batch(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items, uint32_t trial_samples,
                            pico_launch_params* best, pico_launch_params* trials_out, double* trial_msamples_per_s,
                            uint32_t max_trials, uint32_t* ntrials)
{
    int status = validate(ctx, n, items);
    if (status != PICO_OK) return status;
    if (!best) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (ntrials) *ntrials = 0;
    *best = pico_launch_params{};
    if (n == 0) return PICO_OK;
    cudaSetDevice(ctx->device);
    // short renders of the same items into scratch buffers
    std::vector<pico_render_item> trial(items, items + n);
    std::vector<std::vector<float>> px(n), var(n);
    std::vector<std::vector<uint32_t>> cnt(n);
    auto reset = [&]() {
        for (uint32_t r = 0; r < n; ++r) {
            const size_t npx = (size_t)items[r].config.width * items[r].config.height;
            px[r].assign(npx * 3, 0.0f);
            var[r].assign(npx * 3, 0.0f);
            cnt[r].assign(npx, 0u);
            trial[r].pixels_rgb = px[r].data();
            trial[r].variance_rgb = var[r].data();
            trial[r].sample_count = cnt[r].data();
            trial[r].config.max_samples = std::max(1u, trial_samples);
        }
    };
    uint32_t count = 0;
    auto measure = [&](const Params& p, double& msps) -> int {
        reset();
        pico_batch_report rep{};
        const int s = run_batch(ctx, n, trial.data(), p, nullptr, &rep);
        if (s != PICO_OK) return s;
        msps = rep.run_ms > 0.0 ? (double)rep.samples / rep.run_ms / 1e3 : 0.0;
        if (count < max_trials) {
            if (trials_out) trials_out[count] = pico_launch_params{p.wavefront, p.extend_ctas, p.branches, 0};
            if (trial_msamples_per_s) trial_msamples_per_s[count] = msps;
        }
        ++count;
        return PICO_OK;
    };
    Params cur{1u << 20, 0u, n};
    double rate = 0.0;
    status = measure(cur, rate);   // warm-up: module loading, buffer growth
    if (status != PICO_OK) return status;
    count = 0;
    double best_rate = 0.0;
    auto try_axis = [&](auto&& set, std::initializer_list<uint32_t> values) -> int {
        Params keep = cur;
        for (uint32_t v : values) {
            Params p = cur;
            set(p, v);
            double m = 0.0;
            const int s = measure(p, m);
            if (s != PICO_OK) return s;
            if (m > best_rate) { best_rate = m; keep = p; }
        }
        cur = keep;
        return PICO_OK;
    };
    status = try_axis([](Params& p, uint32_t v) { p.wavefront = v; }, {1u << 18, 1u << 20, 1u << 22});
    if (status == PICO_OK) status = try_axis([](Params& p, uint32_t v) { p.extend_ctas = v; }, {2u, 4u, 0u});
    if (status == PICO_OK)
        status = try_axis([n](Params& p, uint32_t v) { p.branches = std::min(v ? v : n, n); }, {8u, 16u, 0u});
    if (status != PICO_OK) return status;
    *best = pico_launch_params{cur.wavefront, cur.extend_ctas, cur.branches, 0};
    if (ntrials) *ntrials = std::min(count, max_trials);
    return PICO_OK;
}

}  // extern "C"
