// Batched rendering (pico_gpu_render_many) and its autotuner: no counterpart in
// the reference, which renders one scene at a time.
//
// Every render gets an image slot (its progressive buffers and active-pixel
// list).  Its active pixels are split into pieces of disjoint pixel ranges
// (one piece unless the render has more than piece_paths paths), and every
// piece gets a device status block of its own.  Each piece's batches are
// captured, without host synchronisation, on one of `branches` streams forked
// from the context's stream (placed by estimated cost: schedule()); the pieces
// of one branch run one after another, so each branch has one path slot (path
// state of at most `wavefront` paths) that its pieces reuse in turn, and the path
// state grows with the branches, not with the renders.  The captured graph is
// instantiated and launched once.  Small renders cannot fill 152 SMs on their
// own, and one large render would otherwise run alone at the end: side by side
// their persistent closest-hit grids and shade kernels share the GPU.  Pieces of
// one render write disjoint pixels of the same buffers.  A 1-thread kernel at
// the graph's start and at the end of each piece stores the device's nanosecond
// timer, from which the per-render completion times (the last of its pieces)
// are read.
#include "render_internal.h"

#include <algorithm>
#include <chrono>
#include <cstdlib>
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
    std::vector<std::unique_ptr<BatchSlot>> images;   // per render: progressive buffers, pixel list
    std::vector<std::unique_ptr<BatchSlot>> pieces;   // per piece: status block
    std::vector<std::unique_ptr<RenderBuffers>> paths;   // per branch: path state its pieces reuse in turn
    std::vector<cudaStream_t> streams;
    unsigned long long* stamps = nullptr;              // [0] graph start, [1 + j] end of piece j
    size_t stamp_cap = 0;
    ~BatchState()
    {
        images.clear();
        pieces.clear();
        paths.clear();
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
    uint32_t wavefront, extend_ctas, branches, piece_paths, extend_threads;
};

// Host-side state of one render between its upload and its download.
struct Prepared {
    uint32_t W = 0, H = 0;
    size_t npx = 0, nactive = 0;
    uint64_t samples_before = 0;
    CameraView cam{};
};

// A pixel range [p0, p1) of a render's active pixels, rendered on its own.
struct Piece {
    uint32_t render;
    size_t p0, p1;
    uint32_t chunk_pix, spb_max;
};

// The device's hardware work queues for this process (CUDA_DEVICE_MAX_CONNECTIONS,
// 8 by default).  More branches than queues share queues, and a cheap piece's
// kernels then wait behind a costly piece's in the same queue whatever their
// priorities, so a batch uses at most this many branches.
uint32_t work_queues()
{
    const char* v = std::getenv("CUDA_DEVICE_MAX_CONNECTIONS");
    const long n = v ? std::strtol(v, nullptr, 10) : 0;
    return n >= 1 && n <= 128 ? (uint32_t)n : 8u;
}

Params resolve(const pico_launch_params* lp)
{
    Params p{1u << 20, 0u, 0u, 0u, 128u};
    if (lp) {
        if (lp->wavefront) p.wavefront = std::min<uint32_t>(std::max<uint32_t>(lp->wavefront, 1u << 12), kMaxPaths);
        p.extend_ctas = lp->extend_ctas_per_sm;
        p.branches = lp->branches;
        p.piece_paths = lp->piece_paths;
        if (lp->extend_threads == 64 || lp->extend_threads == 256) p.extend_threads = lp->extend_threads;
    }
    return p;
}

int validate(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items)
{
    if (!ctx || (n && !items)) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    for (uint32_t r = 0; r < n; ++r) {
        const pico_render_item& it = items[r];
        const pico_render_config& c = it.config;
        const std::string who = "render " + std::to_string(r) + ": ";
        if (!it.scene || !it.pixels_rgb || !it.sample_count || !it.variance_rgb)
            return set_error(ctx, PICO_ERR_INVALID_ARG, who + "null argument");
        if (it.camera.resolution[0] == 0 || it.camera.resolution[1] == 0 || c.width != it.camera.resolution[0] ||
            c.height != it.camera.resolution[1])
            return set_error(ctx, PICO_ERR_INVALID_ARG, who + "bad image size");
        if (c.estimator != PICO_ESTIMATOR_REFERENCE && c.estimator != PICO_ESTIMATOR_PHYSICAL)
            return set_error(ctx, PICO_ERR_INVALID_ARG, who + "batches take the reference or physical estimator");
        if (c.denoise || c.tonemap) return set_error(ctx, PICO_ERR_INVALID_ARG, who + "batches do not denoise or tone map");
        if (it.scene->ctx != ctx) return set_error(ctx, PICO_ERR_INVALID_ARG, who + "scene of another context");
    }
    return PICO_OK;
}

cudaError_t grow(std::vector<std::unique_ptr<BatchSlot>>& slots, size_t n)
{
    while (slots.size() < n) {
        auto s = std::make_unique<BatchSlot>();
        cudaError_t e = cudaMalloc(&s->status, sizeof(DeviceStatus));
        if (e != cudaSuccess) return e;
        slots.push_back(std::move(s));
    }
    return cudaSuccess;
}

cudaError_t ensure_state(pico_gpu_ctx* ctx, uint32_t nrenders, size_t npieces, uint32_t branches)
{
    if (!ctx->batch) ctx->batch = new BatchState();
    BatchState& bs = *ctx->batch;
    cudaError_t e = grow(bs.images, nrenders);
    if (e == cudaSuccess) e = grow(bs.pieces, npieces);
    while (bs.paths.size() < branches) bs.paths.push_back(std::make_unique<RenderBuffers>());
    while (e == cudaSuccess && bs.streams.size() < branches) {
        cudaStream_t s = nullptr;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) bs.streams.push_back(s);
    }
    if (e == cudaSuccess && bs.stamp_cap < npieces + 1) {
        if (bs.stamps) cudaFree(bs.stamps);
        bs.stamps = nullptr;
        bs.stamp_cap = 0;
        e = cudaMalloc(&bs.stamps, (npieces + 1) * sizeof(unsigned long long));
        if (e == cudaSuccess) bs.stamp_cap = npieces + 1;
    }
    return e;
}

// Uploads one render's progressive buffers and active-pixel list into its image slot.
cudaError_t upload_render(const pico_render_item& it, BatchSlot& s, Prepared& pr, cudaStream_t st,
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
    // the pageable sources above must stay alive until the copies finish
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Splits every render's active pixels into pieces of at most piece_paths paths.
std::vector<Piece> make_pieces(uint32_t n, const pico_render_item* items, const std::vector<Prepared>& prep,
                               const Params& p)
{
    std::vector<Piece> pieces;
    for (uint32_t r = 0; r < n; ++r) {
        const uint32_t spp = items[r].config.max_samples;
        const size_t na = prep[r].nactive;
        if (!na || !spp) continue;
        size_t k = 1;
        if (p.piece_paths) k = std::min<size_t>(na, (na * spp + p.piece_paths - 1) / p.piece_paths);
        for (size_t j = 0; j < k; ++j) {
            Piece pc{r, na * j / k, na * (j + 1) / k, 0, 0};
            const size_t range = pc.p1 - pc.p0;
            pc.chunk_pix = (uint32_t)std::min<size_t>(range, p.wavefront);
            pc.spb_max = std::max<uint32_t>(1u, std::min<uint32_t>(spp, p.wavefront / pc.chunk_pix));
            pieces.push_back(pc);
        }
    }
    return pieces;
}

// A piece's cost: its paths times (1 + min(depth, 4)), an estimate of the
// segments a path traces.
std::vector<double> piece_costs(const std::vector<Piece>& pieces, const pico_render_item* items)
{
    std::vector<double> cost(pieces.size());
    for (size_t j = 0; j < pieces.size(); ++j) {
        const pico_render_config& c = items[pieces[j].render].config;
        cost[j] = (double)(pieces[j].p1 - pieces[j].p0) * c.max_samples * (1.0 + std::min(c.max_ray_depth, 4u));
    }
    return cost;
}

// Which pieces run on which branch, in order.  Pieces are placed costliest
// first on the branch with the least cost so far (longest processing time
// first), so that the branches end close together and no lone branch holds the
// GPU at the end; each branch then runs its pieces cheapest first.
std::vector<std::vector<size_t>> schedule(const std::vector<double>& cost, uint32_t branches)
{
    const size_t np = cost.size();
    std::vector<size_t> order(np);
    for (size_t j = 0; j < np; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<double> load(branches, 0.0);
    std::vector<std::vector<size_t>> lanes(branches);
    for (size_t j : order) {
        const size_t k = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
        lanes[k].push_back(j);
        load[k] += cost[j];
    }
    for (std::vector<size_t>& lane : lanes)
        std::stable_sort(lane.begin(), lane.end(), [&](size_t a, size_t b) { return cost[a] < cost[b]; });
    return lanes;
}

// Scheduling priority of every piece's kernels (lower numbers are higher, as
// for streams): the device's priority levels split the pieces by cost rank, the
// cheapest at the greatest.  Branches interleave roughly kernel by kernel, not by
// work, so without priorities a small render waits behind the big batches of
// every other branch; with them its kernels take the next free SMs.
std::vector<int> piece_priorities(const std::vector<double>& cost, int least, int greatest)
{
    const size_t np = cost.size();
    const size_t levels = (size_t)(least - greatest) + 1;
    std::vector<size_t> order(np);
    for (size_t j = 0; j < np; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] < cost[b]; });
    std::vector<int> prio(np, least);
    for (size_t i = 0; i < np; ++i) prio[order[i]] = greatest + (int)(i * levels / np);
    return prio;
}

// A piece's batches on stream st, without synchronisation (they are captured):
// path state from its branch's slot, status from the piece's, pixels and
// progressive buffers from the render's.
cudaError_t enqueue(pico_gpu_ctx* ctx, const pico_render_item& it, BatchSlot& image, RenderBuffers& paths,
                    DeviceStatus* status, const Params& p, const Prepared& pr, const Piece& pc, cudaStream_t st)
{
    const pico_render_config& cfg = it.config;
    const int order = scene_order(ctx, it.scene);
    cudaError_t e = cudaSuccess;
    for (size_t q0 = pc.p0; q0 < pc.p1 && e == cudaSuccess; q0 += pc.chunk_pix) {
        const uint32_t npix = (uint32_t)std::min<size_t>(pc.chunk_pix, pc.p1 - q0);
        for (uint32_t s0 = 0; s0 < cfg.max_samples && e == cudaSuccess; s0 += pc.spb_max) {
            const uint32_t spb = std::min(pc.spb_max, cfg.max_samples - s0);
            PathBatch b = make_batch(paths, npix * spb, npix, pr.W, as<uint32_t>(image.r.pix_list) + q0);
            b.pixels = as<float>(image.r.pixels);
            b.variance = as<float>(image.r.variance);
            b.count = as<uint32_t>(image.r.count);
            b.taken = as<uint32_t>(image.r.taken);
            b.done = as<uint32_t>(image.r.done);
            b.extend_ctas = p.extend_ctas;
            b.extend_threads = p.extend_threads;
            e = launch_render_batch(traversal_view(ctx, it.scene), b, pr.cam, cfg.seed, spb, cfg.max_ray_depth, cfg.max_samples,
                                    cfg.max_variance, (int)cfg.estimator, status, order, st);
        }
    }
    return e;
}

int run_batch(pico_gpu_ctx* ctx, uint32_t n, const pico_render_item* items, const Params& params,
              double* completion_ms, pico_batch_report* rep)
{
    using clock = std::chrono::steady_clock;
    cudaStream_t st = ctx->stream;
    cudaError_t e = ensure_state(ctx, n, 0, 1);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch state");
    std::vector<Prepared> prep(n);
    std::vector<uint32_t> active, done;
    for (uint32_t r = 0; r < n && e == cudaSuccess; ++r)
        e = upload_render(items[r], *ctx->batch->images[r], prep[r], st, active, done);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch upload");
    const std::vector<Piece> pieces = make_pieces(n, items, prep, params);
    const size_t np = pieces.size();
    Params p = params;
    p.branches = (uint32_t)std::max<size_t>(
        1, std::min<size_t>({p.branches ? (size_t)p.branches : np, np, (size_t)work_queues()}));
    e = ensure_state(ctx, n, np, p.branches);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch state");
    BatchState& bs = *ctx->batch;
    const std::vector<double> cost = piece_costs(pieces, items);
    const std::vector<std::vector<size_t>> lanes = schedule(cost, p.branches);
    // one path slot per branch, sized for the largest batch of its pieces
    std::vector<size_t> lane_paths(p.branches, 0);
    size_t total_paths = 0;
    for (uint32_t k = 0; k < p.branches; ++k) {
        for (size_t j : lanes[k])
            lane_paths[k] = std::max(lane_paths[k], (size_t)pieces[j].chunk_pix * pieces[j].spb_max);
        total_paths += lane_paths[k];
    }
    {
        size_t free_b = 0, total_b = 0, held = 0;
        for (uint32_t k = 0; k < p.branches; ++k) held += bs.paths[k]->org.cap / sizeof(float4) * kPathStateBytes;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && total_paths * kPathStateBytes > free_b + held)
            return set_error(ctx, PICO_ERR_OUT_OF_MEMORY,
                             "batch path state: " + std::to_string(p.branches) + " branches of up to " +
                                 std::to_string(p.wavefront) + " paths need " +
                                 std::to_string(total_paths * kPathStateBytes >> 20) + " MiB, " +
                                 std::to_string((free_b + held) >> 20) + " MiB available; lower the wavefront "
                                 "or the branches");
        cudaGetLastError();
    }
    for (uint32_t k = 0; k < p.branches && e == cudaSuccess; ++k)
        if (lane_paths[k]) e = reserve_paths(*bs.paths[k], lane_paths[k]);
    for (size_t j = 0; j < np && e == cudaSuccess; ++j)
        e = cudaMemsetAsync(bs.pieces[j]->status, 0, sizeof(DeviceStatus), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch path state");

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
    int least = 0, greatest = 0;
    if (ce == cudaSuccess) ce = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const std::vector<int> prio = piece_priorities(cost, least, greatest);
    for (uint32_t k = 0; k < p.branches && ce == cudaSuccess; ++k)
        for (size_t j : lanes[k]) {
            const Piece& pc = pieces[j];
            cudaLaunchAttributeValue pv{};
            pv.priority = prio[j];
            ce = cudaStreamSetAttribute(bs.streams[k], cudaStreamAttributePriority, &pv);
            if (ce == cudaSuccess)
                ce = enqueue(ctx, items[pc.render], *bs.images[pc.render], *bs.paths[k], bs.pieces[j]->status, p,
                             prep[pc.render], pc, bs.streams[k]);
            if (ce == cudaSuccess) ce = launch_stamp(bs.stamps + 1 + j, bs.streams[k]);
            if (ce != cudaSuccess) break;
        }
    for (uint32_t k = 0; k < p.branches && ce == cudaSuccess; ++k) {
        ce = cudaEventRecord(events[1 + k], bs.streams[k]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(st, events[1 + k], 0);
    }
    e = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess) e = ce;
    // the kernels keep the priorities they were captured with
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
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

    std::vector<unsigned long long> stamps(np + 1);
    e = cudaMemcpy(stamps.data(), bs.stamps, stamps.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    std::vector<DeviceStatus> status(np);
    for (size_t j = 0; j < np && e == cudaSuccess; ++j)
        e = cudaMemcpy(&status[j], bs.pieces[j]->status, sizeof(DeviceStatus), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch status");
    uint64_t samples = 0, rays = 0;
    int result = PICO_OK;
    if (completion_ms)
        for (uint32_t r = 0; r < n; ++r) completion_ms[r] = 0.0;
    for (size_t j = 0; j < np; ++j) {
        const DeviceStatus& ds = status[j];
        rays += ds.rays[0] + ds.rays[1] + ds.rays[2];
        const uint32_t r = pieces[j].render;
        if (ds.trace_error && result == PICO_OK)
            result = set_error(ctx, (ds.trace_error & kTraceStackOverflow) ? PICO_ERR_STACK_OVERFLOW : PICO_ERR_TIMEOUT,
                               "render " + std::to_string(r) + ": a traversal failed");
        if (completion_ms) completion_ms[r] = std::max(completion_ms[r], (double)(stamps[1 + j] - stamps[0]) * 1e-6);
    }
    for (uint32_t r = 0; r < n && e == cudaSuccess; ++r) {
        const pico_render_item& it = items[r];
        BatchSlot& s = *bs.images[r];
        const Prepared& pr = prep[r];
        e = cudaMemcpyAsync(it.pixels_rgb, s.r.pixels.ptr, pr.npx * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it.variance_rgb, s.r.variance.ptr, pr.npx * 3 * sizeof(float),
                                                  cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it.sample_count, s.r.count.ptr, pr.npx * sizeof(uint32_t),
                                                  cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        uint64_t after = 0;
        for (size_t px = 0; px < pr.npx; ++px) after += it.sample_count[px];
        samples += after - pr.samples_before;
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch download");
    if (rep) {
        rep->build_ms = std::chrono::duration<double, std::milli>(t_run - t_build).count();
        rep->run_ms = std::chrono::duration<double, std::milli>(t_end - t_run).count();
        rep->graph_nodes = nodes;
        rep->samples = samples;
        rep->rays = rays;
    }
    return result;
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
    const DeviceScope device_scope(ctx->device);
    return run_batch(ctx, n, items, resolve(params), completion_ms, report);
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
    const DeviceScope device_scope(ctx->device);
    // short renders of the same items into scratch buffers: the item with the most
    // samples per pixel takes trial_samples, the others the same fraction of theirs
    // (at least 1), so that the trials keep the batch's balance of work
    uint32_t max_spp = 1;
    for (uint32_t r = 0; r < n; ++r) max_spp = std::max(max_spp, items[r].config.max_samples);
    const uint64_t tspp = std::min<uint64_t>(std::max(1u, trial_samples), max_spp);
    std::vector<uint32_t> trial_spp(n);
    std::vector<pico_render_item> trial(items, items + n);
    std::vector<std::vector<float>> px(n), var(n);
    std::vector<std::vector<uint32_t>> cnt(n);
    uint64_t paths_trial = 0, paths_real = 0;
    for (uint32_t r = 0; r < n; ++r) {
        const uint64_t npx = (uint64_t)items[r].config.width * items[r].config.height;
        trial_spp[r] = (uint32_t)std::max<uint64_t>(1, (items[r].config.max_samples * tspp + max_spp / 2) / max_spp);
        paths_trial += npx * trial_spp[r];
        paths_real += npx * items[r].config.max_samples;
    }
    auto reset = [&]() {
        for (uint32_t r = 0; r < n; ++r) {
            const size_t npx = (size_t)items[r].config.width * items[r].config.height;
            px[r].assign(npx * 3, 0.0f);
            var[r].assign(npx * 3, 0.0f);
            cnt[r].assign(npx, 0u);
            trial[r].pixels_rgb = px[r].data();
            trial[r].variance_rgb = var[r].data();
            trial[r].sample_count = cnt[r].data();
            trial[r].config.max_samples = trial_spp[r];
        }
    };
    // the piece size is tuned as a fraction of all paths (1 / pieces_per_total) and
    // scaled from the trial renders' paths to the items' own
    struct Setting {
        Params p;
        uint32_t pieces_per_total;   // 0: no split
    };
    auto piece_paths = [](uint64_t total, uint32_t per) -> uint32_t {
        if (!per) return 0u;
        return (uint32_t)std::min<uint64_t>(0xffffffffull, std::max<uint64_t>(1, total / per));
    };
    uint32_t count = 0;
    auto measure = [&](const Setting& s, double& msps) -> int {
        reset();
        Params p = s.p;
        p.piece_paths = piece_paths(paths_trial, s.pieces_per_total);
        pico_batch_report rep{};
        const int st = run_batch(ctx, n, trial.data(), p, nullptr, &rep);
        if (st != PICO_OK) return st;
        msps = rep.run_ms > 0.0 ? (double)rep.samples / rep.run_ms / 1e3 : 0.0;
        if (count < max_trials) {
            if (trials_out)
                trials_out[count] = pico_launch_params{p.wavefront, p.extend_ctas, p.branches,
                                                       piece_paths(paths_real, s.pieces_per_total),
                                                       p.extend_threads, 0};
            if (trial_msamples_per_s) trial_msamples_per_s[count] = msps;
        }
        ++count;
        return PICO_OK;
    };
    Setting cur{Params{1u << 20, 0u, 0u, 0u, 128u}, 0u};
    double rate = 0.0;
    status = measure(cur, rate);   // warm-up: module loading, buffer growth
    if (status != PICO_OK) return status;
    count = 0;
    double best_rate = 0.0;
    auto try_axis = [&](auto&& set, std::initializer_list<uint32_t> values) -> int {
        Setting keep = cur;
        for (uint32_t v : values) {
            Setting s = cur;
            set(s, v);
            double m = 0.0;
            const int st = measure(s, m);
            if (st != PICO_OK) return st;
            if (m > best_rate) {
                best_rate = m;
                keep = s;
            }
        }
        cur = keep;
        return PICO_OK;
    };
    status = try_axis([](Setting& s, uint32_t v) { s.p.wavefront = v; }, {1u << 18, 1u << 20, 1u << 22});
    if (status == PICO_OK) status = try_axis([](Setting& s, uint32_t v) { s.p.extend_threads = v; }, {64u, 128u, 256u});
    if (status == PICO_OK) status = try_axis([](Setting& s, uint32_t v) { s.p.extend_ctas = v; }, {2u, 4u, 0u});
    if (status == PICO_OK) status = try_axis([](Setting& s, uint32_t v) { s.pieces_per_total = v; }, {0u, 32u, 128u});
    if (status == PICO_OK) status = try_axis([](Setting& s, uint32_t v) { s.p.branches = v; }, {2u, 4u, 0u});
    if (status != PICO_OK) return status;
    *best = pico_launch_params{cur.p.wavefront, cur.p.extend_ctas, cur.p.branches,
                               piece_paths(paths_real, cur.pieces_per_total), cur.p.extend_threads, 0};
    if (ntrials) *ntrials = std::min(count, max_trials);
    return PICO_OK;
}

}  // extern "C"
