// The C ABI of libpico_gpu (include/pico_gpu.h): contexts, scene upload and
// the closest-hit entry points.  Rendering and denoising live in render.cpp.
#include "capi_internal.h"

#include <cuda.h>   // driver types for cuPointerGetAttribute (resolved at run time, not linked)

#include <cstring>
#include <new>

using namespace pico;

namespace pico {

int set_error(pico_gpu_ctx* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_error(pico_gpu_ctx* ctx, cudaError_t e, const char* what)
{
    cudaGetLastError();   // a failed call's (non-sticky) error is reported here, not to the caller's next CUDA call
    if (e == cudaErrorMemoryAllocation)
        return set_error(ctx, PICO_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    return set_error(ctx, PICO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

cudaError_t DeviceBuffer::reserve(size_t bytes)
{
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&ptr, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
}

void DeviceBuffer::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

// Reads and clears the latched device status; returns a PICO status.
int take_device_status(pico_gpu_ctx* ctx, cudaStream_t stream)
{
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, &ctx->status->trace_error, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "status read");
    if (err) {
        cudaMemsetAsync(&ctx->status->trace_error, 0, sizeof(int), stream);
        cudaStreamSynchronize(stream);
        if (err & kTraceStackOverflow)
            return set_error(ctx, PICO_ERR_STACK_OVERFLOW, "a ray exceeded the traversal stack");
        return set_error(ctx, PICO_ERR_TIMEOUT, "a traversal exceeded its iteration bound");
    }
    return PICO_OK;
}

}  // namespace pico

extern "C" {

int pico_gpu_init(int device, pico_gpu_ctx** out)
{
    if (!out) return PICO_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return PICO_ERR_NO_DEVICE;
    if (device < 0 || device >= count) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(device);
    if (device_scope.status != cudaSuccess) return PICO_ERR_CUDA;
    auto* ctx = new (std::nothrow) pico_gpu_ctx();
    if (!ctx) return PICO_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->status, 2 * sizeof(DeviceStatus));
    if (e == cudaSuccess) e = cudaMemset(ctx->status, 0, 2 * sizeof(DeviceStatus));
    if (e != cudaSuccess) {
        pico_gpu_shutdown(ctx);
        return e == cudaErrorMemoryAllocation ? PICO_ERR_OUT_OF_MEMORY : PICO_ERR_CUDA;
    }
    *out = ctx;
    return PICO_OK;
}

void pico_gpu_shutdown(pico_gpu_ctx* ctx)
{
    if (!ctx) return;
    const DeviceScope device_scope(ctx->device);
    for (DeviceBuffer* b : {&ctx->buf_a, &ctx->buf_b, &ctx->buf_c, &ctx->buf_d, &ctx->buf_e}) b->release();
    if (ctx->bounce_in) cudaFreeHost(ctx->bounce_in);
    if (ctx->bounce_out) cudaFreeHost(ctx->bounce_out);
    free_render_buffers(ctx);
    free_batch_state(ctx);
    if (ctx->status) cudaFree(ctx->status);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    delete ctx;
}

const char* pico_gpu_status_string(int status)
{
    switch (status) {
    case PICO_OK: return "ok";
    case PICO_ERR_INVALID_ARG: return "invalid argument";
    case PICO_ERR_CUDA: return "CUDA error";
    case PICO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PICO_ERR_STACK_OVERFLOW: return "traversal stack overflow";
    case PICO_ERR_TIMEOUT: return "device loop bound reached";
    case PICO_ERR_CANCELLED: return "cancelled";
    case PICO_ERR_NO_DEVICE: return "no CUDA device";
    case PICO_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

const char* pico_gpu_last_error(const pico_gpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int pico_gpu_set_traversal_order(pico_gpu_ctx* ctx, int order)
{
    if (!ctx || (order != PICO_ORDER_NEAR_FIRST && order != PICO_ORDER_REFERENCE))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "unknown traversal order");
    ctx->order = order;
    return PICO_OK;
}

int pico_gpu_set_traversal_limits(pico_gpu_ctx* ctx, uint32_t max_iterations, uint32_t stack_entries)
{
    if (!ctx) return PICO_ERR_INVALID_ARG;
    if (max_iterations == 0) max_iterations = kTraceMaxIter;
    if (stack_entries == 0) stack_entries = kTraceStack;
    if (stack_entries > (uint32_t)kTraceStack)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "the traversal stack has 96 entries");
    ctx->max_iterations = max_iterations;
    ctx->stack_entries = stack_entries;
    return PICO_OK;
}

int pico_gpu_set_triangle_test(pico_gpu_ctx* ctx, int test)
{
    if (!ctx || (test != PICO_TRIANGLE_MOLLER_TRUMBORE && test != PICO_TRIANGLE_WATERTIGHT))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "unknown triangle test");
    ctx->triangle_test = test;
    return PICO_OK;
}

int pico_gpu_scene_upload(pico_gpu_ctx* ctx, const pico_scene_desc* desc, pico_gpu_scene** out)
{
    if (!ctx || !desc || !out) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    const DeviceScope device_scope(ctx->device);
    FlatScene fs;
    const std::string why = build_flat_scene(*desc, fs);
    if (!why.empty()) {
        const bool unsupported = why.find("not supported") != std::string::npos;
        return set_error(ctx, unsupported ? PICO_ERR_UNSUPPORTED : PICO_ERR_INVALID_ARG, why);
    }
    auto* s = new (std::nothrow) pico_gpu_scene();
    if (!s) return set_error(ctx, PICO_ERR_OUT_OF_MEMORY, "host allocation");
    s->ctx = ctx;
    s->nlights = (uint32_t)fs.lights.size();
    s->ninstances = (uint32_t)fs.inst_shade.size();
    s->inst_rank_host = fs.inst_rank;
    bool implicit = false;
    for (uint32_t i = 0; i < desc->ninstances; ++i) {
        const uint32_t shape = desc->meshes[desc->instances[i].mesh].shape;
        if (shape == PICO_SHAPE_SPHERE) s->needs_reference_order = true;
        if (shape != PICO_SHAPE_TRIANGLES) implicit = true;
        const uint32_t kind = desc->instances[i].bsdf;
        if (kind == PICO_BSDF_BTDF || kind == PICO_BSDF_FRESNEL) s->has_btdf = true;
    }
    s->light_inst_host.reserve(fs.lights.size());
    for (const GpuLight& l : fs.lights) s->light_inst_host.push_back(l.inst);

    size_t total = 0;
    auto upload = [&](const auto& vec, auto*& dst) -> cudaError_t {
        using T = typename std::decay_t<decltype(vec)>::value_type;
        dst = nullptr;
        const size_t bytes = vec.size() * sizeof(T);
        if (bytes == 0) return cudaSuccess;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return e;
        s->allocations.push_back(p);
        total += bytes;
        e = cudaMemcpy(p, vec.data(), bytes, cudaMemcpyHostToDevice);
        dst = static_cast<std::remove_reference_t<decltype(dst)>>(p);
        return e;
    };
    SceneView& v = s->view;
    std::memset(&v, 0, sizeof v);
    cudaError_t e = cudaSuccess;
    const GpuNode* nodes; const GpuTri* tris; const GpuTriShade* tshade; const GpuInstance* insts;
    const GpuInstanceShade* ishade; const uint32_t* irank; const GpuMaterial* mats; const GpuLight* lights;
    const float* law; const uint32_t* lai; const float* lpos; const unsigned char* skypx; const uint32_t* titems;
    const float* lgeo; const uint32_t* lofi; const float* lpick; const float* lbox;
    if (e == cudaSuccess) e = upload(fs.nodes, nodes);
    if (e == cudaSuccess) e = upload(fs.tris, tris);
    if (e == cudaSuccess) e = upload(fs.tri_shade, tshade);
    if (e == cudaSuccess) e = upload(fs.insts, insts);
    if (e == cudaSuccess) e = upload(fs.inst_shade, ishade);
    if (e == cudaSuccess) e = upload(fs.inst_rank, irank);
    if (e == cudaSuccess) e = upload(fs.materials, mats);
    if (e == cudaSuccess) e = upload(fs.lights, lights);
    if (e == cudaSuccess) e = upload(fs.light_alias_weight, law);
    if (e == cudaSuccess) e = upload(fs.light_alias_index, lai);
    if (e == cudaSuccess) e = upload(fs.light_positions, lpos);
    if (e == cudaSuccess) e = upload(fs.light_tri_geo, lgeo);
    if (e == cudaSuccess) e = upload(fs.light_of_inst, lofi);
    if (e == cudaSuccess) e = upload(fs.light_pick, lpick);
    if (e == cudaSuccess) e = upload(fs.light_boxes, lbox);
    if (e == cudaSuccess) e = upload(fs.sky_pixels, skypx);
    if (e == cudaSuccess) e = upload(fs.tlas_items, titems);
    if (e != cudaSuccess) {
        pico_gpu_scene_free(s);
        return cuda_error(ctx, e, "scene upload");
    }
    v.nodes = nodes; v.tris = tris; v.tri_shade = tshade; v.insts = insts; v.inst_shade = ishade;
    v.inst_rank = irank; v.tlas_items = titems; v.materials = mats; v.lights = lights; v.light_alias_weight = law;
    v.light_alias_index = lai; v.light_positions = lpos; v.light_tri_geo = lgeo; v.light_of_inst = lofi;
    v.light_pick = lpick;
    v.light_boxes = lbox;
    v.light_bounds = fs.light_bounds ? 1u : 0u;
    v.nlights = (uint32_t)fs.lights.size();
    v.tlas_root_ref = fs.tlas_root_ref;
    v.tlas_fast_root_ref = fs.tlas_fast_root_ref;
    for (int a = 0; a < 3; ++a) {
        v.tlas_lo[a] = fs.tlas_lo[a]; v.tlas_hi[a] = fs.tlas_hi[a]; v.sky[a] = fs.sky[a];
        v.tlas_fast_lo[a] = fs.tlas_fast_lo[a]; v.tlas_fast_hi[a] = fs.tlas_fast_hi[a];
    }
    v.ninstances = (uint32_t)fs.inst_shade.size();
    v.has_implicit = implicit ? 1u : 0u;
    v.sky_kind = fs.sky_kind; v.sky_w = fs.sky_w; v.sky_h = fs.sky_h; v.sky_pixels = skypx;
    v.use_sun = fs.use_sun;
    v.max_iterations = kTraceMaxIter;
    v.stack_entries = kTraceStack;
    v.watertight = 0;
    for (int a = 0; a < 3; ++a) { v.sun_dir[a] = fs.sun_dir[a]; v.sun_col[a] = fs.sun_col[a]; }
    {
        bool finite = true;
        auto fin = [](float x) { return std::isfinite(x); };
        for (const GpuNode& n : fs.nodes) {
            if (n.ref0 != PICO_REF_EMPTY)
                finite = finite && fin(n.c0lox) && fin(n.c0hix) && fin(n.c0loy) && fin(n.c0hiy) && fin(n.c0loz) &&
                         fin(n.c0hiz);
            if (n.ref1 != PICO_REF_EMPTY)
                finite = finite && fin(n.c1lox) && fin(n.c1hix) && fin(n.c1loy) && fin(n.c1hiy) && fin(n.c1loz) &&
                         fin(n.c1hiz);
        }
        for (int a = 0; a < 3; ++a)
            finite = finite && fin(fs.tlas_lo[a]) && fin(fs.tlas_hi[a]) && fin(fs.tlas_fast_lo[a]) &&
                     fin(fs.tlas_fast_hi[a]);
        v.finite_boxes = finite ? 1u : 0u;
    }
    s->info[0] = fs.tlas_nodes; s->info[1] = fs.blas_nodes; s->info[2] = fs.tris.size();
    s->info[3] = fs.insts.size(); s->info[4] = total; s->info[5] = fs.lights.size();
    *out = s;
    return PICO_OK;
}

int pico_gpu_reference_bvh(const pico_scene_desc* desc, int32_t which, float* boxes, uint32_t* links,
                           uint32_t* values, uint32_t* nnodes, uint32_t* nvalues)
{
    if (!desc || !nnodes || !nvalues) return PICO_ERR_INVALID_ARG;
    if (which < -1 || which >= (int64_t)desc->nmeshes) return PICO_ERR_INVALID_ARG;
    FlatScene fs;
    fs.keep_trees = true;
    const std::string why = build_flat_scene(*desc, fs);
    if (!why.empty()) return why.find("not supported") != std::string::npos ? PICO_ERR_UNSUPPORTED : PICO_ERR_INVALID_ARG;
    const TreeDump& t = which < 0 ? fs.tlas_tree : fs.blas_trees[which];
    *nnodes = (uint32_t)(t.links.size() / 4);
    *nvalues = (uint32_t)t.values.size();
    if (boxes) std::memcpy(boxes, t.boxes.data(), t.boxes.size() * sizeof(float));
    if (links) std::memcpy(links, t.links.data(), t.links.size() * sizeof(uint32_t));
    if (values) std::memcpy(values, t.values.data(), t.values.size() * sizeof(uint32_t));
    return PICO_OK;
}

void pico_gpu_scene_free(pico_gpu_scene* s)
{
    if (!s) return;
    const DeviceScope device_scope(s->ctx ? s->ctx->device : -1);
    for (void* p : s->allocations) cudaFree(p);
    delete s;
}

int pico_gpu_scene_info(const pico_gpu_scene* s, uint64_t* out6)
{
    if (!s || !out6) return PICO_ERR_INVALID_ARG;
    std::memcpy(out6, s->info, sizeof(s->info));
    return PICO_OK;
}

int pico_gpu_trace_closest_device(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_ray* d_rays,
                                  uint64_t n, pico_hit* d_hits, void* stream)
{
    if (!ctx || !scene || (n && (!d_rays || !d_hits))) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (reinterpret_cast<uintptr_t>(d_rays) % 16 != 0) return set_error(ctx, PICO_ERR_INVALID_ARG, "rays not 16-byte aligned");
    const DeviceScope device_scope(ctx->device);
    const cudaError_t e = launch_trace(traversal_view(ctx, scene), d_rays, n, d_hits, ctx->status, false,
                                       scene_order(ctx, scene), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error(ctx, e, "trace launch");
    return PICO_OK;
}

int pico_gpu_check(pico_gpu_ctx* ctx, void* stream)
{
    if (!ctx) return PICO_ERR_INVALID_ARG;
    const DeviceScope device_scope(ctx->device);
    const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error(ctx, e, "stream");
    return take_device_status(ctx, static_cast<cudaStream_t>(stream));
}

int pico_gpu_trace_stats(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_ray* d_rays, uint64_t n,
                         uint64_t* out3, void* stream)
{
    if (!ctx || !scene || !out3 || (n && !d_rays)) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = ctx->buf_e.reserve(sizeof(pico_hit) * (n ? n : 1));
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status->counters, 0, sizeof(ctx->status->counters), st);
    if (e == cudaSuccess)
        e = launch_trace(traversal_view(ctx, scene), d_rays, n, static_cast<pico_hit*>(ctx->buf_e.ptr), ctx->status, true, scene_order(ctx, scene), st);
    unsigned long long c[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(c, ctx->status->counters, sizeof c, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "trace stats");
    out3[0] = c[0]; out3[1] = c[1]; out3[2] = c[2];
    return take_device_status(ctx, st);
}

}  // extern "C"

namespace {

// cuPointerGetAttribute, resolved through the runtime (the library does not link
// the driver library itself); null where the driver does not provide it.
using PointerAttributeFn = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
PointerAttributeFn pointer_attribute_fn()
{
    static PointerAttributeFn fn = []() -> PointerAttributeFn {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return reinterpret_cast<PointerAttributeFn>(f);
    }();
    return fn;
}

// The address range [start, start + size) of the allocation (or registration) that
// holds p, as the driver reports it; false when it reports none.
bool allocation_range(const void* p, uintptr_t& start, size_t& size)
{
    const PointerAttributeFn fn = pointer_attribute_fn();
    if (!fn) return false;
    CUdeviceptr s = 0;
    size_t n = 0;
    const CUdeviceptr dp = static_cast<CUdeviceptr>(reinterpret_cast<uintptr_t>(p));
    if (fn(&s, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, dp) != CUDA_SUCCESS ||
        fn(&n, CU_POINTER_ATTRIBUTE_RANGE_SIZE, dp) != CUDA_SUCCESS || n == 0)
        return false;
    start = static_cast<uintptr_t>(s);
    size = n;
    return true;
}

// The device address of [p, p + bytes) when the whole range lies in ONE page-locked
// host allocation mapped into `device`'s address space (cudaHostAlloc, or one
// cudaHostRegister under unified addressing, pinned against that device); null
// otherwise: pageable memory, memory pinned against another device, and ranges
// that span several pinned regions (pageable memory may lie between them), which
// the kernels never touch.
void* mapped_range(const void* p, size_t bytes, int device)
{
    cudaPointerAttributes a{}, b{};
    const char* last = static_cast<const char*>(p) + (bytes - 1);
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&b, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer ||
        a.device != device || b.device != device)
        return nullptr;
    if (static_cast<const char*>(b.devicePointer) - static_cast<const char*>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    uintptr_t start = 0;
    size_t size = 0;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(p);
    if (!allocation_range(p, start, size) || lo < start || lo - start > size || bytes > size - (lo - start))
        return nullptr;
    return a.devicePointer;
}

// Whether either end of [p, p + bytes) lies in page-locked host memory.
bool pinned_end(const void* p, size_t bytes)
{
    for (const void* q : {p, static_cast<const void*>(static_cast<const char*>(p) + (bytes - 1))}) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (a.type == cudaMemoryTypeHost) return true;
    }
    return false;
}

// Host-buffer closest hit for ranges that are only partly page-locked (an end in a
// pinned region, the rest not inside it): the copy engine accepts such a range
// neither as pinned nor as pageable memory, so each chunk is copied on the host
// into page-locked bounce buffers of the context and moved from there; chunk by
// chunk on one stream.
int trace_via_bounce(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_ray* rays, uint64_t n, pico_hit* hits)
{
    const uint64_t chunk = n < (1ull << 20) ? n : (1ull << 20);
    cudaError_t e = cudaSuccess;
    if (ctx->bounce_rays < chunk) {
        if (ctx->bounce_in) cudaFreeHost(ctx->bounce_in);
        if (ctx->bounce_out) cudaFreeHost(ctx->bounce_out);
        ctx->bounce_in = ctx->bounce_out = nullptr;
        ctx->bounce_rays = 0;
        e = cudaHostAlloc(&ctx->bounce_in, chunk * sizeof(pico_ray), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaHostAlloc(&ctx->bounce_out, chunk * sizeof(pico_hit), cudaHostAllocDefault);
        if (e == cudaSuccess) ctx->bounce_rays = chunk;
    }
    if (e == cudaSuccess) e = ctx->buf_a.reserve(chunk * sizeof(pico_ray));
    if (e == cudaSuccess) e = ctx->buf_c.reserve(chunk * sizeof(pico_hit));
    if (e != cudaSuccess) return cuda_error(ctx, e, "bounce buffers");
    cudaStream_t st = ctx->stream;
    pico_ray* dr = static_cast<pico_ray*>(ctx->buf_a.ptr);
    pico_hit* dh = static_cast<pico_hit*>(ctx->buf_c.ptr);
    for (uint64_t off = 0; off < n && e == cudaSuccess; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        std::memcpy(ctx->bounce_in, rays + off, m * sizeof(pico_ray));
        e = cudaMemcpyAsync(dr, ctx->bounce_in, m * sizeof(pico_ray), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = launch_trace(traversal_view(ctx, scene), dr, m, dh, ctx->status, false, scene_order(ctx, scene), st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->bounce_out, dh, m * sizeof(pico_hit), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) std::memcpy(hits + off, ctx->bounce_out, m * sizeof(pico_hit));
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "trace");
    return take_device_status(ctx, st);
}

}  // namespace

extern "C" int pico_gpu_host_buffer_in_place(pico_gpu_ctx* ctx, const void* p, uint64_t bytes, int32_t* in_place)
{
    if (!ctx || !in_place || (bytes && !p)) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    *in_place = (bytes && mapped_range(p, (size_t)bytes, ctx->device)) ? 1 : 0;
    return PICO_OK;
}

extern "C" {

// Host-buffer closest hit.  Page-locked, mapped buffers are traversed in place:
// one launch reads the rays and writes the hits through their device addresses
// (over NVLink-C2C on a Grace host), with no staging copies.  Other buffers are
// cut into chunks that alternate between two streams, so the copy of one chunk
// overlaps the traversal of the other.
int pico_gpu_trace_closest(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_ray* rays, uint64_t n,
                           pico_hit* hits)
{
    if (!ctx || !scene || (n && (!rays || !hits))) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    if (n == 0) return PICO_OK;
    {
        const size_t rb = n * sizeof(pico_ray), hb = n * sizeof(pico_hit);
        const void* mr = mapped_range(rays, rb, ctx->device);
        void* mh = mapped_range(hits, hb, ctx->device);
        if (mr && mh) {
            cudaError_t e = launch_trace(traversal_view(ctx, scene), static_cast<const pico_ray*>(mr), n, static_cast<pico_hit*>(mh),
                                         ctx->status, false, scene_order(ctx, scene), ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) return cuda_error(ctx, e, "trace");
            return take_device_status(ctx, ctx->stream);
        }
        if ((!mr && pinned_end(rays, rb)) || (!mh && pinned_end(hits, hb))) return trace_via_bounce(ctx, scene, rays, n, hits);
    }
    // 1M-ray chunks alternate between two streams: each chunk's copies overlap the
    // other stream's traversal, and only the first upload and the last download
    // (32 MB / 20 MB) stay exposed
    const uint64_t chunk = n < (1ull << 20) ? n : (1ull << 20);
    cudaError_t e = ctx->buf_a.reserve(chunk * sizeof(pico_ray));
    if (e == cudaSuccess) e = ctx->buf_b.reserve(chunk * sizeof(pico_ray));
    if (e == cudaSuccess) e = ctx->buf_c.reserve(chunk * sizeof(pico_hit));
    if (e == cudaSuccess) e = ctx->buf_d.reserve(chunk * sizeof(pico_hit));
    if (e != cudaSuccess) return cuda_error(ctx, e, "staging allocation");
    cudaStream_t streams[2] = {ctx->stream, ctx->stream2};
    DeviceBuffer* rbuf[2] = {&ctx->buf_a, &ctx->buf_b};
    DeviceBuffer* hbuf[2] = {&ctx->buf_c, &ctx->buf_d};
    for (uint64_t off = 0, k = 0; off < n && e == cudaSuccess; off += chunk, ++k) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        const int s = (int)(k & 1);
        pico_ray* dr = static_cast<pico_ray*>(rbuf[s]->ptr);
        pico_hit* dh = static_cast<pico_hit*>(hbuf[s]->ptr);
        e = cudaMemcpyAsync(dr, rays + off, m * sizeof(pico_ray), cudaMemcpyHostToDevice, streams[s]);
        if (e == cudaSuccess)
            e = launch_trace(traversal_view(ctx, scene), dr, m, dh, s ? ctx->status2() : ctx->status, false, scene_order(ctx, scene), streams[s]);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hits + off, dh, m * sizeof(pico_hit), cudaMemcpyDeviceToHost, streams[s]);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(streams[0]);
    if (e == cudaSuccess) e = cudaStreamSynchronize(streams[1]);
    if (e != cudaSuccess) return cuda_error(ctx, e, "trace");
    // both streams' latched statuses are read and cleared, whatever the first holds,
    // so that no error of this call is left for the next one to report
    int err2 = 0;
    e = cudaMemcpy(&err2, &ctx->status2()->trace_error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && err2) e = cudaMemset(&ctx->status2()->trace_error, 0, sizeof(int));
    const int st = take_device_status(ctx, ctx->stream);
    if (e != cudaSuccess) return cuda_error(ctx, e, "status read");
    if (st == PICO_OK && err2)
        return set_error(ctx, (err2 & kTraceStackOverflow) ? PICO_ERR_STACK_OVERFLOW : PICO_ERR_TIMEOUT,
                         (err2 & kTraceStackOverflow) ? "a ray exceeded the traversal stack"
                                                      : "a traversal exceeded its iteration bound");
    return st;
}

}  // extern "C"
