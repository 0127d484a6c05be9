// Roofline probe: the read bandwidth of the L2 cache, the roof of the closest-hit
// kernels, whose scene data (nodes, triangles, instances: a few MB) stays
// resident in L2 while only the ray and hit streams reach DRAM.
//
// One launch reads an L2-resident buffer `passes` times with loads that are
// cached in L2 only (ld.global.cg: an L1 hit would measure L1 instead), 16 bytes
// per load, four independent loads in flight per thread, on a persistent grid of
// every SM's full thread complement.  Nothing is written (a data-dependent store
// that never happens keeps the loads), so the bytes are reads alone.
#include "capi_internal.h"

namespace {

constexpr int kProbeThreads = 512;

__device__ __forceinline__ uint4 load_cg(const uint4* p)
{
    uint4 v;
    asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t mix(uint32_t acc, uint4 v)
{
    return acc * 31u + (v.x ^ v.y ^ v.z ^ v.w);
}

__global__ void __launch_bounds__(kProbeThreads) l2_read_kernel(const uint4* __restrict__ buf, size_t n16,
                                                                uint32_t passes, uint32_t* sink)
{
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (uint32_t p = 0; p < passes; ++p) {
        size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            const uint4 a = load_cg(buf + i), b = load_cg(buf + i + stride);
            const uint4 c = load_cg(buf + i + 2 * stride), d = load_cg(buf + i + 3 * stride);
            acc = mix(mix(mix(mix(acc, a), b), c), d);
        }
        for (; i < n16; i += stride) acc = mix(acc, load_cg(buf + i));
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;   // keeps the loads; practically never taken
}

}  // namespace

using namespace pico;

extern "C" int pico_gpu_l2_read_bandwidth(pico_gpu_ctx* ctx, uint64_t bytes, uint32_t passes, double* gbs)
{
    if (!ctx || !gbs) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (bytes == 0) bytes = 32ull << 20;
    if (passes == 0) passes = 100;
    bytes &= ~15ull;
    if (bytes < (1ull << 20) || bytes > (1ull << 30))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "probe buffer must hold 1 MiB to 1 GiB");
    const DeviceScope device_scope(ctx->device);
    cudaStream_t st = ctx->stream;
    void* buf = nullptr;
    uint32_t* sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0x5a, bytes, st);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, l2_read_kernel, kProbeThreads, 0);
    const unsigned grid = (unsigned)(sm_count() * (per_sm > 0 ? per_sm : 1));
    const size_t n16 = bytes / 16;
    float best = 0.0f;
    if (e == cudaSuccess) {
        l2_read_kernel<<<grid, kProbeThreads, 0, st>>>(static_cast<const uint4*>(buf), n16, 2, sink);   // into L2
        e = cudaGetLastError();
    }
    for (int trial = 0; trial < 5 && e == cudaSuccess; ++trial) {
        e = cudaEventRecord(a, st);
        if (e == cudaSuccess) l2_read_kernel<<<grid, kProbeThreads, 0, st>>>(static_cast<const uint4*>(buf), n16,
                                                                            passes, sink);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(b, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && ms > 0.0f) {
            const float g = (float)((double)bytes * passes / (ms * 1e-3) / 1e9);
            if (g > best) best = g;
        }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (sink) cudaFree(sink);
    if (buf) cudaFree(buf);
    if (e != cudaSuccess) return cuda_error(ctx, e, "L2 probe");
    *gbs = best;
    return PICO_OK;
}
