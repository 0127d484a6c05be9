// pico_gpu_atrous_device_noalloc: the a-trous denoiser (Util::atrous_denoise,
// the same kernels as pico_gpu_atrous_device) on caller device buffers, with its
// scratch in a fixed device array instead of buffers grown on demand.
//
// Who needs it: callers that must not allocate device memory from inside their
// denoise step.  cudaFree (and often cudaMalloc) synchronises the whole device,
// so a frame loop that overlaps rendering, denoising and copies on several
// streams would stall whenever the context's buffers grow; and a process whose
// device memory is owned by another allocator (a framework's caching allocator
// holding most of HBM, or a fixed per-process memory budget) cannot let a
// library take memory behind that allocator's back.  On success this entry
// point allocates nothing, on the device or the host: no cudaMalloc, cudaFree
// or allocating library routine.  Its scratch is the file-scope array below,
// which the CUDA runtime creates with this file's module on each device.
//
// Limits and sharing:
//   * at most kNoAllocMaxPixels = 2,097,152 pixels (1920 x 1080 fits) and
//     65,535 rows per call; larger images are rejected with
//     PICO_ERR_INVALID_ARG and a message in the context, before any launch;
//   * the array takes 48 MiB + 5.5 MiB of device memory on each device;
//   * the output must not overlap any input (the last level writes it while it
//     still reads the colour and the G-buffer): rejected with PICO_ERR_INVALID_ARG;
//   * every call on a device shares that one array, so calls whose kernels
//     overlap on the GPU (different streams, or different host threads) race
//     and corrupt each other's output: order them on one stream or with events;
//   * nothing in the scratch has to start at zero: each level writes its tile
//     statistics and its ping-pong image in full before reading them;
//   * set-up: the first call on a device (with that device current) looks up
//     the array's address with cudaGetSymbolAddress and caches it; that first
//     call should come before any stream capture.
#include "capi_internal.h"
#include "kernels_render.h"

#include <atomic>
#include <mutex>

namespace {

constexpr size_t kNoAllocMaxPixels = size_t(1) << 21;
constexpr uint32_t kNoAllocMaxRows = 65535;            // the blend kernel's grid.y
// 64 x 64 statistics tiles: ceil(W / 64) * ceil(H / 64).  An image of at most 2^21
// pixels in at most 64 rows has one tile row of at most 2^21 / 64 tiles (a single
// row of 2^21 pixels is the worst case); from 65 rows on it has at most 2^21 / 65
// columns, so at most 505 tiles per tile row and far fewer than 2^15 in all.
constexpr size_t kNoAllocMaxTiles = kNoAllocMaxPixels / 64;
static_assert(kNoAllocMaxTiles == 32768, "32,768 statistics tiles");
constexpr size_t kNoAllocImageFloats = 3 * kNoAllocMaxPixels;
// The statistics (pico::atrous_stats_floats): 14 floats per tile, and 10 per image row and
// tile column, of which an accepted image has at most 2^21 / 64 + 65,535 (H * ceil(W / 64)
// <= W * H / 64 + H).
constexpr size_t kNoAllocStatsFloats = 14 * kNoAllocMaxTiles + 10 * (kNoAllocMaxPixels / 64 + kNoAllocMaxRows);
constexpr size_t kNoAllocFloats = 2 * kNoAllocImageFloats + kNoAllocStatsFloats;
constexpr int kNoAllocMaxDevices = 64;

}  // namespace

// Ping-pong image A, ping-pong image B, then the per-tile statistics (white-point
// partials and per-level |position| ranges).
static __device__ __align__(256) float pico_atrous_noalloc_scratch[kNoAllocFloats];

namespace {

std::atomic<float*> g_scratch_of_device[kNoAllocMaxDevices];
std::mutex g_setup_mutex;

// The scratch array's address on `device`, which must be current.
cudaError_t scratch_for_device(int device, float** out)
{
    float* p = g_scratch_of_device[device].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        p = g_scratch_of_device[device].load(std::memory_order_relaxed);
        if (!p) {
            void* addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, pico_atrous_noalloc_scratch);
            if (e != cudaSuccess) return e;
            p = static_cast<float*>(addr);
            g_scratch_of_device[device].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace

using namespace pico;

extern "C" int pico_gpu_atrous_device_noalloc(pico_gpu_ctx* ctx, const float* d_pixels, const float* d_normals,
                                              const float* d_positions, const float* d_diffuse, uint32_t width,
                                              uint32_t height, float* d_out, void* stream)
{
    if (!ctx || !d_pixels || !d_normals || !d_positions || !d_diffuse || !d_out)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const size_t npx = (size_t)width * height;
    const size_t tiles = (size_t)((width + 63) / 64) * ((height + 63) / 64);
    if (npx > kNoAllocMaxPixels || height > kNoAllocMaxRows || tiles > kNoAllocMaxTiles ||
        atrous_stats_floats(width, height) > kNoAllocStatsFloats)
        return set_error(ctx, PICO_ERR_INVALID_ARG,
                         "a-trous without allocation: the image exceeds the fixed scratch "
                         "(at most 2,097,152 pixels and 65,535 rows)");
    if (atrous_output_aliases(d_out, d_pixels, d_normals, d_positions, d_diffuse, 3 * npx))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "the output must not overlap an input");
    if (npx == 0) return PICO_OK;
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return set_error(ctx, PICO_ERR_INVALID_ARG, "a-trous without allocation: device index above 63");
    const DeviceScope device_scope(ctx->device);   // the caller's current device comes back on return
    cudaError_t e = device_scope.status;
    float* scratch = nullptr;
    if (e == cudaSuccess) e = scratch_for_device(ctx->device, &scratch);
    if (e == cudaSuccess)
        e = launch_atrous(d_pixels, d_normals, d_positions, d_diffuse, width, height, scratch,
                          scratch + kNoAllocImageFloats, scratch + 2 * kNoAllocImageFloats, d_out,
                          static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error(ctx, e, "a-trous without allocation");
    return PICO_OK;
}
