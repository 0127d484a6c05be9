// Closest-hit kernel for ray batches (UpperLevelBVH::get_closest_intersection
// over many rays, Core/UpperLevelBVH.cpp:12-20).
//
// Persistent: the grid is a whole number of CTAs per SM and the warps pull rays
// from a global counter, so long rays do not leave SMs idle at the tail of the
// batch.  In the near-first order a warp's lanes walk the batch with
// walk_queue: one ballot per move decides whether the rarer moves wait, and
// idle lanes take new rays in batches; in the reference order each warp takes
// 32 rays at a time and each lane runs its ray to completion.  128 threads with
// at most 64 registers each keep eight CTAs resident per SM.  Rays are 32 B
// (two 16-byte loads), hits 20 B.
#include "kernels.h"
#include "traverse.cuh"

#include <map>
#include <mutex>
#include <utility>

namespace pico {

constexpr int kTraceThreads = 128;
constexpr int kTraceMinBlocks = 8;

__device__ __forceinline__ void write_hit(const SceneView& sc, const TraceHit& h, int s, pico_hit* out)
{
    pico_hit r;
    if (h.rank != kNoHit && s == kTraceOk) {
        r.inst = sc.insts[h.rank].inst_id;
        r.prim = h.tri == kImplicitTri ? kImplicitTri : sc.tris[h.tri].prim;
        r.t = h.t; r.u = h.u; r.v = h.v;
    } else {
        r.inst = kNoHit; r.prim = kNoHit;
        r.t = __int_as_float(0x7f800000); r.u = 0.0f; r.v = 0.0f;
    }
    *out = r;
}

// The rays of a batch for walk_queue: a lane's tag is the ray's index.
struct BatchRays {
    using Tag = uint64_t;
    using Index = uint64_t;
    const SceneView& sc;
    const float4* rays;
    pico_hit* hits;
    DeviceStatus* status;

    __device__ __forceinline__ uint64_t load(uint64_t k, float4& o, float4& d, float& tmax, float& exit_below,
                                             bool& occlusion) const
    {
        o = __ldg(rays + 2 * k);
        d = __ldg(rays + 2 * k + 1);
        tmax = INFINITY;
        exit_below = -INFINITY;
        occlusion = false;
        return k;
    }

    __device__ __forceinline__ void finish(uint64_t tag, const TraceHit& h, int s) const
    {
        if (s != kTraceOk) atomicOr(&status->trace_error, s);
        write_hit(sc, h, s, hits + tag);
    }
};

template <bool kCount, int kOrder>
__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks)
    trace_kernel(SceneView sc, const float4* __restrict__ rays, uint64_t n, pico_hit* __restrict__ hits,
                 DeviceStatus* status)
{
    TraceCounters cnt{0, 0, 0, 0};
    if constexpr ((kOrder & kReferenceOrder) == 0) {
        BatchRays src{sc, rays, hits, status};
        walk_queue<kCount, (kOrder & kWithImplicit) != 0, (kOrder & kBounded) != 0, (kOrder & kWatertight) != 0>(
            sc, src, n, &status->work, &cnt);
    } else {
        const unsigned lane = threadIdx.x & 31u;
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&status->work, 32ull);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            const unsigned long long i = base + lane;
            if (i < n) {
                const float4 o = __ldg(rays + 2 * i), d = __ldg(rays + 2 * i + 1);
                TraceHit h;
                const int s = trace_closest<kCount, kOrder>(sc, o, d, h, &cnt);
                if (s != kTraceOk) atomicOr(&status->trace_error, s);
                write_hit(sc, h, s, hits + i);
            }
        }
    }
    if (kCount) flush_counters(cnt, status->counters);
}

int sm_count()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

int resident_blocks(const void* kernel, int threads)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> cache;
    const std::pair<const void*, int> key(kernel, threads);
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess || n < 1) {
        cudaGetLastError();   // a failed query leaves no error behind for the next launch check
        n = 1;
    }
    cache.emplace(key, n);
    return n;
}

template <bool kCount, int kOrder>
static cudaError_t launch_trace_t(const SceneView& sc, const float4* r, uint64_t n, pico_hit* hits,
                                  DeviceStatus* status, cudaStream_t stream)
{
    static int per_sm = 0;
    if (!per_sm) {
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel<kCount, kOrder>,
                                                                            kTraceThreads, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    uint64_t blocks = (uint64_t)sm_count() * (uint64_t)per_sm;
    const uint64_t needed = (n + kTraceThreads - 1) / kTraceThreads;
    if (blocks > needed) blocks = needed;
    trace_kernel<kCount, kOrder><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(sc, r, n, hits, status);
    return cudaGetLastError();
}

cudaError_t launch_trace(const SceneView& sc, const pico_ray* rays, uint64_t n, pico_hit* hits,
                         DeviceStatus* status, bool count, int order, cudaStream_t stream)
{
    cudaError_t e = cudaMemsetAsync(&status->work, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess || n == 0) return e;
    const float4* r = reinterpret_cast<const float4*>(rays);
    return with_variant(order, sc, [&](auto v) {
        constexpr int V = decltype(v)::value;
        // the counting variant (measurement only) always reads the bounds at run time
        return count ? launch_trace_t<true, V | kBounded>(sc, r, n, hits, status, stream)
                     : launch_trace_t<false, V>(sc, r, n, hits, status, stream);
    });
}

}  // namespace pico
