// Closest-hit kernel for ray batches (UpperLevelBVH::get_closest_intersection
// over many rays, Core/UpperLevelBVH.cpp:12-20).
//
// Persistent: the grid is a whole number of CTAs per SM and every warp pulls
// 32 rays at a time from a global counter, so long rays do not leave SMs idle
// at the tail of the batch.  Rays are 32 B (two 16-byte loads), hits 20 B.
#include "kernels.h"
#include "traverse.cuh"

namespace pico {

constexpr int kTraceThreads = 128;

__device__ __forceinline__ void write_hit(const SceneView& sc, const TraceHit& h, int s, pico_hit* out)
{
    pico_hit r;
    if (h.rank != kNoHit && s == kTraceOk) {
        r.inst = sc.insts[h.rank].inst_id;
        r.prim = sc.tris[h.tri].prim;
        r.t = h.t; r.u = h.u; r.v = h.v;
    } else {
        r.inst = kNoHit; r.prim = kNoHit;
        r.t = __int_as_float(0x7f800000); r.u = 0.0f; r.v = 0.0f;
    }
    *out = r;
}

// Persistent closest-hit kernel.  Each lane owns one ray; when a quarter of a
// warp's lanes have finished, the warp refills them from the ray pool with one
// atomic, so lanes are not held idle by the longest ray of a 32-ray batch.
template <bool kCount, int kOrder>
__global__ void __launch_bounds__(kTraceThreads) trace_kernel(SceneView sc, const float4* __restrict__ rays,
                                                              uint64_t n, pico_hit* __restrict__ hits,
                                                              DeviceStatus* status)
{
    constexpr unsigned kFull = 0xffffffffu;
    TraceCounters cnt{0, 0, 0};
    const unsigned lane = threadIdx.x & 31u;
    Traversal<kCount, kOrder> tr;
    StackEntry stack[kTraceStack];
    unsigned long long rid = 0;
    uint32_t steps = 0;
    bool active = false, exhausted = false;
    for (;;) {
        if (!exhausted) {
            const unsigned idle = __ballot_sync(kFull, !active);
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == (unsigned)leader) base = atomicAdd(&status->work, (unsigned long long)__popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (base + __popc(idle) >= n) exhausted = true;
            if (!active) {
                rid = base + __popc(idle & ((1u << lane) - 1u));
                if (rid < n) {
                    tr.start(sc, __ldg(rays + 2 * rid), __ldg(rays + 2 * rid + 1));
                    active = true;
                    steps = 0;
                }
            }
        }
        if (!__any_sync(kFull, active)) break;
        const int refill_at = exhausted ? 32 : 8;
        for (;;) {
            if (active) {
                int s = tr.step(sc, stack, &cnt);
                if (s == kTraceOk && ++steps >= kTraceMaxIter) s = kTraceIterLimit;
                if (s != kTraceOk) {
                    if (s != kTraceDone) atomicOr(&status->trace_error, s);
                    write_hit(sc, tr.best, s == kTraceDone ? kTraceOk : s, hits + rid);
                    active = false;
                }
            }
            if (__popc(__ballot_sync(kFull, !active)) >= refill_at) break;
        }
    }
    if (kCount) {
        // one atomic per warp per counter
        for (int off = 16; off > 0; off >>= 1) {
            cnt.nodes += __shfl_down_sync(kFull, cnt.nodes, off);
            cnt.tris += __shfl_down_sync(kFull, cnt.tris, off);
            cnt.insts += __shfl_down_sync(kFull, cnt.insts, off);
        }
        if (lane == 0) {
            atomicAdd(&status->counters[0], cnt.nodes);
            atomicAdd(&status->counters[1], cnt.tris);
            atomicAdd(&status->counters[2], cnt.insts);
        }
    }
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
    if (order == kReferenceOrder)
        return count ? launch_trace_t<true, kReferenceOrder>(sc, r, n, hits, status, stream)
                     : launch_trace_t<false, kReferenceOrder>(sc, r, n, hits, status, stream);
    return count ? launch_trace_t<true, kNearFirst>(sc, r, n, hits, status, stream)
                 : launch_trace_t<false, kNearFirst>(sc, r, n, hits, status, stream);
}

}  // namespace pico
