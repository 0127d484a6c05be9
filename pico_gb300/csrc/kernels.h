// Host-callable launchers for the device kernels (defined in the .cu files).
#pragma once

#include "layout.h"
#include "pico_gpu.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pico {

// Device-side status words shared by all kernels of a context.
struct DeviceStatus {
    int trace_error;                 // TraceStatus bits
    int pad[3];
    unsigned long long work;         // persistent-kernel work counter
    unsigned long long counters[4];  // nodes, triangles, instances, spare
    unsigned long long rays[4];      // render tallies: camera, bounce, shadow rays traced; spare
};

int sm_count();
// Blocks of `threads` threads of `kernel` resident on one SM at once (at least 1), cached per
// kernel and block size.
int resident_blocks(const void* kernel, int threads);

cudaError_t launch_trace(const SceneView& sc, const pico_ray* rays, uint64_t n, pico_hit* hits,
                         DeviceStatus* status, bool count, int order, cudaStream_t stream);

}  // namespace pico
