// Status bits the traversal latches in device memory (host and device view).
#pragma once

#include <stdint.h>

namespace pico {
enum TraceStatus : int { kTraceOk = 0, kTraceStackOverflow = 1, kTraceIterLimit = 2 };
// The traversal stack's entries and the bound on one walk's iterations (the
// defaults of pico_gpu_set_traversal_limits).
constexpr int kTraceStack = 96;
constexpr uint32_t kTraceMaxIter = 1u << 24;
}  // namespace pico
