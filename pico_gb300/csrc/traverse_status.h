// Status bits the traversal latches in device memory (host and device view).
#pragma once

namespace pico {
enum TraceStatus : int { kTraceOk = 0, kTraceStackOverflow = 1, kTraceIterLimit = 2 };
}  // namespace pico
