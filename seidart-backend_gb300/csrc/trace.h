// trace.h -- NVTX ranges around the C ABI's long-running entry points
// (set-up, steps, synchronisation, autotuning, gradients, file runs), so a
// profiler's timeline or an NVTX filter (ncu --nvtx) shows them by name.
// NVTX 3 is header-only: with no tool attached a range costs two calls that
// return at once.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace seidart_trace {

struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

}  // namespace seidart_trace
