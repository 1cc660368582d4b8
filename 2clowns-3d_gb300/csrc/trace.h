// NVTX ranges around the library's entry points and the phases of a solve, so
// that Nsight Systems and Nsight Compute (--nvtx) show where a run spends its
// time.  NVTX v3 is header-only: without a tool attached, each push and pop is
// one call through an unset entry of its function table.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace clowns {

struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace clowns
