// pa_trace.h -- NVTX ranges (header-only NVTX v3 of the CUDA toolkit) around
// the library's entry points and pipeline stages, so that Nsight tools and
// `ncu --nvtx` can attribute kernels to them.  Without an attached tool a
// range costs one call into an empty stub.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace pa {
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
}  // namespace pa
