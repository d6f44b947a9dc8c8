// NVTX ranges around the library's host-side phases (mesh generation and
// upload, state copies, steps, batch steps, server ticks). They show in a
// profiler's timeline and let ncu select kernels by range (--nvtx
// --nvtx-include "ma_solver_step/"). NVTX v3 is header-only: with no tool
// attached a range costs a null-pointer check.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace miniaero {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace miniaero
