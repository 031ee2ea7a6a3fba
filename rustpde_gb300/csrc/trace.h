// trace.h -- NVTX ranges around the library's host-side stages: each entry
// point that enqueues a step, the batch's copy/step/copy per group, the
// serving loop's rebuilds and chunks, and every stage of the profiling entry
// points (named by kernel).  Nsight Systems and `ncu --nvtx` show them; without
// a tool attached a range costs a call through an empty function pointer.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace rbc {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace rbc
