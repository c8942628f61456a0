// trace.h -- NVTX ranges around the library's launches and host phases.
//
// The reference gates its trace output behind a command-line flag and
// prefixes each message with the function, time and thread
// (tweakseq/Core/DebuggingInfo.h:51-71, tweakseq/Core/Main.cpp:48-66).  Here
// each launch sequence, kernel launch and planning phase opens a named NVTX
// range in the "tweakseq_gb300" domain, so a profiler shows them on its
// timeline next to the kernels.  NVTX v3 is header-only: without a profiler
// attached a range costs one check of a function pointer.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace tsq {

struct TraceDomain {
  nvtxDomainHandle_t h;
  TraceDomain() : h(nvtxDomainCreateA("tweakseq_gb300")) {}
};

inline nvtxDomainHandle_t trace_domain() {
  static TraceDomain d;
  return d.h;
}

// Opens a range for the life of the object.
class TraceRange {
 public:
  explicit TraceRange(const char *name) {
    nvtxEventAttributes_t a{};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = name;
    nvtxDomainRangePushEx(trace_domain(), &a);
  }
  ~TraceRange() { nvtxDomainRangePop(trace_domain()); }
  TraceRange(const TraceRange &) = delete;
  TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace tsq
