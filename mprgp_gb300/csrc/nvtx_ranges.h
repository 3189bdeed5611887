// NVTX ranges on the host timeline (domain "mprgp"): engine runs per lane,
// synchronous solves, server admission and result read-back.  NVTX v3 is
// header-only; without a profiler attached each call returns at once.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace mprgp {

inline nvtxDomainHandle_t nvtx_domain() {
  static nvtxDomainHandle_t d = nvtxDomainCreateA("mprgp");
  return d;
}

inline nvtxRangeId_t nvtx_start(const char *msg) {
  nvtxEventAttributes_t a = {};
  a.version = NVTX_VERSION;
  a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
  a.messageType = NVTX_MESSAGE_TYPE_ASCII;
  a.message.ascii = msg;
  return nvtxDomainRangeStartEx(nvtx_domain(), &a);
}

inline void nvtx_end(nvtxRangeId_t id) {
  if (id) nvtxDomainRangeEnd(nvtx_domain(), id);
}

// A range over a C++ scope.
struct NvtxScope {
  nvtxRangeId_t id;
  explicit NvtxScope(const char *msg) : id(nvtx_start(msg)) {}
  ~NvtxScope() { nvtx_end(id); }
  NvtxScope(const NvtxScope &) = delete;
  NvtxScope &operator=(const NvtxScope &) = delete;
};

}  // namespace mprgp
