// NVTX ranges (header-only NVTX 3) marking the library's entry points and the render pass's
// wavefront stages on the host timeline, in the "PLT GB300" domain.  A range spans the enqueue of its
// stage's launches; with the render's frame graph the per-stage ranges appear when the graph is
// recorded (and on every frame under PLT_OPTION_NO_GRAPH), so profilers can filter kernels by stage
// (e.g. ncu --nvtx --nvtx-include "PLT GB300@pt_solve/").  Without a profiler attached the calls
// return at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace plt {

inline nvtxDomainHandle_t nvtxDomain() {
    static const nvtxDomainHandle_t d = nvtxDomainCreateA("PLT GB300");
    return d;
}

// Pushes a range on construction and pops it on destruction.
class NvtxRange {
public:
    explicit NvtxRange(const char* name) {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(nvtxDomain(), &a);
    }
    ~NvtxRange() { nvtxDomainRangePop(nvtxDomain()); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace plt
