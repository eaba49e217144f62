// wt_nvtx.h — one NVTX range per C-ABI call that enqueues GPU work, named
// after the entry point, so a profiler's timeline groups each call's
// kernels.  NVTX 3 is header-only: without a tool attached a range costs a
// few nanoseconds.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace wt {
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace wt

#define WT_NVTX_RANGE(name) ::wt::NvtxRange wt_nvtx_range_(name)
