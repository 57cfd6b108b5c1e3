// NVTX ranges around the C-ABI entry points, so a timeline profiler shows
// the set-up phases and the time loop by name (header-only NVTX v3: without
// a profiler attached each range is a no-op).
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace lbm {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace lbm
