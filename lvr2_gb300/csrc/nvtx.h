// nvtx.h -- NVTX ranges around the library's stages (visible in Nsight
// Systems / Compute timelines; no cost without a tool attached).
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace lvrgb {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace lvrgb
