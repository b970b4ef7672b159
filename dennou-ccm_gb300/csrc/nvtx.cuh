// NVTX ranges of the library's host entry points and of the stages of a
// timed step (internal header).  The reference marks the same regions with
// ProfUtil_RapStart / ProfUtil_RapEnd (atm/dcpam_main_mod.f90:1167, 2167,
// 2203).  NVTX v3 is header-only: with no profiler attached a push or pop
// is a call through a null-checked pointer.  Ranges are host-side, so a
// replayed CUDA graph shows as the one range of the call that launches it.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace dccm {

struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace dccm

// One range over the rest of the enclosing scope, named after the function.
#define DCCM_NVTX_FUNC() ::dccm::NvtxRange dccm_nvtx_scope_(__func__)
