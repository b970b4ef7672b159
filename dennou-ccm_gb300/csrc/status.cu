// Status strings, version and per-thread CUDA error record.
#include "common.cuh"

namespace dccm {
static thread_local int g_last_cuda_error = 0;
void set_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }

Tunables &tunables() {
  static Tunables t;
  return t;
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

int greatest_priority() {
  static int cached = 1;  // 1: not read yet (priorities are 0 or negative)
  if (cached == 1) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) greatest = 0;
    cached = greatest;
  }
  return cached;
}
}  // namespace dccm

extern "C" {

const char *dccm_status_string(int status) {
  switch (status) {
    case DCCM_OK: return "ok";
    case DCCM_ERR_INVALID_ARG: return "invalid argument";
    case DCCM_ERR_SHAPE: return "array shape inconsistent with the plan";
    case DCCM_ERR_CUDA: return "CUDA runtime error (see dccm_last_cuda_error)";
    case DCCM_ERR_INDEX_RANGE: return "table index outside the grid";
    case DCCM_ERR_SEARCH: return "overlap search failed";
    case DCCM_ERR_IO: return "table file I/O error";
    case DCCM_ERR_NOMEM: return "allocation failed";
    case DCCM_ERR_TIMEOUT: return "bounded device wait timed out";
    case DCCM_ERR_UNSUPPORTED: return "unsupported size or mode";
    default: return "unknown status";
  }
}

int dccm_abi_version(void) { return DCCM_ABI_VERSION; }

int dccm_last_cuda_error(void) { return dccm::g_last_cuda_error; }

}  // extern "C"
