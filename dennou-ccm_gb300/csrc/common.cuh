// Shared helpers of the dccm_gb300 library (internal header).
#pragma once
#include <cuda_runtime.h>

#include <utility>
#include <stdint.h>
#include <stdio.h>

#include "dccm_gb300.h"

namespace dccm {

// Records the CUDA error of the calling thread for dccm_last_cuda_error().
void set_cuda_error(cudaError_t e);

// Evaluate a CUDA runtime call; on failure record it and return DCCM_ERR_CUDA.
#define DCCM_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) {                              \
      ::dccm::set_cuda_error(e_);                         \
      return DCCM_ERR_CUDA;                               \
    }                                                     \
  } while (0)

// Check the launch status of the preceding kernel launch.
#define DCCM_LAUNCH_CHECK() DCCM_CUDA(cudaGetLastError())

// Launch-shape knobs read by the kernel launchers (0 = the launcher's own
// default).  dccm_step_autotune chooses them per step by timing candidates;
// dccm_tune_set / dccm_tune_get expose them.
struct Tunables {
  int tc_ctas = 0;        // persistent CTAs of the tensor-core Legendre kernel (at most one wave)
  int tc_shape = 0;       // tensor-core Legendre kernel: 0 wide, 1 narrow where the table allows (2 CTAs an SM)
  int fft_bb = 0;         // warps per FFT CTA (4, 8, 16)
  int fft_rpw = 0;        // row pairs per FFT warp where a row pair takes one warp (1, 2; 0: 1)
  int flux_threads = 0;   // threads per CTA of the bulk-flux kernel
  int flux_ctas = 0;      // CTA cap of the bulk-flux kernel's grid-stride loop (0: 16 per SM)
  int remap_threads = 0;  // threads per CTA of the remap kernel
  int remap_fc = 0;       // fields per thread of the remap kernel (1, 2, 3, 4, 6; 0: 3, or all below 6)
  int serial = 0;         // 1: launch_pdl makes ordinary launches
  int prio = 0;           // 1: the transform chain's launches (launch_pdl), 2: the surface branch's
                          // (launch_surface) at the device's greatest priority; the step graphs
                          // then run their nodes at their own priorities
  int upload_order = 0;   // dccm_step_run_host: 1 transforms' inputs first, 2 surface inputs first
  int host_path = 0;      // dccm_step_run_host: 1 + mask of the copy groups moved through the host mapping (0: 1)
  int wait_limit_ms = 0;  // limit of the tensor-core kernel's bounded waits (0: 1000 ms)
  int tc_withhold_loads = 0;  // 1: the tensor-core kernel's load thread issues no copies, so its
                              // waits expire (tests the timeout path; nothing is left in flight)
};
Tunables &tunables();

// Programmatic dependent launch between the kernels of the transform chain:
// a kernel launched with launch_pdl may start while the previous kernel in
// its stream is still running (its prologue overlaps that kernel's tail).
// It must execute pdl_wait() before it reads anything the previous kernel
// writes or writes anything the previous kernel reads; pdl_trigger() lets
// the next kernel start.  Both are no-ops for an ordinary launch (the
// "serial" knob), which the step autotuner picks where early-resident CTAs
// of the chain would keep a concurrent branch of the step off the SMs.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// The device's greatest (most urgent) stream priority (cached).
int greatest_priority();

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  unsigned n = 0;
  if (!tunables().serial) {
    attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[n++].val.programmaticStreamSerializationAllowed = 1;
  }
  if (tunables().prio == 1) {
    attr[n].id = cudaLaunchAttributePriority;
    attr[n++].val.priority = greatest_priority();
  }
  cfg.attrs = attr;
  cfg.numAttrs = n;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Launch of a surface-branch kernel (remap, flux): at the device's greatest
// priority with the "prio" knob at 2, else an ordinary launch.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_surface(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                  Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = greatest_priority();
  cfg.attrs = attr;
  cfg.numAttrs = tunables().prio == 2 ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#define DCCM_TRY(expr)           \
  do {                           \
    int st_ = (expr);            \
    if (st_ != DCCM_OK) return st_; \
  } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();

// Device buffer that grows on demand (never shrinks); used for the host
// entry points' staging copies.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t n) {
    if (n <= bytes) return DCCM_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
      set_cuda_error(e);
      return DCCM_ERR_NOMEM;
    }
    bytes = n;
    return DCCM_OK;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

}  // namespace dccm
