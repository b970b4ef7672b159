// Global area integral that allocates no device memory.
//
// dccm_area_integral_dev reduces through a small device buffer that it
// allocates on every call.  Some callers cannot do that: a model that
// reserves all of the GPU's memory for its own allocator at start-up leaves
// nothing for a library's cudaMalloc, and a component linked into such a
// model (the coupler's diagnostics, for instance) must work inside what the
// model already holds.  This variant keeps its scratch (one partial sum per
// block, plus the final result) in a fixed array that lives in the
// library's device image, so each GPU that loads the library holds it
// until the process exits.
//
// What it does not avoid: like dccm_area_integral_dev it copies the result
// into the caller's host double and synchronises the stream before it
// returns, so it blocks the calling thread until the integral is done.
//
// Limits and sharing:
//   - at most NOALLOC_MAX_PARTIALS blocks of NOALLOC_BLOCK_ELEMS elements,
//     i.e. n <= 2^26 = 67,108,864 elements; larger n is refused with
//     DCCM_ERR_SHAPE;
//   - every call uses the same array, so calls that overlap on the GPU
//     (two streams, two host threads) race and corrupt each other's sums;
//     serialise them;
//   - each call writes every partial slot it reads before reading it, and
//     the final slot before copying it out, so nothing has to be cleared
//     between calls (the array keeps the last call's values).
// The host must pass kernels a device address of the array, which in host
// code the array's name is not: the first call in each CUDA context (per
// device, and again after cudaDeviceReset has replaced a device's primary
// context) looks the address up with cudaGetSymbolAddress, with that
// device current, and keeps it for the calls that follow in that context.
#include <mutex>

#include "common.cuh"
#include "nvtx.cuh"

namespace dccm {
namespace noalloc {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_PER_THREAD = 16;
constexpr int64_t NOALLOC_BLOCK_ELEMS = (int64_t)NOALLOC_THREADS * NOALLOC_PER_THREAD;  // 4096
constexpr int NOALLOC_MAX_PARTIALS = 16384;                                             // 256 KB
constexpr int64_t NOALLOC_MAX_N = NOALLOC_BLOCK_ELEMS * NOALLOC_MAX_PARTIALS;

// Slots 0..NOALLOC_MAX_PARTIALS-1: (sum, compensation) of each block;
// slot NOALLOC_MAX_PARTIALS: the final sum in .x.
static __device__ __align__(256) double2 g_scratch[NOALLOC_MAX_PARTIALS + 1];

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

// Tree reduction of the block's (sum, compensation) pairs in shared memory;
// the result is in ss[0], cs[0] for thread 0.
__device__ __forceinline__ void block_pairs(double s, double c, double (&ss)[NOALLOC_THREADS],
                                            double (&cs)[NOALLOC_THREADS]) {
  ss[threadIdx.x] = s;
  cs[threadIdx.x] = c;
  __syncthreads();
  for (int w = NOALLOC_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double s2, e;
      two_sum(ss[threadIdx.x], ss[threadIdx.x + w], s2, e);
      ss[threadIdx.x] = s2;
      cs[threadIdx.x] = __dadd_rn(__dadd_rn(cs[threadIdx.x], cs[threadIdx.x + w]), e);
    }
    __syncthreads();
  }
}

// Same compensated accumulation as the allocating kernel, but block b owns
// elements [b*4096, (b+1)*4096) so the number of partials follows from n.
__global__ void __launch_bounds__(NOALLOC_THREADS)
area_partial_fixed(const double *__restrict__ f, const double *__restrict__ a, int64_t n,
                   double2 *__restrict__ part) {
  const int64_t base = blockIdx.x * NOALLOC_BLOCK_ELEMS;
  double s = 0.0, c = 0.0;
#pragma unroll 4
  for (int k = 0; k < NOALLOC_PER_THREAD; ++k) {
    const int64_t i = base + (int64_t)k * NOALLOC_THREADS + threadIdx.x;
    if (i < n) {
      const double p = __dmul_rn(f[i], a[i]);
      const double pe = fma(f[i], a[i], -p);
      double e;
      two_sum(s, p, s, e);
      c = __dadd_rn(__dadd_rn(c, e), pe);
    }
  }
  __shared__ double ss[NOALLOC_THREADS], cs[NOALLOC_THREADS];
  block_pairs(s, c, ss, cs);
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(ss[0], cs[0]);
}

// One block: thread t sums partials t, t + 256, ... (compensated), then the
// block's tree gives the total.
__global__ void __launch_bounds__(NOALLOC_THREADS) area_final_fixed(double2 *__restrict__ scratch, int np) {
  double s = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < np; i += NOALLOC_THREADS) {
    double e;
    two_sum(s, scratch[i].x, s, e);
    c = __dadd_rn(__dadd_rn(c, e), scratch[i].y);
  }
  __shared__ double ss[NOALLOC_THREADS], cs[NOALLOC_THREADS];
  block_pairs(s, c, ss, cs);
  if (threadIdx.x == 0) scratch[NOALLOC_MAX_PARTIALS] = make_double2(__dadd_rn(ss[0], cs[0]), 0.0);
}

// Device address of g_scratch in each CUDA context.  The key is the
// context's process-unique id (cuCtxGetId), so a context that replaced an
// earlier one on the same device (after cudaDeviceReset) looks it up again.
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
constexpr int MAX_CONTEXTS = 64;
struct Slot {
  unsigned long long ctx_id;
  double2 *addr;
};
static Slot g_slots[MAX_CONTEXTS];
static int g_nslots = 0;
static std::mutex g_mutex;

static void *driver_fn(const char *name) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return p;
}

static int scratch_address(double2 **out) {
  static CtxGetCurrentFn get_ctx = reinterpret_cast<CtxGetCurrentFn>(driver_fn("cuCtxGetCurrent"));
  static CtxGetIdFn get_id = reinterpret_cast<CtxGetIdFn>(driver_fn("cuCtxGetId"));
  if (!get_ctx || !get_id) return DCCM_ERR_UNSUPPORTED;
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_ctx(&ctx) != 0) return DCCM_ERR_CUDA;
  if (!ctx) {  // no context current on this thread yet: the device's primary one
    int dev = 0;
    DCCM_CUDA(cudaGetDevice(&dev));
    DCCM_CUDA(cudaSetDevice(dev));
    if (get_ctx(&ctx) != 0 || !ctx) return DCCM_ERR_CUDA;
  }
  if (get_id(ctx, &id) != 0) return DCCM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  for (int k = 0; k < g_nslots; ++k)
    if (g_slots[k].ctx_id == id) {
      *out = g_slots[k].addr;
      return DCCM_OK;
    }
  void *p = nullptr;
  DCCM_CUDA(cudaGetSymbolAddress(&p, g_scratch));
  Slot sl = {id, static_cast<double2 *>(p)};
  if (g_nslots < MAX_CONTEXTS) g_slots[g_nslots++] = sl;
  else g_slots[id % MAX_CONTEXTS] = sl;  // more contexts than slots: reuse one
  *out = sl.addr;
  return DCCM_OK;
}

}  // namespace noalloc
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_area_integral_noalloc_dev(const double *f, const double *area, int64_t n,
                                              double *result, void *stream) {
  DCCM_NVTX_FUNC();
  if (!f || !area || !result || n < 0) return DCCM_ERR_INVALID_ARG;
  if (n > noalloc::NOALLOC_MAX_N) return DCCM_ERR_SHAPE;
  double2 *scratch = nullptr;
  DCCM_TRY(noalloc::scratch_address(&scratch));
  cudaStream_t s = as_stream(stream);
  int np = (int)((n + noalloc::NOALLOC_BLOCK_ELEMS - 1) / noalloc::NOALLOC_BLOCK_ELEMS);
  if (np > 0) {
    noalloc::area_partial_fixed<<<np, noalloc::NOALLOC_THREADS, 0, s>>>(f, area, n, scratch);
    DCCM_LAUNCH_CHECK();
  }
  noalloc::area_final_fixed<<<1, noalloc::NOALLOC_THREADS, 0, s>>>(scratch, np);
  DCCM_LAUNCH_CHECK();
  DCCM_CUDA(cudaMemcpyAsync(result, &scratch[noalloc::NOALLOC_MAX_PARTIALS].x, sizeof(double),
                            cudaMemcpyDeviceToHost, s));
  DCCM_CUDA(cudaStreamSynchronize(s));
  return DCCM_OK;
}
