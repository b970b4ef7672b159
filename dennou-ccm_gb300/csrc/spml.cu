// The SHT in SPML's real spectral layout: the drop-in for a DCPAM caller.
//
// DCPAM's dynamics (atm/dcpam_main_mod.f90:2173-2180, through libdcpam5)
// and the coupler's tools (tool/gmapgen/gmapgen_main.f90:262-305) call SPML,
// whose spectral arrays are real: wa(l, k) holds the (N+1)^2 coefficients
// of field-level k at l = l_nm(n, m) = n(n+1) + m + 1 (1-based), m = -n..n,
// with Re s_n^m at m >= 0 and Im s_n^|m| at m < 0 (SPML's l_nm / nm_l, as
// its documentation publishes them; SPML itself is external and not
// vendored, so this restatement is unpinned against its code).  SPML's
// expansion is f = sum_n sum_{m=-n..n} s_n^m Pbar_n^m(mu) e^{i m lon},
// s_n^-m = conj(s_n^m), with Pbar of unit mean square over the sphere and
// no Condon-Shortley phase: the same as this library's, so the two layouts
// differ by a permutation alone (no scale, no sign).  Grids are the same
// (0:im-1, 1:jm, k) arrays, latitudes south to north.
//
// The entry points permute on the device (one pass each way, gathers from
// L2-resident tables) and call the plan's transforms; the plan keeps a
// spectral buffer of max_batch field-levels for the native layout, set up by
// the first call that needs it.
#include <string.h>

#include <new>
#include <vector>

#include "nvtx.cuh"
#include "sht_plan.cuh"

struct dccm_sht_plan {
  dccm::sht::Plan P;
};

namespace dccm {
namespace sht {

__global__ void __launch_bounds__(256)
wa_to_spec_kernel(const double *__restrict__ wa, long long L, const int2 *__restrict__ pos, long long ncoef,
                  long long total, double2 *__restrict__ spec) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / ncoef, k = t - b * ncoef;
    const int2 p = __ldg(pos + k);
    const double *w = wa + b * L;
    spec[t] = make_double2(__ldg(w + p.x), p.y >= 0 ? __ldg(w + p.y) : 0.0);
  }
}

__global__ void __launch_bounds__(256)
spec_to_wa_kernel(const double2 *__restrict__ spec, long long ncoef, const int *__restrict__ src, long long L,
                  long long total, double *__restrict__ wa) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / L, l = t - b * L;
    const int s = __ldg(src + l);
    const double *sp = reinterpret_cast<const double *>(spec + b * ncoef);
    wa[t] = __ldg(sp + s);
  }
}

// 0-based position of (n, m) in SPML's layout, m = -n..n.
static inline long long wa_l(int n, int m) { return (long long)n * (n + 1) + m; }

static int wa_setup(Plan &P) {
  if (P.d_wa_pos) return DCCM_OK;
  const int N = P.N;
  const long long L = (long long)(N + 1) * (N + 1);
  std::vector<int2> pos((size_t)P.ncoef);
  std::vector<int> src((size_t)L);
  for (int m = 0; m <= N; ++m)
    for (int n = m; n <= N; ++n) {
      const long long k = idx_mn(N, m, n);
      pos[(size_t)k] = make_int2((int)wa_l(n, m), m > 0 ? (int)wa_l(n, -m) : -1);
      src[(size_t)wa_l(n, m)] = (int)(2 * k);
      if (m > 0) src[(size_t)wa_l(n, -m)] = (int)(2 * k + 1);
    }
  int2 *dp = nullptr;
  int *ds = nullptr;
  DCCM_CUDA(cudaMalloc(&dp, pos.size() * sizeof(int2)));
  cudaError_t e = cudaMalloc(&ds, src.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dp, pos.data(), pos.size() * sizeof(int2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ds, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dp);
    if (ds) cudaFree(ds);
    set_cuda_error(e);
    return DCCM_ERR_CUDA;
  }
  P.d_wa_pos = dp;
  P.d_wa_src = ds;
  return P.wa_spec.ensure((size_t)P.max_batch * P.ncoef * sizeof(double2));
}

static unsigned grid_for(long long total) {
  long long g = (total + 255) / 256;
  const long long cap = 8LL * sm_count();
  return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

int spec_from_wa(Plan &P, const double *wa, double *spec, int batch, cudaStream_t s) {
  DCCM_TRY(wa_setup(P));
  if (batch <= 0) return DCCM_OK;
  const long long L = (long long)(P.N + 1) * (P.N + 1), total = (long long)batch * P.ncoef;
  wa_to_spec_kernel<<<grid_for(total), 256, 0, s>>>(wa, L, P.d_wa_pos, P.ncoef, total,
                                                      reinterpret_cast<double2 *>(spec));
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int wa_from_spec(Plan &P, const double *spec, double *wa, int batch, cudaStream_t s) {
  DCCM_TRY(wa_setup(P));
  if (batch <= 0) return DCCM_OK;
  const long long L = (long long)(P.N + 1) * (P.N + 1), total = (long long)batch * L;
  spec_to_wa_kernel<<<grid_for(total), 256, 0, s>>>(reinterpret_cast<const double2 *>(spec), P.ncoef,
                                                      P.d_wa_src, L, total, wa);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int xya_wa(Plan &P, const double *wa, double *xya, int batch, cudaStream_t s) {
  DCCM_TRY(wa_setup(P));
  double *spec = static_cast<double *>(P.wa_spec.ptr);
  DCCM_TRY(spec_from_wa(P, wa, spec, batch, s));
  return inverse(P, spec, xya, batch, s);
}

int wa_xya(Plan &P, const double *xya, double *wa, int batch, cudaStream_t s) {
  DCCM_TRY(wa_setup(P));
  double *spec = static_cast<double *>(P.wa_spec.ptr);
  DCCM_TRY(forward(P, xya, spec, batch, s));
  return wa_from_spec(P, spec, wa, batch, s);
}

}  // namespace sht
}  // namespace dccm

using namespace dccm;

static int wa_check(dccm_sht_plan *p, const void *a, const void *b, int batch) {
  if (!p || batch < 0) return DCCM_ERR_INVALID_ARG;
  if (batch > p->P.max_batch) return DCCM_ERR_SHAPE;
  if (batch > 0 && (!a || !b)) return DCCM_ERR_INVALID_ARG;
  return DCCM_OK;
}

extern "C" int dccm_sht_spec_from_wa_dev(dccm_sht_plan *p, const double *wa, double *spec, int batch,
                                         void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, wa, spec, batch));
  return sht::spec_from_wa(p->P, wa, spec, batch, as_stream(stream));
}

extern "C" int dccm_sht_wa_from_spec_dev(dccm_sht_plan *p, const double *spec, double *wa, int batch,
                                         void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, spec, wa, batch));
  return sht::wa_from_spec(p->P, spec, wa, batch, as_stream(stream));
}

extern "C" int dccm_sht_xya_wa_dev(dccm_sht_plan *p, const double *wa, double *xya, int batch, void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, wa, xya, batch));
  return sht::xya_wa(p->P, wa, xya, batch, as_stream(stream));
}

extern "C" int dccm_sht_wa_xya_dev(dccm_sht_plan *p, const double *xya, double *wa, int batch, void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, xya, wa, batch));
  return sht::wa_xya(p->P, xya, wa, batch, as_stream(stream));
}

// Host arrays: copy in, permute and transform, copy out, check the device
// error flag of the bounded waits (as the native host entry points do).
static int wa_host(dccm_sht_plan *p, const double *in, size_t in_n, double *out, size_t out_n, int batch,
                   bool inv) {
  sht::Plan &P = p->P;
  if (!P.stream) DCCM_CUDA(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
  DCCM_TRY(P.stage.ensure((in_n + out_n) * sizeof(double)));
  double *din = (double *)P.stage.ptr, *dout = din + in_n;
  DCCM_CUDA(cudaMemcpyAsync(din, in, in_n * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  if (inv) DCCM_TRY(sht::xya_wa(P, din, dout, batch, P.stream));
  else DCCM_TRY(sht::wa_xya(P, din, dout, batch, P.stream));
  DCCM_CUDA(cudaMemcpyAsync(out, dout, out_n * sizeof(double), cudaMemcpyDeviceToHost, P.stream));
  DCCM_CUDA(cudaStreamSynchronize(P.stream));
  int e = 0;
  DCCM_CUDA(cudaMemcpy(&e, P.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(P.d_err, 0, sizeof(int));
    return DCCM_ERR_TIMEOUT;
  }
  return DCCM_OK;
}

extern "C" int dccm_sht_xya_wa(dccm_sht_plan *p, const double *wa, double *xya, int batch) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, wa, xya, batch));
  if (batch == 0) return DCCM_OK;
  const size_t nw = (size_t)batch * (p->P.N + 1) * (p->P.N + 1), ng = (size_t)batch * p->P.J * p->P.I;
  return wa_host(p, wa, nw, xya, ng, batch, true);
}

extern "C" int dccm_sht_wa_xya(dccm_sht_plan *p, const double *xya, double *wa, int batch) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(wa_check(p, xya, wa, batch));
  if (batch == 0) return DCCM_OK;
  const size_t nw = (size_t)batch * (p->P.N + 1) * (p->P.N + 1), ng = (size_t)batch * p->P.J * p->P.I;
  return wa_host(p, xya, ng, wa, nw, batch, false);
}
