// Spherical-harmonic transform plans and their C ABI.
//
// Replaces the SPML transforms the atmosphere dynamics call through
// libdcpam5 (atm/dcpam_main_mod.f90:2173-2180) and SPML's w_Initial and
// grid axes (tool/gmapgen/gmapgen_main.f90:262-305).  Plan creation runs the
// FP64 set-up on the GPU: Gauss-Legendre nodes and weights by Newton
// iteration and the normalised associated Legendre functions by the
// three-term recurrence in n; for the mixed-precision plan the table is then
// split into BF16 x 3 tensor-core tiles.
//
// Transform paths (precision chosen at plan creation):
//   DCCM_SHT_FP64   Legendre on the FP64 CUDA cores, FP64 FFT;
//   DCCM_SHT_MIXED  Legendre on tcgen05 tensor cores (BF16 x 3, FP32
//                   accumulation), FP32 FFT; spectra and grids stay FP64;
//   DCCM_SHT_MIXED_FP16  the same with FP16 hi + lo operands (3 products
//                   instead of 6): tables scaled by a power of two per
//                   zonal wavenumber m, spectra and Fourier coefficients
//                   per field-level, so that both fit FP16's range.
#include <math.h>
#include <string.h>

#include <new>

#include "sht_plan.cuh"
#include "nvtx.cuh"

struct dccm_sht_plan {
  dccm::sht::Plan P;
};

namespace dccm {
namespace sht {

// Newton iteration for the positive roots of P_J (one thread per root).
__global__ void gauss_newton_kernel(int J, double *mu, double *w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= J / 2) return;
  const double PI = 3.141592653589793238462643383279502884;
  double x = cos(PI * (k + 0.75) / (J + 0.5));
  double dp = 0.0;
  bool last = false;
  for (int it = 0; it < 100; ++it) {
    double p0 = 1.0, p1 = x;
    for (int l = 2; l <= J; ++l) {
      const double p2 = ((2.0 * l - 1.0) * x * p1 - (l - 1.0) * p0) / l;
      p0 = p1;
      p1 = p2;
    }
    dp = J * (x * p1 - p0) / (x * x - 1.0);
    const double dx = p1 / dp;
    x -= dx;
    if (last) break;  // one more step after |dx| <= 1e-15 |x| (quadratic convergence)
    if (fabs(dx) <= 1e-15 * fabs(x)) last = true;
  }
  double p0 = 1.0, p1 = x;
  for (int l = 2; l <= J; ++l) {
    const double p2 = ((2.0 * l - 1.0) * x * p1 - (l - 1.0) * p0) / l;
    p0 = p1;
    p1 = p2;
  }
  dp = J * (x * p1 - p0) / (x * x - 1.0);
  mu[J - 1 - k] = x;
  mu[k] = -x;
  const double wk = 2.0 / ((1.0 - x * x) * dp * dp);
  w[J - 1 - k] = wk;
  w[k] = wk;
}

// Pbar_n^m(mu_{Jh+jj}) for n = m..N; one thread per (m, jj).  Sectoral
// values underflow to zero near the poles at high m (harmless: the whole
// column is then below 1e-300).
__global__ void pnm_kernel(int N, int Jh, const double *__restrict__ mu, double *__restrict__ p) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)(N + 1) * Jh) return;
  const int m = (int)(t / Jh), jj = (int)(t % Jh);
  const double x = mu[Jh + jj];
  const double sx = sqrt((1.0 - x) * (1.0 + x));
  double pmm = 1.0;
  for (int k = 1; k <= m; ++k) pmm = pmm * sqrt((2.0 * k + 1.0) / (2.0 * k)) * sx;
  p[idx_mn(N, m, m) * Jh + jj] = pmm;
  if (m + 1 > N) return;
  double pa = pmm, pb = sqrt(2.0 * m + 3.0) * x * pmm;
  p[idx_mn(N, m, m + 1) * Jh + jj] = pb;
  for (int n = m + 2; n <= N; ++n) {
    const double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
    const double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
    const double pc = a * (x * pb - b * pa);
    p[idx_mn(N, m, n) * Jh + jj] = pc;
    pa = pb;
    pb = pc;
  }
}

static void destroy(Plan &P) {
  void *ptrs[] = {P.d_mu,      P.d_w,        P.d_pnm,       P.d_tw64,  P.d_tw32,  P.d_twl32,
                  P.tinv.d,    P.tfwd.d,     P.tinv.d_mi,   P.tfwd.d_mi, P.tinv.d_items,
                  P.tfwd.d_items, P.d_work,  P.d_err,       P.d_apack, P.d_punits, P.d_cexp,
                  P.d_wa_pos, P.d_wa_src};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  P.stage.release();
  P.wa_spec.release();
  if (P.stream) cudaStreamDestroy(P.stream);
}

static int create(Plan &P, int N, int I, int J, int precision, int max_batch) {
  P.N = N;
  P.I = I;
  P.J = J;
  P.Jh = J / 2;
  P.precision = precision;
  P.nsplit = precision == DCCM_SHT_MIXED_FP16 ? 2 : 3;
  P.max_batch = max_batch;
  P.ncoef = (int64_t)(N + 1) * (N + 2) / 2;
  if (!fft_length_supported(I)) return DCCM_ERR_UNSUPPORTED;
  DCCM_CUDA(cudaMalloc(&P.d_mu, J * sizeof(double)));
  DCCM_CUDA(cudaMalloc(&P.d_w, J * sizeof(double)));
  DCCM_CUDA(cudaMalloc(&P.d_pnm, (size_t)P.ncoef * P.Jh * sizeof(double)));
  DCCM_CUDA(cudaMalloc(&P.d_err, sizeof(int)));
  DCCM_CUDA(cudaMemset(P.d_err, 0, sizeof(int)));
  gauss_newton_kernel<<<(P.Jh + 127) / 128, 128>>>(J, P.d_mu, P.d_w);
  DCCM_LAUNCH_CHECK();
  const long long nt = (long long)(N + 1) * P.Jh;
  pnm_kernel<<<(unsigned)((nt + 127) / 128), 128>>>(N, P.Jh, P.d_mu, P.d_pnm);
  DCCM_LAUNCH_CHECK();
  P.mu.resize(J);
  P.w.resize(J);
  DCCM_CUDA(cudaMemcpy(P.mu.data(), P.d_mu, J * sizeof(double), cudaMemcpyDeviceToHost));
  DCCM_CUDA(cudaMemcpy(P.w.data(), P.d_w, J * sizeof(double), cudaMemcpyDeviceToHost));
  // FFT twiddles e^{-2 pi i t / I} in FP64 on the host.
  // and, for the FP32 warp transform, the per-lane table e^{-2 pi i l k / I}
  // at [k][l] (l < 32, k < I/32).
  std::vector<double2> tw64(I);
  std::vector<float2> tw32(I), twl32(I);
  const double PI = acos(-1.0);
  for (int t = 0; t < I; ++t) {
    const double ang = 2.0 * PI * (double)t / (double)I;
    tw64[t] = make_double2(cos(ang), -sin(ang));
    tw32[t] = make_float2((float)tw64[t].x, (float)tw64[t].y);
    const int k = t / 32, l = t % 32;
    const double al = 2.0 * PI * (double)(l * k) / (double)I;
    twl32[t] = make_float2((float)cos(al), (float)-sin(al));
  }
  DCCM_CUDA(cudaMalloc(&P.d_tw64, I * sizeof(double2)));
  DCCM_CUDA(cudaMalloc(&P.d_tw32, I * sizeof(float2)));
  DCCM_CUDA(cudaMalloc(&P.d_twl32, I * sizeof(float2)));
  DCCM_CUDA(cudaMemcpy(P.d_tw64, tw64.data(), I * sizeof(double2), cudaMemcpyHostToDevice));
  DCCM_CUDA(cudaMemcpy(P.d_tw32, tw32.data(), I * sizeof(float2), cudaMemcpyHostToDevice));
  DCCM_CUDA(cudaMemcpy(P.d_twl32, twl32.data(), I * sizeof(float2), cudaMemcpyHostToDevice));
  if (precision != DCCM_SHT_FP64) {
    // F (FP32, [m][j][2 max_batch]) and G3 (three BF16 or two FP16 planes,
    // rows of C2Bp) share the Fourier buffer.
    const size_t c2bp = (size_t)(2 * max_batch + 7) / 8 * 8;
    const size_t f_bytes = (size_t)(N + 1) * J * 2 * (size_t)max_batch * sizeof(float);
    const size_t g3_bytes = 3 * (size_t)(N + 1) * J * c2bp * sizeof(uint16_t);
    P.work_bytes = f_bytes > g3_bytes ? f_bytes : g3_bytes;
  } else {
    P.work_bytes = (size_t)(N + 1) * J * 2 * (size_t)max_batch * sizeof(double);
  }
  DCCM_CUDA(cudaMalloc(&P.d_work, P.work_bytes));
  if (precision == DCCM_SHT_MIXED_FP16) DCCM_CUDA(cudaMalloc(&P.d_cexp, 2 * (size_t)max_batch * sizeof(int)));
  if (precision != DCCM_SHT_FP64) DCCM_TRY(build_tiles(P));
  DCCM_CUDA(cudaDeviceSynchronize());
  return DCCM_OK;
}

int inverse(Plan &P, const double *spec, double *grid, int batch, cudaStream_t s) {
  if (P.precision != DCCM_SHT_FP64) {
    DCCM_TRY(legendre_inv_tc(P, batch, spec, (float *)P.d_work, s));
    return fft_inverse(P, batch, true, P.d_work, grid, s);
  }
  DCCM_TRY(legendre_inv_f64(P, batch, spec, (double *)P.d_work, s));
  return fft_inverse(P, batch, false, P.d_work, grid, s);
}

int forward(Plan &P, const double *grid, double *spec, int batch, cudaStream_t s) {
  if (P.precision != DCCM_SHT_FP64) {
    DCCM_TRY(fft_forward(P, batch, true, grid, P.d_work, s));
    return legendre_fwd_tc(P, batch, P.d_work, spec, s);
  }
  DCCM_TRY(fft_forward(P, batch, false, grid, P.d_work, s));
  return legendre_fwd_f64(P, batch, (const double *)P.d_work, spec, s);
}

}  // namespace sht
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_sht_plan_create(int nmax, int imax, int jmax, int precision, int max_batch,
                                    dccm_sht_plan **plan) {
  DCCM_NVTX_FUNC();
  if (!plan) return DCCM_ERR_INVALID_ARG;
  *plan = nullptr;
  if (precision != DCCM_SHT_FP64 && precision != DCCM_SHT_MIXED && precision != DCCM_SHT_MIXED_FP16)
    return DCCM_ERR_INVALID_ARG;
  if (nmax < 1 || imax < 1 || jmax < 2 || max_batch < 1) return DCCM_ERR_INVALID_ARG;
  if (jmax % 2 != 0 || jmax < nmax + 1 || imax <= 2 * nmax) return DCCM_ERR_UNSUPPORTED;
  if (precision != DCCM_SHT_FP64 && (jmax / 2) % 16 != 0) return DCCM_ERR_UNSUPPORTED;
  dccm_sht_plan *p = new (std::nothrow) dccm_sht_plan();
  if (!p) return DCCM_ERR_NOMEM;
  int st = sht::create(p->P, nmax, imax, jmax, precision, max_batch);
  if (st != DCCM_OK) {
    sht::destroy(p->P);
    delete p;
    return st;
  }
  *plan = p;
  return DCCM_OK;
}

extern "C" int dccm_sht_plan_destroy(dccm_sht_plan *p) {
  DCCM_NVTX_FUNC();
  if (!p) return DCCM_OK;
  sht::destroy(p->P);
  delete p;
  return DCCM_OK;
}

extern "C" int dccm_sht_axes(const dccm_sht_plan *p, double *x_Lon, double *y_Lat, double *x_Lon_Weight,
                             double *y_Lat_Weight) {
  if (!p) return DCCM_ERR_INVALID_ARG;
  const sht::Plan &P = p->P;
  const double PI = acos(-1.0);
  for (int i = 0; i < P.I; ++i) {
    if (x_Lon) x_Lon[i] = 2.0 * PI * i / P.I;
    if (x_Lon_Weight) x_Lon_Weight[i] = 2.0 * PI / P.I;
  }
  for (int j = 0; j < P.J; ++j) {
    if (y_Lat) y_Lat[j] = asin(P.mu[j]);
    if (y_Lat_Weight) y_Lat_Weight[j] = P.w[j];
  }
  return DCCM_OK;
}

extern "C" int dccm_sht_gauss(const dccm_sht_plan *p, double *mu, double *w) {
  if (!p || !mu || !w) return DCCM_ERR_INVALID_ARG;
  memcpy(mu, p->P.mu.data(), p->P.J * sizeof(double));
  memcpy(w, p->P.w.data(), p->P.J * sizeof(double));
  return DCCM_OK;
}

extern "C" int dccm_sht_pnm(const dccm_sht_plan *p, double *pnm) {
  DCCM_NVTX_FUNC();
  if (!p || !pnm) return DCCM_ERR_INVALID_ARG;
  DCCM_CUDA(cudaMemcpy(pnm, p->P.d_pnm, (size_t)p->P.ncoef * p->P.Jh * sizeof(double),
                       cudaMemcpyDeviceToHost));
  return DCCM_OK;
}

static int check_batch(const dccm_sht_plan *p, int batch) {
  if (!p || batch < 0) return DCCM_ERR_INVALID_ARG;
  if (batch > p->P.max_batch) return DCCM_ERR_SHAPE;
  return DCCM_OK;
}

extern "C" int dccm_sht_inverse_dev(dccm_sht_plan *p, const double *spec, double *grid, int batch,
                                    void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(check_batch(p, batch));
  if (batch > 0 && (!spec || !grid)) return DCCM_ERR_INVALID_ARG;
  return sht::inverse(p->P, spec, grid, batch, as_stream(stream));
}

extern "C" int dccm_sht_forward_dev(dccm_sht_plan *p, const double *grid, double *spec, int batch,
                                    void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(check_batch(p, batch));
  if (batch > 0 && (!spec || !grid)) return DCCM_ERR_INVALID_ARG;
  return sht::forward(p->P, grid, spec, batch, as_stream(stream));
}

extern "C" int dccm_sht_status(dccm_sht_plan *p, int *device_error) {
  DCCM_NVTX_FUNC();
  if (!p) return DCCM_ERR_INVALID_ARG;
  DCCM_CUDA(cudaDeviceSynchronize());
  int e = 0;
  DCCM_CUDA(cudaMemcpy(&e, p->P.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (device_error) *device_error = e;
  if (e) {
    DCCM_CUDA(cudaMemset(p->P.d_err, 0, sizeof(int)));
    return DCCM_ERR_TIMEOUT;
  }
  return DCCM_OK;
}

// Host arrays: copies in, transform, copies out, checks the device error flag.
static int host_call(dccm_sht_plan *p, const double *in, size_t in_n, double *out, size_t out_n, int batch,
                     bool inv) {
  sht::Plan &P = p->P;
  if (!P.stream) DCCM_CUDA(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
  DCCM_TRY(P.stage.ensure((in_n + out_n) * sizeof(double)));
  double *din = (double *)P.stage.ptr, *dout = din + in_n;
  DCCM_CUDA(cudaMemcpyAsync(din, in, in_n * sizeof(double), cudaMemcpyHostToDevice, P.stream));
  if (inv) DCCM_TRY(sht::inverse(P, din, dout, batch, P.stream));
  else DCCM_TRY(sht::forward(P, din, dout, batch, P.stream));
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

extern "C" int dccm_sht_inverse(dccm_sht_plan *p, const double *spec, double *grid, int batch) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(check_batch(p, batch));
  if (batch == 0) return DCCM_OK;
  if (!spec || !grid) return DCCM_ERR_INVALID_ARG;
  const size_t ns = (size_t)batch * p->P.ncoef * 2, ng = (size_t)batch * p->P.J * p->P.I;
  return host_call(p, spec, ns, grid, ng, batch, true);
}

extern "C" int dccm_sht_forward(dccm_sht_plan *p, const double *grid, double *spec, int batch) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(check_batch(p, batch));
  if (batch == 0) return DCCM_OK;
  if (!spec || !grid) return DCCM_ERR_INVALID_ARG;
  const size_t ns = (size_t)batch * p->P.ncoef * 2, ng = (size_t)batch * p->P.J * p->P.I;
  return host_call(p, grid, ng, spec, ns, batch, false);
}

// ----------------------------------------------------------------- ensemble
// Several truncation groups (an ensemble of members with mixed truncations,
// members of one truncation concatenated into one group).  On the mixed
// path each direction is one persistent tcgen05 Legendre launch and one FFT
// launch over all groups; the FP64 path runs the groups one after another.
struct dccm_sht_ensemble {
  std::vector<dccm_sht_plan *> plans;
  int precision = 0;
};

extern "C" int dccm_sht_ensemble_create(int ngroups, const int *nmax, const int *imax, const int *jmax,
                                        const int *max_batch, int precision, dccm_sht_ensemble **ens) {
  DCCM_NVTX_FUNC();
  if (!ens) return DCCM_ERR_INVALID_ARG;
  *ens = nullptr;
  if (ngroups < 1 || ngroups > 8 || !nmax || !imax || !jmax || !max_batch) return DCCM_ERR_INVALID_ARG;
  dccm_sht_ensemble *e = new (std::nothrow) dccm_sht_ensemble();
  if (!e) return DCCM_ERR_NOMEM;
  e->precision = precision;
  for (int g = 0; g < ngroups; ++g) {
    dccm_sht_plan *p = nullptr;
    const int st = dccm_sht_plan_create(nmax[g], imax[g], jmax[g], precision, max_batch[g], &p);
    if (st != DCCM_OK) {
      dccm_sht_ensemble_destroy(e);
      return st;
    }
    e->plans.push_back(p);
  }
  *ens = e;
  return DCCM_OK;
}

extern "C" int dccm_sht_ensemble_destroy(dccm_sht_ensemble *e) {
  DCCM_NVTX_FUNC();
  if (!e) return DCCM_OK;
  for (dccm_sht_plan *p : e->plans) dccm_sht_plan_destroy(p);
  delete e;
  return DCCM_OK;
}

static int ens_check(dccm_sht_ensemble *e, const void *a, const void *b, const int *batch) {
  if (!e || !a || !b || !batch) return DCCM_ERR_INVALID_ARG;
  for (size_t g = 0; g < e->plans.size(); ++g)
    if (batch[g] < 0 || batch[g] > e->plans[g]->P.max_batch) return DCCM_ERR_SHAPE;
  return DCCM_OK;
}

namespace dccm {
namespace sht {
int ensemble_inverse(dccm_sht_ensemble *e, const double *const *spec, double *const *grid, const int *batch,
                     cudaStream_t s) {
  const int ng = (int)e->plans.size();
  if (e->precision == DCCM_SHT_FP64) {
    for (int g = 0; g < ng; ++g)
      if (batch[g] > 0) DCCM_TRY(inverse(e->plans[g]->P, spec[g], grid[g], batch[g], s));
    return DCCM_OK;
  }
  Plan *pp[8];
  const void *in[8];
  void *work[8];
  for (int g = 0; g < ng; ++g) {
    pp[g] = &e->plans[g]->P;
    in[g] = spec[g];
    work[g] = pp[g]->d_work;
  }
  DCCM_TRY(pack_spectra(pp, batch, spec, ng, s));
  DCCM_TRY(legendre_tc_multi(pp, batch, in, work, ng, 0, s));
  return fft_multi(pp, batch, (const void *const *)work, (void *const *)grid, ng, false, s);
}

int ensemble_forward(dccm_sht_ensemble *e, const double *const *grid, double *const *spec, const int *batch,
                     cudaStream_t s) {
  const int ng = (int)e->plans.size();
  if (e->precision == DCCM_SHT_FP64) {
    for (int g = 0; g < ng; ++g)
      if (batch[g] > 0) DCCM_TRY(forward(e->plans[g]->P, grid[g], spec[g], batch[g], s));
    return DCCM_OK;
  }
  Plan *pp[8];
  void *work[8];
  for (int g = 0; g < ng; ++g) {
    pp[g] = &e->plans[g]->P;
    work[g] = pp[g]->d_work;
  }
  DCCM_TRY(fft_multi(pp, batch, (const void *const *)grid, work, ng, true, s));
  return legendre_tc_multi(pp, batch, (const void *const *)work, (void *const *)spec, ng, 1, s);
}
}  // namespace sht
}  // namespace dccm

extern "C" int dccm_sht_ensemble_inverse_dev(dccm_sht_ensemble *e, const double *const *spec,
                                             double *const *grid, const int *batch, void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(ens_check(e, spec, grid, batch));
  return sht::ensemble_inverse(e, spec, grid, batch, as_stream(stream));
}

extern "C" int dccm_sht_ensemble_forward_dev(dccm_sht_ensemble *e, const double *const *grid,
                                             double *const *spec, const int *batch, void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(ens_check(e, grid, spec, batch));
  return sht::ensemble_forward(e, grid, spec, batch, as_stream(stream));
}

extern "C" int dccm_sht_ensemble_status(dccm_sht_ensemble *e, int *device_error) {
  DCCM_NVTX_FUNC();
  if (!e) return DCCM_ERR_INVALID_ARG;
  int worst = 0, st = DCCM_OK;
  for (dccm_sht_plan *p : e->plans) {
    int d = 0;
    const int s = dccm_sht_status(p, &d);
    if (d) worst = d;
    if (s != DCCM_OK) st = s;
  }
  if (device_error) *device_error = worst;
  return st;
}

extern "C" int dccm_sht_ensemble_groups(const dccm_sht_ensemble *e, int *ngroups) {
  if (!e || !ngroups) return DCCM_ERR_INVALID_ARG;
  *ngroups = (int)e->plans.size();
  return DCCM_OK;
}

namespace dccm {
namespace sht {
Plan *ensemble_plan(dccm_sht_ensemble *e, int g) { return &e->plans[g]->P; }
}  // namespace sht
}  // namespace dccm
