// Spectral-space operators around the transform: per total wavenumber n
// scalings of [batch][ncoef] complex spectra (m-major, the SHT layout,
// idx(m, n) = m(N+1) - m(m-1)/2 + (n - m)).
//
// The reference calls them inside DynamicsHSplVAS83 (atm/dcpam_main_mod.f90:
// 2173-2180, from the external dcpam5 library, not in the source tree) with
// HDOrder = 8 and an e-folding time of the largest wavenumber
// (exp/APEI07Couple/common/dcpam/dcpam_APEI07Couple_T21L16.conf:205-227).
// They are built here from the mathematics, with a the planet radius:
//   Laplacian             f_n = -n(n+1)/a^2
//   inverse Laplacian     f_n = -a^2/(n(n+1)), f_0 = 0
//   hyperdiffusion        D_n = nu (K_n - c), K_n = (n(n+1)/a^2)^(order/2),
//                         c = K_1 with the rotation correction (rigid
//                         rotation, n = 1, is not damped), else 0; D_0 = 0
//                         (the global mean is never diffused),
//                         nu = 1 / (tau (K_N - c)): wavenumber N decays by e
//                         in tau
//     tendency            f_n = -D_n
//     implicit step       f_n = 1 / (1 + dt D_n)
//
// The host evaluates f_n for n = 0..N once (N <= 2047) and passes the
// table as a kernel parameter; a CTA covers one order m (its coefficients
// n = m..N are contiguous) for a slice of the batch, so every element costs
// one load, two FP64 multiplies and one store: HBM-bound, 32 bytes per
// coefficient and field-level.
#include "common.cuh"
#include "nvtx.cuh"

namespace dccm {
namespace spec {

constexpr int NT_MAX = 2048;  // f_n table entries: 16 KB of kernel parameters
struct NTable {
  double f[NT_MAX];
};

// Factor table of the operator (the formulas above), on the host.
int factors(int nmax, const dccm_spec_op *o, NTable &t) {
  if (!o || nmax < 0 || !(o->radius > 0.0)) return DCCM_ERR_INVALID_ARG;
  if (o->kind < DCCM_SPEC_LAPLACIAN || o->kind > DCCM_SPEC_HDIFF_IMPLICIT) return DCCM_ERR_INVALID_ARG;
  if (nmax >= NT_MAX) return DCCM_ERR_UNSUPPORTED;
  const double a2 = o->radius * o->radius;
  int p = 0;
  double nu = 0.0, c = 0.0;
  auto K = [&](double n) {
    double r = 1.0;
    for (int i = 0; i < p; ++i) r *= n * (n + 1.0) / a2;
    return r;
  };
  if (o->kind >= DCCM_SPEC_HDIFF_TENDENCY) {
    if (o->order < 2 || o->order % 2 || o->order > 32 || !(o->efold_time > 0.0) || nmax < 2)
      return DCCM_ERR_INVALID_ARG;
    p = o->order / 2;
    c = o->rotation_correction ? K(1.0) : 0.0;
    nu = 1.0 / (o->efold_time * (K((double)nmax) - c));
  }
  for (int n = 0; n <= nmax; ++n) {
    const double nn = (double)n * (double)(n + 1);
    double f;
    switch (o->kind) {
      case DCCM_SPEC_LAPLACIAN:
        f = -nn / a2;
        break;
      case DCCM_SPEC_INV_LAPLACIAN:
        f = n == 0 ? 0.0 : -a2 / nn;
        break;
      default: {
        double r = 1.0;
        for (int i = 0; i < p; ++i) r *= nn / a2;
        const double d = n == 0 ? 0.0 : nu * (r - c);
        f = o->kind == DCCM_SPEC_HDIFF_TENDENCY ? -d : 1.0 / (1.0 + o->dt * d);
      }
    }
    t.f[n] = f;
  }
  return DCCM_OK;
}

// CTA (m, batch slice of per_block field-levels); in may equal out: each
// element is read once, then written by the same thread.
constexpr int U = 4;
__global__ void __launch_bounds__(256) apply_kernel(int N, int ncoef, const double2 *in, double2 *out, int batch,
                                                    int per_block, const __grid_constant__ NTable t) {
  const int m = blockIdx.x;
  const int k0 = m * (2 * N + 3 - m) / 2;
  const int len = N + 1 - m;
  const int b0 = blockIdx.y * per_block;
  const int b1 = min(batch, b0 + per_block);
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    const double f = t.f[m + i];
    const size_t k = (size_t)(k0 + i);
    for (int b = b0; b < b1; b += U) {
      double2 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (b + u < b1) v[u] = in[(size_t)(b + u) * ncoef + k];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (b + u < b1) out[(size_t)(b + u) * ncoef + k] = make_double2(f * v[u].x, f * v[u].y);
    }
  }
}

}  // namespace spec
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_spec_apply_dev(int nmax, const dccm_spec_op *o, const double *spec_in, double *spec_out,
                                   int batch, void *stream) {
  DCCM_NVTX_FUNC();
  static thread_local spec::NTable t;
  DCCM_TRY(spec::factors(nmax, o, t));
  if (batch < 0 || (batch > 0 && (!spec_in || !spec_out))) return DCCM_ERR_INVALID_ARG;
  if (batch == 0) return DCCM_OK;
  const int ncoef = (nmax + 1) * (nmax + 2) / 2;
  const int threads = nmax + 1 >= 256 ? 256 : ((nmax + 1 + 31) / 32) * 32;
  // U field-levels per CTA: every thread issues its U loads at once, and the
  // (m, slice) grid holds many CTAs in flight for the short rows of large m
  int per = spec::U;
  if ((batch + per - 1) / per > 65535) per = (batch + 65534) / 65535;
  spec::apply_kernel<<<dim3(nmax + 1, (batch + per - 1) / per), threads, 0, as_stream(stream)>>>(
      nmax, ncoef, reinterpret_cast<const double2 *>(spec_in), reinterpret_cast<double2 *>(spec_out), batch, per, t);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

extern "C" int dccm_spec_apply(int nmax, const dccm_spec_op *o, const double *spec_in, double *spec_out,
                               int batch) {
  DCCM_NVTX_FUNC();
  static thread_local spec::NTable t;
  DCCM_TRY(spec::factors(nmax, o, t));
  if (batch < 0 || (batch > 0 && (!spec_in || !spec_out))) return DCCM_ERR_INVALID_ARG;
  if (batch == 0) return DCCM_OK;
  const size_t bytes = (size_t)batch * (nmax + 1) * (nmax + 2) / 2 * 2 * sizeof(double);
  static thread_local DevBuf buf;
  DCCM_TRY(buf.ensure(bytes));
  DCCM_CUDA(cudaMemcpy(buf.ptr, spec_in, bytes, cudaMemcpyHostToDevice));
  DCCM_TRY(dccm_spec_apply_dev(nmax, o, (const double *)buf.ptr, (double *)buf.ptr, batch, nullptr));
  DCCM_CUDA(cudaMemcpy(spec_out, buf.ptr, bytes, cudaMemcpyDeviceToHost));
  return DCCM_OK;
}
