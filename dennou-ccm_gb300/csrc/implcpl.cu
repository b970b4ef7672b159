// Implicit surface coupling of the vertical diffusion (the producer of the
// bulk-flux kernel's ImplCplCoef1/2 and the consumer of its DelVarImplCPL):
//   forward   SfcImplicitCoupling_VDiffForward
//             (atm/dcpam_sfc_implicit_coupling_mod.f90:72-378) with
//             Solve_TriDiagSystem_Forward (:380-405);
//   backward  SfcImplicitCoupling_VDiffBackward (:25-70) with
//             Solve_TriDiagSystem_Backward (:407-420).
// One thread per atmosphere column; every array is the reference's
// (i, j, k[, n]) layout with the columns flattened, so consecutive threads
// touch consecutive addresses at every level.  The three tridiagonal
// systems (momentum, temperature, tracers) are built and eliminated from
// the model top down in place, in the plan-owned matrices that the
// reference keeps as module state for the backward sweep.
//
// FP64 throughout.  Divisions are the scarce operation on this GPU (the
// FP64 pipe is 1/64 of FP32), so the elimination computes one reciprocal
// of (M(k,-1) M(k+1,0)) per level and matrix and multiplies every
// right-hand side by it (the momentum matrix serves U and V, the tracer
// matrix every tracer), the mass term uses 1 / (g 2 dt), and each level's
// full Exner function is inverted once.  Results agree with the
// reference's operation order to rounding (the tests hold 1e-13).  Level 1
// of the eliminated systems divides by the zero sub-diagonal the reference
// sets at k = 1 (:199, :237, :272), as the reference does: the coupler
// replaces U, V, T and the vapour tracer there with the surface solution
// before the backward sweep (atm/dccm_atm_mod.f90:832-835).
#include <new>

#include "common.cuh"

struct dccm_implcpl {
  int ncol = 0, kmax = 0, ncmax = 0, ih2o = 1;
  dccm_implcpl_consts k;
  double *d_mtx = nullptr;  // UV, Temp, QMix: each (ncol, kmax, -1:1)
  dccm::DevBuf stage;       // host entry points
  cudaStream_t stream = nullptr;
};

namespace dccm {
namespace implcpl {

struct Fwd {
  const double *MomX, *MomY, *Heat, *QFlx, *P, *Ef, *Eh, *Tv, *Z, *Kv, *Kt, *Kq;
  double *DU, *DV, *DT, *DQ, *C1, *C2;
  double *uv, *tm, *qm;
  long long ncol;
  int kmax, ncmax, ih2o;
  double Grav, CpDry, GasR, inv_g2dt;
};

__global__ void __launch_bounds__(128) forward_kernel(const Fwd a) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  const long long n = a.ncol;
  const int K = a.kmax;
  const long long mstr = n * K;  // one diagonal
  auto H = [&](const double *x, int k) { return x[c + n * k]; };                 // half level k = 0..K
  auto F = [&](auto *x, int k) -> auto & { return x[c + n * (k - 1)]; };          // full level k = 1..K
  auto M = [&](double *m, int k, int d) -> double & { return m[c + n * (k - 1) + mstr * (d + 1)]; };

  // ---- matrices and right-hand sides (:188-308), level by level, carrying
  // the transfer coefficients and inverse Exner functions of k-1, k, k+1
  double vp = 0.0, tp = 0.0, qp = 0.0;  // transfer coefficients at half level k-1
  double iep = 0.0;                     // 1 / Exner at full level k-1
  double iec = 1.0 / F(a.Ef, 1);
  double Pprev = H(a.P, 0);
  double dfadt1 = 0.0;
  for (int k = 1; k <= K; ++k) {
    double vk = 0.0, tk = 0.0, qk = 0.0, ien = 0.0;
    if (k < K) {
      const double tmp = H(a.P, k) / (a.GasR * H(a.Tv, k) * (F(a.Z, k + 1) - F(a.Z, k)));
      vk = H(a.Kv, k) * tmp;
      tk = H(a.Kt, k) * tmp;
      qk = H(a.Kq, k) * tmp;
      ien = 1.0 / F(a.Ef, k + 1);
    }
    const double Pk = H(a.P, k);
    const double mass = -(Pk - Pprev) * a.inv_g2dt;
    Pprev = Pk;
    // momentum and tracers
    // (+0 where the reference assigns 0: the sign of the level-1 division
    // by the zero sub-diagonal follows it)
    M(a.uv, k, -1) = k > 1 ? -vp : 0.0;
    M(a.uv, k, 0) = mass + vp + vk;
    M(a.uv, k, 1) = k < K ? -vk : 0.0;
    M(a.qm, k, -1) = k > 1 ? -qp : 0.0;
    M(a.qm, k, 0) = mass + qp + qk;
    M(a.qm, k, 1) = k < K ? -qk : 0.0;
    // temperature: the Exner ratios of the reference's dry static energy form
    const double ehp = k > 1 ? a.CpDry * H(a.Eh, k - 1) * tp : 0.0;
    const double ehk = a.CpDry * H(a.Eh, k) * tk;
    M(a.tm, k, -1) = k > 1 ? -(ehp * iep) : 0.0;
    M(a.tm, k, 0) = a.CpDry * mass + ehp * iec + ehk * iec;
    M(a.tm, k, 1) = k < K ? -(ehk * ien) : 0.0;
    if (k == 1) dfadt1 = ehk * iec;  // DFADT1 = Cp Exner_h(1) TTC(1) / Exner_f(1)
    // right-hand sides: flux divergences
    F(a.DU, k) = -(H(a.MomX, k) - H(a.MomX, k - 1));
    F(a.DV, k) = -(H(a.MomY, k) - H(a.MomY, k - 1));
    F(a.DT, k) = -(H(a.Heat, k) - H(a.Heat, k - 1));
    for (int t = 0; t < a.ncmax; ++t) {
      const double *q = a.QFlx + n * (long long)(K + 1) * t;
      a.DQ[c + n * ((k - 1) + (long long)K * t)] = -(q[c + n * k] - q[c + n * (k - 1)]);
    }
    vp = vk;
    tp = tk;
    qp = qk;
    iep = iec;
    iec = ien;
  }
  const double vt1 = M(a.uv, 1, 1), qt1 = M(a.qm, 1, 1);  // -(transfer coefficient at half level 1)
  const double tt1 = M(a.tm, 1, 1);  // DFADT2 = -Cp Exner_h(1) TTC(1) / Exner_f(2)
  a.C2[c + n * 0] = F(a.DU, 1);      // :310-313
  a.C2[c + n * 1] = F(a.DV, 1);
  a.C2[c + n * 2] = F(a.DT, 1);
  a.C2[c + n * 3] = a.DQ[c + n * ((long long)K * (a.ih2o - 1))];

  // ---- elimination from the top (:380-405) for all systems at once
  {
    const double iu = 1.0 / M(a.uv, K, -1), it = 1.0 / M(a.tm, K, -1), iq = 1.0 / M(a.qm, K, -1);
    M(a.uv, K, 0) *= iu;
    F(a.DU, K) *= iu;
    F(a.DV, K) *= iu;
    M(a.uv, K, -1) = 1.0;
    M(a.tm, K, 0) *= it;
    F(a.DT, K) *= it;
    M(a.tm, K, -1) = 1.0;
    M(a.qm, K, 0) *= iq;
    for (int t = 0; t < a.ncmax; ++t) a.DQ[c + n * ((K - 1) + (long long)K * t)] *= iq;
    M(a.qm, K, -1) = 1.0;
  }
  double u0 = M(a.uv, K, 0), t0 = M(a.tm, K, 0), q0 = M(a.qm, K, 0);  // M(k+1, 0)
  for (int k = K - 1; k >= 1; --k) {
    const double iu = 1.0 / (M(a.uv, k, -1) * u0);
    const double it = 1.0 / (M(a.tm, k, -1) * t0);
    const double iq = 1.0 / (M(a.qm, k, -1) * q0);
    const double pu = M(a.uv, k, 1), pt = M(a.tm, k, 1), pq = M(a.qm, k, 1);
    F(a.DU, k) = (F(a.DU, k) * u0 - pu * F(a.DU, k + 1)) * iu;
    F(a.DV, k) = (F(a.DV, k) * u0 - pu * F(a.DV, k + 1)) * iu;
    F(a.DT, k) = (F(a.DT, k) * t0 - pt * F(a.DT, k + 1)) * it;
    for (int t = 0; t < a.ncmax; ++t) {
      double *q = a.DQ + n * (long long)K * t;
      q[c + n * (k - 1)] = (q[c + n * (k - 1)] * q0 - pq * q[c + n * k]) * iq;
    }
    u0 = (M(a.uv, k, 0) * u0 - pu) * iu;
    t0 = (M(a.tm, k, 0) * t0 - pt) * it;
    q0 = (M(a.qm, k, 0) * q0 - pq) * iq;
    M(a.uv, k, 0) = u0;
    M(a.tm, k, 0) = t0;
    M(a.qm, k, 0) = q0;
    M(a.uv, k, -1) = 1.0;
    M(a.uv, k, 1) = 0.0;
    M(a.tm, k, -1) = 1.0;
    M(a.tm, k, 1) = 0.0;
    M(a.qm, k, -1) = 1.0;
    M(a.qm, k, 1) = 0.0;
  }

  // ---- coupling coefficients (:342-375); DFADUV1 = -DFADUV2 = the
  // transfer coefficient at half level 1 (vt1 is the super-diagonal)
  const double Tmp = -(H(a.P, 1) - H(a.P, 0)) * a.inv_g2dt;
  const double iu2 = 1.0 / M(a.uv, 2, 0), it2 = 1.0 / M(a.tm, 2, 0), iq2 = 1.0 / M(a.qm, 2, 0);
  const double cu = Tmp - vt1 - vt1 * iu2;
  a.C1[c + n * 0] = cu;
  a.C2[c + n * 0] = a.C2[c + n * 0] - vt1 * F(a.DU, 2) * iu2;
  a.C1[c + n * 1] = cu;
  a.C2[c + n * 1] = a.C2[c + n * 1] - vt1 * F(a.DV, 2) * iu2;
  a.C1[c + n * 2] = a.CpDry * Tmp + dfadt1 - tt1 * it2;
  a.C2[c + n * 2] = a.C2[c + n * 2] - tt1 * F(a.DT, 2) * it2;
  a.C1[c + n * 3] = Tmp - qt1 - qt1 * iq2;
  a.C2[c + n * 3] = a.C2[c + n * 3] - qt1 * a.DQ[c + n * (1 + (long long)K * (a.ih2o - 1))] * iq2;
}

// Back substitution (:407-420) and the division by 2 dt (:53-61).
struct Bwd {
  const double *uv, *tm, *qm;
  double *DU, *DV, *DT, *DQ;
  long long ncol;
  int kmax, ncmax;
  double inv_2dt;
};

__global__ void __launch_bounds__(128) backward_kernel(const Bwd a) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  const long long n = a.ncol;
  const int K = a.kmax;
  const long long mstr = n * K;
  auto M = [&](const double *m, int k, int d) { return m[c + n * (k - 1) + mstr * (d + 1)]; };
  double u = a.DU[c], v = a.DV[c], t = a.DT[c];
  a.DU[c] = u * a.inv_2dt;
  a.DV[c] = v * a.inv_2dt;
  a.DT[c] = t * a.inv_2dt;
  for (int k = 2; k <= K; ++k) {
    const long long o = c + n * (k - 1);
    const double iu = 1.0 / M(a.uv, k, 0), it = 1.0 / M(a.tm, k, 0);
    u = (a.DU[o] - M(a.uv, k, -1) * u) * iu;
    v = (a.DV[o] - M(a.uv, k, -1) * v) * iu;
    t = (a.DT[o] - M(a.tm, k, -1) * t) * it;
    a.DU[o] = u * a.inv_2dt;
    a.DV[o] = v * a.inv_2dt;
    a.DT[o] = t * a.inv_2dt;
  }
  for (int s = 0; s < a.ncmax; ++s) {
    double *q = a.DQ + n * (long long)K * s;
    double x = q[c];
    q[c] = x * a.inv_2dt;
    for (int k = 2; k <= K; ++k) {
      const long long o = c + n * (k - 1);
      x = (q[o] - M(a.qm, k, -1) * x) / M(a.qm, k, 0);
      q[o] = x * a.inv_2dt;
    }
  }
}

}  // namespace implcpl
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_implcpl_create(int ncol, int kmax, int ncmax, int index_h2ovap,
                                   const dccm_implcpl_consts *consts, dccm_implcpl **plan) {
  if (!plan || !consts) return DCCM_ERR_INVALID_ARG;
  *plan = nullptr;
  if (ncol < 1 || kmax < 2 || ncmax < 1 || index_h2ovap < 1 || index_h2ovap > ncmax) return DCCM_ERR_INVALID_ARG;
  if (!(consts->Grav > 0.0) || !(consts->DelTime > 0.0)) return DCCM_ERR_INVALID_ARG;
  dccm_implcpl *p = new (std::nothrow) dccm_implcpl();
  if (!p) return DCCM_ERR_NOMEM;
  p->ncol = ncol;
  p->kmax = kmax;
  p->ncmax = ncmax;
  p->ih2o = index_h2ovap;
  p->k = *consts;
  const cudaError_t e = cudaMalloc(&p->d_mtx, (size_t)3 * 3 * kmax * ncol * sizeof(double));
  if (e != cudaSuccess) {
    set_cuda_error(e);
    delete p;
    return DCCM_ERR_CUDA;
  }
  *plan = p;
  return DCCM_OK;
}

extern "C" int dccm_implcpl_destroy(dccm_implcpl *p) {
  if (!p) return DCCM_OK;
  if (p->d_mtx) cudaFree(p->d_mtx);
  p->stage.release();
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return DCCM_OK;
}

static size_t mstride(const dccm_implcpl *p) { return (size_t)3 * p->kmax * p->ncol; }

extern "C" int dccm_implcpl_forward_dev(dccm_implcpl *p, const dccm_implcpl_forward_args *a, void *stream) {
  if (!p || !a) return DCCM_ERR_INVALID_ARG;
  const void *need[] = {a->xyr_MomFluxX, a->xyr_MomFluxY, a->xyr_HeatFlux, a->xyrf_QMixFlux, a->xyr_Press,
                        a->xyz_Exner, a->xyr_Exner, a->xyr_VirTemp, a->xyz_Height, a->xyr_VelDiffCoef,
                        a->xyr_TempDiffCoef, a->xyr_QMixDiffCoef, a->xyz_DUDt, a->xyz_DVDt, a->xyz_DTempDt,
                        a->xyzf_DQMixDt, a->xya_ImplCplCoef1, a->xya_ImplCplCoef2};
  for (const void *q : need)
    if (!q) return DCCM_ERR_INVALID_ARG;
  implcpl::Fwd f;
  f.MomX = a->xyr_MomFluxX;
  f.MomY = a->xyr_MomFluxY;
  f.Heat = a->xyr_HeatFlux;
  f.QFlx = a->xyrf_QMixFlux;
  f.P = a->xyr_Press;
  f.Ef = a->xyz_Exner;
  f.Eh = a->xyr_Exner;
  f.Tv = a->xyr_VirTemp;
  f.Z = a->xyz_Height;
  f.Kv = a->xyr_VelDiffCoef;
  f.Kt = a->xyr_TempDiffCoef;
  f.Kq = a->xyr_QMixDiffCoef;
  f.DU = a->xyz_DUDt;
  f.DV = a->xyz_DVDt;
  f.DT = a->xyz_DTempDt;
  f.DQ = a->xyzf_DQMixDt;
  f.C1 = a->xya_ImplCplCoef1;
  f.C2 = a->xya_ImplCplCoef2;
  f.uv = p->d_mtx;
  f.tm = p->d_mtx + mstride(p);
  f.qm = p->d_mtx + 2 * mstride(p);
  f.ncol = p->ncol;
  f.kmax = p->kmax;
  f.ncmax = p->ncmax;
  f.ih2o = p->ih2o;
  f.Grav = p->k.Grav;
  f.CpDry = p->k.CpDry;
  f.GasR = p->k.GasRDry;
  f.inv_g2dt = 1.0 / (p->k.Grav * (2.0 * p->k.DelTime));
  const int threads = 128;
  implcpl::forward_kernel<<<(unsigned)((p->ncol + threads - 1) / threads), threads, 0, as_stream(stream)>>>(f);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

extern "C" int dccm_implcpl_backward_dev(dccm_implcpl *p, double *xyz_DUDt, double *xyz_DVDt,
                                         double *xyz_DTempDt, double *xyzf_DQMixDt, void *stream) {
  if (!p || !xyz_DUDt || !xyz_DVDt || !xyz_DTempDt || !xyzf_DQMixDt) return DCCM_ERR_INVALID_ARG;
  implcpl::Bwd b;
  b.uv = p->d_mtx;
  b.tm = p->d_mtx + mstride(p);
  b.qm = p->d_mtx + 2 * mstride(p);
  b.DU = xyz_DUDt;
  b.DV = xyz_DVDt;
  b.DT = xyz_DTempDt;
  b.DQ = xyzf_DQMixDt;
  b.ncol = p->ncol;
  b.kmax = p->kmax;
  b.ncmax = p->ncmax;
  b.inv_2dt = 1.0 / (2.0 * p->k.DelTime);
  const int threads = 128;
  implcpl::backward_kernel<<<(unsigned)((p->ncol + threads - 1) / threads), threads, 0, as_stream(stream)>>>(b);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

// Host entry points: stage through the plan's device buffer.
static int host_stream(dccm_implcpl *p) {
  if (!p->stream) DCCM_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  return DCCM_OK;
}

extern "C" int dccm_implcpl_forward(dccm_implcpl *p, const dccm_implcpl_forward_args *a) {
  if (!p || !a) return DCCM_ERR_INVALID_ARG;
  DCCM_TRY(host_stream(p));
  const size_t n = p->ncol, K = p->kmax, nc = p->ncmax;
  const size_t half = n * (K + 1), full = n * K;
  // inputs: 9 half-level arrays, 2 full-level, tracer fluxes; outputs: 3 full,
  // tracer tendencies, 2 x 4 coefficients
  const size_t tot = 9 * half + 2 * full + nc * half + 3 * full + nc * full + 8 * n;
  DCCM_TRY(p->stage.ensure(tot * sizeof(double)));
  double *d = static_cast<double *>(p->stage.ptr);
  const double *hin[] = {a->xyr_MomFluxX, a->xyr_MomFluxY, a->xyr_HeatFlux, a->xyr_Press, a->xyr_Exner,
                         a->xyr_VirTemp, a->xyr_VelDiffCoef, a->xyr_TempDiffCoef, a->xyr_QMixDiffCoef};
  for (const double *q : hin)
    if (!q) return DCCM_ERR_INVALID_ARG;
  if (!a->xyz_Exner || !a->xyz_Height || !a->xyrf_QMixFlux || !a->xyz_DUDt || !a->xyz_DVDt ||
      !a->xyz_DTempDt || !a->xyzf_DQMixDt || !a->xya_ImplCplCoef1 || !a->xya_ImplCplCoef2)
    return DCCM_ERR_INVALID_ARG;
  double *dh[9];
  size_t off = 0;
  for (int i = 0; i < 9; ++i, off += half) {
    dh[i] = d + off;
    DCCM_CUDA(cudaMemcpyAsync(dh[i], hin[i], half * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  }
  double *dEf = d + off;
  off += full;
  double *dZ = d + off;
  off += full;
  double *dQF = d + off;
  off += nc * half;
  DCCM_CUDA(cudaMemcpyAsync(dEf, a->xyz_Exner, full * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(dZ, a->xyz_Height, full * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(dQF, a->xyrf_QMixFlux, nc * half * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  dccm_implcpl_forward_args g;
  g.xyr_MomFluxX = dh[0];
  g.xyr_MomFluxY = dh[1];
  g.xyr_HeatFlux = dh[2];
  g.xyr_Press = dh[3];
  g.xyr_Exner = dh[4];
  g.xyr_VirTemp = dh[5];
  g.xyr_VelDiffCoef = dh[6];
  g.xyr_TempDiffCoef = dh[7];
  g.xyr_QMixDiffCoef = dh[8];
  g.xyz_Exner = dEf;
  g.xyz_Height = dZ;
  g.xyrf_QMixFlux = dQF;
  g.xyz_DUDt = d + off;
  off += full;
  g.xyz_DVDt = d + off;
  off += full;
  g.xyz_DTempDt = d + off;
  off += full;
  g.xyzf_DQMixDt = d + off;
  off += nc * full;
  g.xya_ImplCplCoef1 = d + off;
  off += 4 * n;
  g.xya_ImplCplCoef2 = d + off;
  DCCM_TRY(dccm_implcpl_forward_dev(p, &g, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xyz_DUDt, g.xyz_DUDt, full * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xyz_DVDt, g.xyz_DVDt, full * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xyz_DTempDt, g.xyz_DTempDt, full * sizeof(double), cudaMemcpyDeviceToHost,
                            p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xyzf_DQMixDt, g.xyzf_DQMixDt, nc * full * sizeof(double), cudaMemcpyDeviceToHost,
                            p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xya_ImplCplCoef1, g.xya_ImplCplCoef1, 4 * n * sizeof(double),
                            cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(a->xya_ImplCplCoef2, g.xya_ImplCplCoef2, 4 * n * sizeof(double),
                            cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaStreamSynchronize(p->stream));
  return DCCM_OK;
}

extern "C" int dccm_implcpl_backward(dccm_implcpl *p, double *xyz_DUDt, double *xyz_DVDt, double *xyz_DTempDt,
                                     double *xyzf_DQMixDt) {
  if (!p || !xyz_DUDt || !xyz_DVDt || !xyz_DTempDt || !xyzf_DQMixDt) return DCCM_ERR_INVALID_ARG;
  DCCM_TRY(host_stream(p));
  const size_t full = (size_t)p->ncol * p->kmax, nc = p->ncmax;
  DCCM_TRY(p->stage.ensure((3 + nc) * full * sizeof(double)));
  double *d = static_cast<double *>(p->stage.ptr);
  double *h[4] = {xyz_DUDt, xyz_DVDt, xyz_DTempDt, xyzf_DQMixDt};
  const size_t len[4] = {full, full, full, nc * full};
  double *dv[4];
  size_t off = 0;
  for (int i = 0; i < 4; ++i) {
    dv[i] = d + off;
    off += len[i];
    DCCM_CUDA(cudaMemcpyAsync(dv[i], h[i], len[i] * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  }
  DCCM_TRY(dccm_implcpl_backward_dev(p, dv[0], dv[1], dv[2], dv[3], p->stream));
  for (int i = 0; i < 4; ++i)
    DCCM_CUDA(cudaMemcpyAsync(h[i], dv[i], len[i] * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaStreamSynchronize(p->stream));
  return DCCM_OK;
}

extern "C" int dccm_implcpl_matrices(dccm_implcpl *p, double *uv, double *temp, double *qmix) {
  if (!p) return DCCM_ERR_INVALID_ARG;
  double *h[3] = {uv, temp, qmix};
  for (int i = 0; i < 3; ++i)
    if (h[i]) DCCM_CUDA(cudaMemcpy(h[i], p->d_mtx + i * mstride(p), mstride(p) * sizeof(double), cudaMemcpyDeviceToHost));
  return DCCM_OK;
}
