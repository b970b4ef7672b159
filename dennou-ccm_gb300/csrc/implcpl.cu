// Implicit surface coupling of the vertical diffusion (the producer of the
// bulk-flux kernel's ImplCplCoef1/2 and the consumer of its DelVarImplCPL):
//   forward   SfcImplicitCoupling_VDiffForward
//             (atm/dcpam_sfc_implicit_coupling_mod.f90:72-378) with
//             Solve_TriDiagSystem_Forward (:380-405);
//   backward  SfcImplicitCoupling_VDiffBackward (:25-70) with
//             Solve_TriDiagSystem_Backward (:407-420).
// One thread per atmosphere column and system (momentum, temperature, each
// tracer); every array is the reference's (i, j, k[, n]) layout with the
// columns flattened, so consecutive threads touch consecutive addresses at
// every level.  The forward sweep builds each level's row and eliminates it
// in the same pass from the model top down, so the matrices that the
// reference keeps as module state for the backward sweep are written once
// and never re-read.
//
// FP64 throughout.  Divisions are the scarce operation on this GPU (the
// FP64 pipe is 1/64 of FP32), so the elimination computes one reciprocal
// of (M(k,-1) M(k+1,0)) per level and matrix and multiplies every
// right-hand side by it (the momentum matrix serves U and V, the tracer
// matrix every tracer), the mass term uses 1 / (g 2 dt), and each level's
// full Exner function is inverted once.  The reciprocals are fp64::rcp
// (an FP32 seed and one cubic Newton step: 3 DFMA, within half an ulp
// and a little; zeros, infinities and out-of-range values take the exact
// division).  Results agree with the reference's operation order to
// rounding (the tests hold 1e-13).  Level 1
// of the eliminated systems divides by the zero sub-diagonal the reference
// sets at k = 1 (:199, :237, :272), as the reference does: the coupler
// replaces U, V, T and the vapour tracer there with the surface solution
// before the backward sweep (atm/dccm_atm_mod.f90:832-835).
#include <new>

#include "common.cuh"
#include "fp64_fast.cuh"
#include "nvtx.cuh"

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
  double *G, *IEF;  // per (level, column) factors shared by the systems (geo_kernel)
  long long ncol;
  int kmax, ncmax, ih2o;
  double Grav, CpDry, GasR, inv_g2dt;
};

// One thread per (column, system): blockIdx.y 0 = momentum (U and V share
// the matrix), 1 = temperature, 2 + t = tracer t (each tracer thread
// eliminates the tracer matrix; tracer 0 stores it).  A single pass from
// the model top down builds each level's row (:188-308) and eliminates it
// at once (:380-405), carrying the eliminated M(k+1,0) and right-hand sides
// of the level above; the eliminated matrix and tendencies are written
// once.  The level inputs are fetched LV levels ahead into registers, so
// the loads of a chunk overlap while the serial elimination runs.
constexpr int LV = 4;   // forward sweep: levels fetched ahead
constexpr int LVB = 8;  // backward sweep

// The factors every system's row uses, once per (level, column) instead of
// once per system: G(j) = P_h(j) / (R Tv_h(j) (z(j+1) - z(j))) at half level
// j = 1..kmax-1 (the transfer coefficient of :182-195 is K(j) G(j)), and the
// reciprocal Exner function 1 / Exner_f(j) at full level j (0-based index,
// the temperature rows of :222-260).  Same expressions; G as a product
// with the reciprocal.
__global__ void __launch_bounds__(256) geo_kernel(const Fwd a) {
  const long long n = a.ncol;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n * a.kmax) return;
  const int j = (int)(t / n);
  const long long c = t - j * n;
  a.IEF[t] = fp64::rcp(a.Ef[c + n * j]);
  if (j >= 1)
    a.G[t] = a.P[c + n * j] * fp64::rcp(a.GasR * a.Tv[c + n * j] * (a.Z[c + n * j] - a.Z[c + n * (j - 1)]));
}

template <int SYS>
__device__ __forceinline__ void forward_column(const Fwd &a, long long c, int tracer) {
  constexpr int NR = SYS == 0 ? 2 : 1;
  const long long n = a.ncol;
  const int K = a.kmax;
  const long long mstr = n * K;
  const double *__restrict__ Kd = SYS == 0 ? a.Kv : (SYS == 1 ? a.Kt : a.Kq);
  const double *__restrict__ fl[NR];
  double *__restrict__ out[NR];
  if constexpr (SYS == 0) {
    fl[0] = a.MomX;
    fl[1] = a.MomY;
    out[0] = a.DU;
    out[1] = a.DV;
  } else if constexpr (SYS == 1) {
    fl[0] = a.Heat;
    out[0] = a.DT;
  } else {
    fl[0] = a.QFlx + n * (long long)(K + 1) * tracer;
    out[0] = a.DQ + n * (long long)K * tracer;
  }
  double *mat = SYS == 0 ? a.uv : (SYS == 1 ? a.tm : a.qm);
  const bool store_mat = SYS != 2 || tracer == 0;
  // values at level k carried from the previous (upper) iteration
  double Pk = a.P[c + n * K], Ehk = a.Eh[c + n * K];
  double flk[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) flk[r] = fl[r][c + n * K];
  double tck = 0.0, ief_k1 = 0.0, ief_k = a.IEF[c + n * (K - 1)];
  double m0p = 0.0, rp[NR], m0_2 = 0.0, r_2[NR], c2[NR], tc1 = 0.0, dfadt1 = 0.0, dfadt2 = 0.0;
  for (int k0 = K; k0 >= 1; k0 -= LV) {
    // fetch half level k-1 and full level k-1 of the next LV levels
    double Pm[LV], Gm[LV], Kdm[LV], Ehm[LV], Iefm[LV], flm[LV][NR];
#pragma unroll
    for (int i = 0; i < LV; ++i) {
      const int k = k0 - i;
      if (k >= 1) {
        Pm[i] = a.P[c + n * (k - 1)];
        if (k > 1) {
          Gm[i] = a.G[c + n * (k - 1)];
          Kdm[i] = Kd[c + n * (k - 1)];
          if (SYS == 1) {
            Ehm[i] = a.Eh[c + n * (k - 1)];
            Iefm[i] = a.IEF[c + n * (k - 2)];
          }
        }
#pragma unroll
        for (int r = 0; r < NR; ++r) flm[i][r] = fl[r][c + n * (k - 1)];
      }
    }
#pragma unroll
    for (int i = 0; i < LV; ++i) {
      const int k = k0 - i;
      if (k < 1) break;
      // transfer coefficient at half level k-1 (0 at the surface, :182-195)
      double tkm = 0.0, ief_km = 0.0;
      if (k > 1) {
        tkm = Kdm[i] * Gm[i];
        if (SYS == 1) ief_km = Iefm[i];
      }
      const double mass = -(Pk - Pm[i]) * a.inv_g2dt;
      double mm, m0, mp;  // row k; +0 where the reference assigns 0
      if constexpr (SYS != 1) {
        mm = k > 1 ? -tkm : 0.0;
        m0 = mass + tkm + tck;
        mp = k < K ? -tck : 0.0;
      } else {
        const double ehm = k > 1 ? a.CpDry * Ehm[i] * tkm : 0.0;
        const double ehk = a.CpDry * Ehk * tck;
        mm = k > 1 ? -(ehm * ief_km) : 0.0;
        m0 = a.CpDry * mass + ehm * ief_k + ehk * ief_k;
        mp = k < K ? -(ehk * ief_k1) : 0.0;
        if (k == 1) {
          dfadt1 = ehk * ief_k;  // DFADT1 = Cp Exner_h(1) TTC(1) / Exner_f(1)
          dfadt2 = mp;           // DFADT2 = -Cp Exner_h(1) TTC(1) / Exner_f(2)
        }
      }
      if (k == 1) tc1 = tck;
      double inv, m0e;
      if (k == K) {
        inv = fp64::rcp(mm);
        m0e = m0 * inv;
      } else {
        inv = fp64::rcp(mm * m0p);
        m0e = (m0 * m0p - mp) * inv;
      }
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const double b = -(flk[r] - flm[i][r]);
        if (k == 1) c2[r] = b;  // ImplCplCoef2 starts from the level-1 divergence (:310-313)
        const double re = k == K ? b * inv : (b * m0p - mp * rp[r]) * inv;
        out[r][c + n * (k - 1)] = re;
        rp[r] = re;
        if (k == 2) r_2[r] = re;
        flk[r] = flm[i][r];
      }
      if (store_mat) {
        mat[c + n * (k - 1)] = 1.0;
        mat[c + n * (k - 1) + mstr] = m0e;
        mat[c + n * (k - 1) + 2 * mstr] = 0.0;
      }
      if (k == 2) m0_2 = m0e;
      m0p = m0e;
      tck = tkm;
      ief_k1 = ief_k;
      ief_k = ief_km;
      Pk = Pm[i];
      if (SYS == 1 && k > 1) Ehk = Ehm[i];
    }
  }
  // coupling coefficients (:342-375); DFADUV1 = -DFADUV2 = TC(1)
  const double Tmp = -(a.P[c + n] - a.P[c]) * a.inv_g2dt;
  const double i2 = fp64::rcp(m0_2);
  if constexpr (SYS == 0) {
    const double cu = Tmp + tc1 + tc1 * i2;
    a.C1[c + n * 0] = cu;
    a.C2[c + n * 0] = c2[0] + tc1 * r_2[0] * i2;
    a.C1[c + n * 1] = cu;
    a.C2[c + n * 1] = c2[1] + tc1 * r_2[1] * i2;
  } else if constexpr (SYS == 1) {
    a.C1[c + n * 2] = a.CpDry * Tmp + dfadt1 - dfadt2 * i2;
    a.C2[c + n * 2] = c2[0] - dfadt2 * r_2[0] * i2;
  } else {
    if (tracer == a.ih2o - 1) {
      a.C1[c + n * 3] = Tmp + tc1 + tc1 * i2;
      a.C2[c + n * 3] = c2[0] + tc1 * r_2[0] * i2;
    }
  }
}

__global__ void __launch_bounds__(128) forward_kernel(const Fwd a) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  if (blockIdx.y == 0) forward_column<0>(a, c, 0);
  else if (blockIdx.y == 1) forward_column<1>(a, c, 0);
  else forward_column<2>(a, c, blockIdx.y - 2);
}

// Back substitution (:407-420) and the division by 2 dt (:53-61), one
// thread per (column, matrix): blockIdx.y 0 = momentum (U and V), 1 =
// temperature, 2 = the tracers; one reciprocal of M(k,0) per level serves
// every right-hand side of the matrix, and levels are fetched LVB at a time
// ahead of the serial chains.
struct Bwd {
  const double *uv, *tm, *qm;
  double *DU, *DV, *DT, *DQ;
  long long ncol;
  int kmax, ncmax;
  double inv_2dt;
};

template <int NR>
__device__ __forceinline__ void backward_chains(const double *__restrict__ mat, double *const *x, long long c,
                                                long long n, int K, double inv_2dt) {
  const long long mstr = n * K;
  double v[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    v[r] = x[r][c];
    x[r][c] = v[r] * inv_2dt;
  }
  for (int k0 = 2; k0 <= K; k0 += LVB) {
    double xs[LVB][NR], mm[LVB], m0[LVB];
#pragma unroll
    for (int i = 0; i < LVB; ++i) {
      const int k = k0 + i;
      if (k <= K) {
        const long long o = c + n * (k - 1);
#pragma unroll
        for (int r = 0; r < NR; ++r) xs[i][r] = x[r][o];
        mm[i] = mat[o];
        m0[i] = mat[o + mstr];
      }
    }
#pragma unroll
    for (int i = 0; i < LVB; ++i) {
      const int k = k0 + i;
      if (k > K) break;
      const double im = fp64::rcp(m0[i]);
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        v[r] = (xs[i][r] - mm[i] * v[r]) * im;
        x[r][c + n * (k - 1)] = v[r] * inv_2dt;
      }
    }
  }
}

__global__ void __launch_bounds__(128) backward_kernel(const Bwd a) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  const long long n = a.ncol;
  const int K = a.kmax;
  if (blockIdx.y == 0) {
    double *x[2] = {a.DU, a.DV};
    backward_chains<2>(a.uv, x, c, n, K, a.inv_2dt);
  } else if (blockIdx.y == 1) {
    double *x[1] = {a.DT};
    backward_chains<1>(a.tm, x, c, n, K, a.inv_2dt);
  } else {
    // tracers in pairs (one reciprocal per level for both)
    for (int t = 0; t < a.ncmax; t += 2) {
      if (t + 1 < a.ncmax) {
        double *x[2] = {a.DQ + n * (long long)K * t, a.DQ + n * (long long)K * (t + 1)};
        backward_chains<2>(a.qm, x, c, n, K, a.inv_2dt);
      } else {
        double *x[1] = {a.DQ + n * (long long)K * t};
        backward_chains<1>(a.qm, x, c, n, K, a.inv_2dt);
      }
    }
  }
}

}  // namespace implcpl
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_implcpl_create(int ncol, int kmax, int ncmax, int index_h2ovap,
                                   const dccm_implcpl_consts *consts, dccm_implcpl **plan) {
  DCCM_NVTX_FUNC();
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
  // the three matrices (3 diagonals each), then the forward sweep's shared
  // factors G and 1/Exner_f (kmax x ncol each)
  const cudaError_t e = cudaMalloc(&p->d_mtx, (size_t)(3 * 3 + 2) * kmax * ncol * sizeof(double));
  if (e != cudaSuccess) {
    set_cuda_error(e);
    delete p;
    return DCCM_ERR_CUDA;
  }
  *plan = p;
  return DCCM_OK;
}

extern "C" int dccm_implcpl_destroy(dccm_implcpl *p) {
  DCCM_NVTX_FUNC();
  if (!p) return DCCM_OK;
  if (p->d_mtx) cudaFree(p->d_mtx);
  p->stage.release();
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return DCCM_OK;
}

static size_t mstride(const dccm_implcpl *p) { return (size_t)3 * p->kmax * p->ncol; }

extern "C" int dccm_implcpl_forward_dev(dccm_implcpl *p, const dccm_implcpl_forward_args *a, void *stream) {
  DCCM_NVTX_FUNC();
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
  f.G = p->d_mtx + 3 * mstride(p);
  f.IEF = f.G + (size_t)p->kmax * p->ncol;
  const long long nk = (long long)p->ncol * p->kmax;
  implcpl::geo_kernel<<<(unsigned)((nk + 255) / 256), 256, 0, as_stream(stream)>>>(f);
  DCCM_LAUNCH_CHECK();
  const int threads = 128;
  implcpl::forward_kernel<<<dim3((unsigned)((p->ncol + threads - 1) / threads), 2 + p->ncmax), threads, 0,
                            as_stream(stream)>>>(f);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

extern "C" int dccm_implcpl_backward_dev(dccm_implcpl *p, double *xyz_DUDt, double *xyz_DVDt,
                                         double *xyz_DTempDt, double *xyzf_DQMixDt, void *stream) {
  DCCM_NVTX_FUNC();
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
  implcpl::backward_kernel<<<dim3((unsigned)((p->ncol + threads - 1) / threads), 3), threads, 0,
                             as_stream(stream)>>>(b);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

extern "C" int dccm_implcpl_info(const dccm_implcpl *p, int *ncol, int *kmax, int *ncmax) {
  if (!p) return DCCM_ERR_INVALID_ARG;
  if (ncol) *ncol = (int)p->ncol;
  if (kmax) *kmax = p->kmax;
  if (ncmax) *ncmax = p->ncmax;
  return DCCM_OK;
}

// Host entry points: stage through the plan's device buffer.
static int host_stream(dccm_implcpl *p) {
  if (!p->stream) DCCM_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  return DCCM_OK;
}

extern "C" int dccm_implcpl_forward(dccm_implcpl *p, const dccm_implcpl_forward_args *a) {
  DCCM_NVTX_FUNC();
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
  DCCM_NVTX_FUNC();
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
  DCCM_NVTX_FUNC();
  if (!p) return DCCM_ERR_INVALID_ARG;
  double *h[3] = {uv, temp, qmix};
  for (int i = 0; i < 3; ++i)
    if (h[i]) DCCM_CUDA(cudaMemcpy(h[i], p->d_mtx + i * mstride(p), mstride(p) * sizeof(double), cudaMemcpyDeviceToHost));
  return DCCM_OK;
}
