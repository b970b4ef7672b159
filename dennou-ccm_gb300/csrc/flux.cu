// Surface bulk flux: one fused FP64 column kernel.
//
// Replaces DSFCM_Util_SfcBulkFlux_Get + BulkCoefL82
// (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-572; constants :35-58; limits
// :574-591).  The reference runs four OpenMP loop nests over the grid and
// keeps ~25 full-grid temporaries; here every statement is column-local,
// so one thread evaluates the whole routine for one column in registers:
// 21 FP64 reads and 42 FP64 writes per column, nothing else touches HBM.
// Expressions follow the reference's, except that divisions not followed
// by a cancelling difference are products with a shared reciprocal, the
// elementary functions are those of fp64_fast.cuh (within 2 ulp), and a
// few common factors are computed once; each such step moves a result by
// an ulp or two, far inside the 1e-13 agreement tested.  The two reference
// behaviours without a single defined result are given the meaning stated
// in dccm_gb300.h (per-type sea-ice flag in the final loop; slot-3 latent
// heat flux as the fraction-weighted merge of slots 1 and 2).
#include <string.h>

#include "common.cuh"
#include "flux_rows.cuh"
#include "fp64_fast.cuh"
#include "nvtx.cuh"

namespace dccm {
namespace flux {

// Constants (:35-58) and read_config limits (:574-591).
constexpr double FKarm = 0.4;
constexpr double GasRUniv = 8.3144621;
constexpr double StB = 5.670373e-8;
constexpr double Grav = 9.8;
constexpr double MolWtDry = 1.8e-2;
constexpr double MolWtWet = 1.8e-2;
constexpr double CpDry = 1616.0;
constexpr double LatentHeat = 2425300.0;
constexpr double LatentHeatFusion = 334000.0;
constexpr double RefPress = 1e5;
constexpr double Es0 = 611.0;
constexpr double RoughLength = 1e-4;
constexpr double RoughLenHeatFactor = 1.0;
constexpr double VelMinForRi = 0.01, VelMinForVel = 0.01, VelMinForTemp = 0.01,
                 VelMinForQVap = 0.01;
constexpr double VelMaxForVel = 1000.0, VelMaxForTemp = 1000.0, VelMaxForQVap = 1000.0;
constexpr double VelBulkCoefMin = 0.0, TempBulkCoefMin = 0.0, QVapBulkCoefMin = 0.0;
constexpr double VelBulkCoefMax = 1.0, TempBulkCoefMax = 1.0, QVapBulkCoefMax = 1.0;

struct Ptrs {
  double *__restrict__ WSX, *__restrict__ WSY, *__restrict__ Sen, *__restrict__ QV,
      *__restrict__ Lat, *__restrict__ CVel, *__restrict__ CTemp, *__restrict__ CQ,
      *__restrict__ DelV, *__restrict__ SUw, *__restrict__ LUw, *__restrict__ Fns,
      *__restrict__ Fsr, *__restrict__ DFdT;
  const double *__restrict__ U, *__restrict__ V, *__restrict__ Ta, *__restrict__ q1,
      *__restrict__ SDw, *__restrict__ LDw, *__restrict__ C1, *__restrict__ C2;
  double *__restrict__ Ts, *__restrict__ Alb;
  const double *__restrict__ Ice, *__restrict__ Zs, *__restrict__ Ps;
};

struct Geom {
  int64_t plane;  // IA*JA
  int IA, IS, JS, NI;
  int64_t ncol;  // NI*NJ
  double sig1;
  double sig1k;  // sig1^(R/Cp): Exner(p1) = Exner(ps) * sig1k
  double hfac;   // (R/g) (1 - sig1): the first level's height above the surface is hfac VirTemp
};

// qm = (z - zs + z0m) / z0m and qh = (z - zs + z0h) / z0h, the arguments of
// the neutral coefficients' logarithms (computed once by the caller).
__device__ __forceinline__ void bulk_coef_l82(double Ri, double qm, double qh, double cmn, double chn, bool flag,
                                              double &cm, double &ch, double &cq) {
  double vm, th;
  if (flag) {
    if (Ri > 0.0) {
      double h;  // 1 / (2 r)
      const double r = fp64::sqrt_h(1.0 + 5.0 * Ri, h);
      vm = cmn * fp64::rcp(1.0 + 20.0 * Ri * h);  // 10 Ri / r
      th = chn * fp64::rcp(1.0 + 15.0 * Ri * r);
    } else {
      vm = cmn * (1.0 - 10.0 * Ri * fp64::rcp(1.0 + 75.0 * cmn * fp64::sqrt(-(qm * Ri))));
      th = chn * (1.0 - 15.0 * Ri * fp64::rcp(1.0 + 75.0 * chn * fp64::sqrt(-(qh * Ri))));
    }
  } else {
    vm = 0.0;
    th = 0.0;
  }
  cm = fmax(fmin(vm, VelBulkCoefMax), VelBulkCoefMin);
  ch = fmax(fmin(th, TempBulkCoefMax), TempBulkCoefMin);
  cq = fmax(fmin(th, QVapBulkCoefMax), QVapBulkCoefMin);
}

// Input row k of column t (linear interior index) at device element c: the
// bound host row, or the device array.  HOST = false is the kernel without
// host rows (the table is not read).
template <bool HOST>
__device__ __forceinline__ double rd(const HostRows &h, int k, const double *dev, int64_t c, int64_t t) {
  if (HOST && h.in[k]) return h.in[k][t];
  return dev[c];
}
// A bound input's value into its device row: after every input is read, so
// that no load waits behind these stores.
template <bool HOST>
__device__ __forceinline__ void mirror(const HostRows &h, int k, int64_t t, double v) {
  if (HOST && h.in[k]) h.din[k][t] = v;
}
// Output row k: the device array, and the bound host row.
template <bool HOST>
__device__ __forceinline__ void wr(const HostRows &h, int k, double *dev, int64_t c, int64_t t, double v) {
  dev[c] = v;
  if (HOST && h.out[k]) h.out[k][t] = v;
}

// One column t (device element c).  PURE: the caller's whole warp has no
// sea ice at all (SIceCon = 0), so Frac = (1, 0), the ice slot is skipped
// and every merged value 0 + 1 X[0] is X[0] (up to the sign of an exact
// zero) with no FP64 operation; PURE = false is the general column.  The
// two are separate code paths so that the general one keeps its register
// allocation.
template <bool HOST, bool PURE>
__device__ __forceinline__ void flux_column(const Ptrs &p, const Geom &g, const HostRows &h, int64_t t, int64_t c,
                                            double SIceCon) {
  constexpr double GasRDry = GasRUniv / MolWtDry;
  constexpr double GasRWet = GasRUniv / MolWtWet;
  constexpr double EpsV = MolWtWet / MolWtDry;
  const double aL[2] = {LatentHeat, LatentHeat + LatentHeatFusion};
  const int64_t P = g.plane;
  const double Ps = rd<HOST>(h, I_PS, p.Ps, c, t);
  const double Ta = rd<HOST>(h, I_TA, p.Ta, c, t);
  const double q1 = rd<HOST>(h, I_Q1, p.q1, c, t);
  const double U = rd<HOST>(h, I_U, p.U, c, t), V = rd<HOST>(h, I_V, p.V, c, t);
  const double zs = rd<HOST>(h, I_ZS, p.Zs, c, t);
  const double SDw = rd<HOST>(h, I_SDW, p.SDw, c, t), LDw = rd<HOST>(h, I_LDW, p.LDw, c, t);
  const double z0m = RoughLength;
  const double z0h = RoughLenHeatFactor * z0m;
  const double humd = 1.0;

  // FP64 is the scarce pipe on this GPU: divisions that do not feed a
  // cancelling difference become products with a reciprocal (fp64::rcp,
  // three DFMA from an FP32 seed), exp and log are the table-driven ones
  // of fp64_fast.cuh, and the two Exner functions share one exp/log pair,
  // (ps/P0)^k = exp(k log), with Exner(sig1 ps) = Exner(ps) sig1^k.  Each
  // rewrite moves a result by an ulp or two, far inside the 1e-13
  // agreement with the reference.
  const double rPs = fp64::rcp(Ps);
  double Frac[2], QSat[2], SVT[2], Tsn[2], Albn[2], rTs[2];
  Frac[0] = 1.0 - SIceCon;
  Frac[1] = SIceCon;
  // Sea-ice flag (:269-273, :389-393): with no ice the reference still
  // evaluates the ice column, but every ice output is then an exact zero
  // (bulk coefficients clamp to 0); the ice physics is skipped here.  The
  // results are the same for any positive finite ice temperature.
  const bool ice = !PURE && Frac[1] > 1e-12;
  constexpr bool pure = PURE;
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    Tsn[n] = rd<HOST>(h, I_TS + n, p.Ts, c + P * n, t);
    Albn[n] = rd<HOST>(h, I_ALB + n, p.Alb, c + P * n, t);
    if (n == 1 && !ice) {
      rTs[n] = QSat[n] = SVT[n] = 0.0;
      continue;
    }
    rTs[n] = fp64::rcp(Tsn[n]);
    QSat[n] = (EpsV * Es0) * rPs * fp64::exp(fma(-aL[n] / GasRWet, rTs[n], aL[n] / GasRWet * (1.0 / 273.0)));
    SVT[n] = Tsn[n] * (1.0 + (((1.0 / EpsV) - 1.0) * QSat[n]));
  }
  const double VirTemp = Ta * (1.0 + (((1.0 / EpsV) - 1.0) * q1));
  const double SfcExner = fp64::exp((GasRDry / CpDry) * fp64::log(Ps * (1.0 / RefPress)));
  const double Exner = SfcExner * g.sig1k;
  const double rExner = fp64::rcp(Exner);
  const double rSfcExner = fp64::rcp(SfcExner);
  const double VelAbs = fp64::sqrt(U * U + V * V);
  // Height - zs, the reference's Height (:223-225) less the surface height
  const double dH = g.hfac * VirTemp;

  // Neutral coefficients (:250-260) depend only on the column (the
  // roughness lengths are the same constants for both surface types).
  const double qm = (dH + z0m) * (1.0 / z0m);
  const double qh = RoughLenHeatFactor == 1.0 ? qm : (dH + z0h) * (1.0 / z0h);
  const double tmp = FKarm * fp64::rcp(fp64::log(qm));
  const double cmn = tmp * tmp;
  // z0h = RoughLenHeatFactor z0m: with the factor 1 both logarithms are one
  const double chn = RoughLenHeatFactor == 1.0 ? cmn : tmp * (FKarm * fp64::rcp(fp64::log(qh)));
  const double vmx = fmax(VelAbs, VelMinForRi);
  const double vmx2 = vmx * vmx;
  // The Richardson number and the sensible heat flux subtract nearly equal
  // quotients: these keep correctly rounded divisions (Markstein's
  // correction of a times the shared reciprocal).
  const double VT_E = fp64::div_rb(VirTemp, Exner, rExner);
  const double Ta_E = fp64::div_rb(Ta, Exner, rExner);

  double CVel[2], CTemp[2], CQ[2], WSX[2], WSY[2], Sen[2], QV[2], LatH[2], LUw[2], SUw[2];
  bool flag[2];
  double WSX3 = 0.0, WSY3 = 0.0, Sen3 = 0.0, QV3 = 0.0, SUw3 = 0.0, LUw3 = 0.0, Ts3 = 0.0,
         Alb3 = 0.0, CVel3 = 0.0, CTemp3 = 0.0, CQ3 = 0.0;
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    const bool f = (n == 0) ? true : ice;
    flag[n] = f;
    if (!f) {
      CVel[n] = CTemp[n] = CQ[n] = 0.0;
      WSX[n] = WSY[n] = Sen[n] = QV[n] = LatH[n] = LUw[n] = SUw[n] = 0.0;
      continue;
    }
    const double SVT_SE = fp64::div_rb(SVT[n], SfcExner, rSfcExner);
    // Ri = g / SVT_SE (VT_E - SVT_SE) / vmx^2 dH and rho = Ps / (R SVT)
    // from one reciprocal y = 1 / (SVT vmx^2): 1 / SVT_SE = SfcExner y vmx^2
    const double y = fp64::rcp(SVT[n] * vmx2);
    const double Ri = (Grav * SfcExner) * (VT_E - SVT_SE) * dH * y;
    double cm, ch, cq;
    bulk_coef_l82(Ri, qm, qh, cmn, chn, f, cm, ch, cq);
    const double rho = (Ps * (1.0 / GasRDry)) * (vmx2 * y);
    CVel[n] = cm * rho * fmin(fmax(VelAbs, VelMinForVel), VelMaxForVel);
    CTemp[n] = ch * rho * fmin(fmax(VelAbs, VelMinForTemp), VelMaxForTemp);
    CQ[n] = cq * rho * fmin(fmax(VelAbs, VelMinForQVap), VelMaxForQVap);
    if (f) {
      WSX[n] = -CVel[n] * U;
      WSY[n] = -CVel[n] * V;
      Sen[n] = -CpDry * SfcExner * CTemp[n] * (Ta_E - fp64::div_rb(Tsn[n], SfcExner, rSfcExner));
      QV[n] = -humd * CQ[n] * (q1 - QSat[n]);
      LatH[n] = aL[n] * QV[n];
      const double T2 = Tsn[n] * Tsn[n];
      const double T4 = T2 * T2;
      LUw[n] = StB * T4;
      SUw[n] = Albn[n] * SDw;
      if (pure) {  // n = 0 only
        Ts3 = T4;
        Alb3 = Albn[n];
        WSX3 = WSX[n];
        WSY3 = WSY[n];
        Sen3 = Sen[n];
        QV3 = QV[n];
        LUw3 = LUw[n];
        SUw3 = SUw[n];
        CVel3 = CVel[n];
        CTemp3 = CTemp[n];
        CQ3 = CQ[n];
      } else {
        Ts3 = Ts3 + Frac[n] * T4;
        Alb3 = Alb3 + Frac[n] * Albn[n];
        WSX3 = WSX3 + Frac[n] * WSX[n];
        WSY3 = WSY3 + Frac[n] * WSY[n];
        Sen3 = Sen3 + Frac[n] * Sen[n];
        QV3 = QV3 + Frac[n] * QV[n];
        LUw3 = LUw3 + Frac[n] * LUw[n];
        SUw3 = SUw3 + Frac[n] * SUw[n];
        CVel3 = CVel3 + Frac[n] * CVel[n];
        CTemp3 = CTemp3 + Frac[n] * CTemp[n];
        CQ3 = CQ3 + Frac[n] * CQ[n];
      }
    } else {
      WSX[n] = WSY[n] = Sen[n] = QV[n] = LatH[n] = LUw[n] = SUw[n] = 0.0;
    }
  }

  // Implicit-coupling back-substitution (:355-382).
  const double c11 = rd<HOST>(h, I_C1, p.C1, c, t), c12 = rd<HOST>(h, I_C1 + 1, p.C1, c + P, t),
               c13 = rd<HOST>(h, I_C1 + 2, p.C1, c + 2 * P, t), c14 = rd<HOST>(h, I_C1 + 3, p.C1, c + 3 * P, t);
  const double c21 = rd<HOST>(h, I_C2, p.C2, c, t), c22 = rd<HOST>(h, I_C2 + 1, p.C2, c + P, t),
               c23 = rd<HOST>(h, I_C2 + 2, p.C2, c + 2 * P, t), c24 = rd<HOST>(h, I_C2 + 3, p.C2, c + 3 * P, t);
  if (HOST) {  // every input has been read: the bound ones into their device rows
    const double vin[NIN] = {SIceCon, Ps, Ta, q1, U, V, zs, SDw, LDw, Tsn[0], Tsn[1], Albn[0], Albn[1],
                             c11, c12, c13, c14, c21, c22, c23, c24};
#pragma unroll
    for (int k = 0; k < NIN; ++k) mirror<HOST>(h, k, t, vin[k]);
  }
  const double DFsDT1 = -CpDry * SfcExner * CTemp3 * rExner;
  const double f1 = fp64::rcp(c11 + CVel3) * (WSX3 + c21);
  const double f2 = fp64::rcp(c12 + CVel3) * (WSY3 + c22);
  const double f3 = fp64::rcp(c13 - DFsDT1) * (Sen3 + c23);
  const double f4 = fp64::rcp(c14 + humd * CQ3) * (QV3 + c24);
  wr<HOST>(h, O_DELV, p.DelV, c, t, f1);
  wr<HOST>(h, O_DELV + 1, p.DelV, c + P, t, f2);
  wr<HOST>(h, O_DELV + 2, p.DelV, c + 2 * P, t, f3);
  wr<HOST>(h, O_DELV + 3, p.DelV, c + 3 * P, t, f4);

  const double sfac = CpDry * SfcExner * rExner;
  double Lat3 = 0.0;
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    if (n == 1 && !ice) break;  // the ice slot's zeros stay zeros (0 - 0 f = 0 for finite f)
    WSX[n] = WSX[n] - CVel[n] * f1;
    WSY[n] = WSY[n] - CVel[n] * f2;
    Sen[n] = Sen[n] - sfac * CTemp[n] * f3;
    QV[n] = QV[n] - humd * CQ[n] * f4;
    LatH[n] = aL[n] * QV[n];
    if (flag[n] && !pure) Lat3 = Lat3 + Frac[n] * LatH[n];
  }
  if (pure) {  // the merged values are slot 0's and get its update
    WSX3 = WSX[0];
    WSY3 = WSY[0];
    Sen3 = Sen[0];
    QV3 = QV[0];
    Lat3 = LatH[0];
  } else {
    WSX3 = WSX3 - CVel3 * f1;
    WSY3 = WSY3 - CVel3 * f2;
    Sen3 = Sen3 - sfac * CTemp3 * f3;
    QV3 = QV3 - humd * CQ3 * f4;
  }

  // Net heat fluxes and dF/dTs (:384-415), flag per surface type.
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    double fns = 0.0, fsr = 0.0, dfdt = 0.0;
    if (flag[n]) {
      fns = +LUw[n] - LDw + LatH[n] + Sen[n];
      fsr = SUw[n] - SDw;
      dfdt = +4.0 * StB * (Tsn[n] * Tsn[n] * Tsn[n]) + CpDry * CTemp[n] +
             (aL[n] * aL[n] * humd / GasRWet) * (CQ[n] * QSat[n]) * (rTs[n] * rTs[n]);
    }
    const int64_t cn = c + P * n;
    wr<HOST>(h, O_FNS + n, p.Fns, cn, t, fns);
    wr<HOST>(h, O_FSR + n, p.Fsr, cn, t, fsr);
    wr<HOST>(h, O_DFDT + n, p.DFdT, cn, t, dfdt);
    wr<HOST>(h, O_WSX + n, p.WSX, cn, t, WSX[n]);
    wr<HOST>(h, O_WSY + n, p.WSY, cn, t, WSY[n]);
    wr<HOST>(h, O_SEN + n, p.Sen, cn, t, Sen[n]);
    wr<HOST>(h, O_QV + n, p.QV, cn, t, QV[n]);
    wr<HOST>(h, O_LAT + n, p.Lat, cn, t, LatH[n]);
    wr<HOST>(h, O_CVEL + n, p.CVel, cn, t, CVel[n]);
    wr<HOST>(h, O_CTEMP + n, p.CTemp, cn, t, CTemp[n]);
    wr<HOST>(h, O_CQ + n, p.CQ, cn, t, CQ[n]);
    wr<HOST>(h, O_SUW + n, p.SUw, cn, t, SUw[n]);
    wr<HOST>(h, O_LUW + n, p.LUw, cn, t, LUw[n]);
  }
  const int64_t c3 = c + 2 * P;
  wr<HOST>(h, O_WSX + 2, p.WSX, c3, t, WSX3);
  wr<HOST>(h, O_WSY + 2, p.WSY, c3, t, WSY3);
  wr<HOST>(h, O_SEN + 2, p.Sen, c3, t, Sen3);
  wr<HOST>(h, O_QV + 2, p.QV, c3, t, QV3);
  wr<HOST>(h, O_LAT + 2, p.Lat, c3, t, Lat3);
  wr<HOST>(h, O_CVEL + 2, p.CVel, c3, t, CVel3);
  wr<HOST>(h, O_CTEMP + 2, p.CTemp, c3, t, CTemp3);
  wr<HOST>(h, O_CQ + 2, p.CQ, c3, t, CQ3);
  wr<HOST>(h, O_SUW + 2, p.SUw, c3, t, SUw3);
  wr<HOST>(h, O_LUW + 2, p.LUw, c3, t, LUw3);
  wr<HOST>(h, O_TS3, p.Ts, c3, t, Ts3);
  wr<HOST>(h, O_ALB3, p.Alb, c3, t, Alb3);
}

template <bool HOST>
__global__ void __launch_bounds__(256, 2) bulk_flux_column(Ptrs p, Geom g, const __grid_constant__ HostRows h) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < g.ncol;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int ii = (int)(t % g.NI);
    const int jj = (int)(t / g.NI);
    const int64_t c = (int64_t)(g.IS - 1 + ii) + (int64_t)g.IA * (g.JS - 1 + jj);
    const double SIceCon = rd<HOST>(h, I_ICE, p.Ice, c, t);
    const bool pure = ((unsigned long long)__double_as_longlong(SIceCon) << 1) == 0ull;
    if (__all_sync(__activemask(), pure)) flux_column<HOST, true>(p, g, h, t, c, SIceCon);
    else flux_column<HOST, false>(p, g, h, t, c, SIceCon);
  }
}

static int check_grid(const dccm_sfc_grid *g) {
  if (!g) return DCCM_ERR_INVALID_ARG;
  if (g->IA <= 0 || g->JA <= 0) return DCCM_ERR_SHAPE;
  if (g->IS < 1 || g->JS < 1 || g->IE > g->IA || g->JE > g->JA) return DCCM_ERR_SHAPE;
  return DCCM_OK;
}

static int check_args(const dccm_sfc_bulk_flux_args *a) {
  if (!a) return DCCM_ERR_INVALID_ARG;
  const void *const ptrs[] = {a->WindStressX, a->WindStressY, a->SenHFlx, a->QVapMFlx,
                              a->LatHFlx, a->SfcVelTransCoef, a->SfcTempTransCoef,
                              a->SfcQVapTransCoef, a->DelVarImplCPL, a->SUwRFlx, a->LUwRFlx,
                              a->SfcHFlx_ns, a->SfcHFlx_sr, a->DSfcHFlxDTs, a->WindU,
                              a->WindV, a->SfcAirTemp, a->QVap1, a->SDwRFlx, a->LDwRFlx,
                              a->ImplCplCoef1, a->ImplCplCoef2, a->SfcTemp, a->SfcAlbedo,
                              a->SIceCon, a->a_Sig1Info, a->SfcHeight, a->SfcPress};
  for (const void *q : ptrs)
    if (!q) return DCCM_ERR_INVALID_ARG;
  return DCCM_OK;
}

static Ptrs make_ptrs(const dccm_sfc_bulk_flux_args *a) {
  Ptrs p;
  p.WSX = a->WindStressX; p.WSY = a->WindStressY; p.Sen = a->SenHFlx; p.QV = a->QVapMFlx;
  p.Lat = a->LatHFlx; p.CVel = a->SfcVelTransCoef; p.CTemp = a->SfcTempTransCoef;
  p.CQ = a->SfcQVapTransCoef; p.DelV = a->DelVarImplCPL; p.SUw = a->SUwRFlx;
  p.LUw = a->LUwRFlx; p.Fns = a->SfcHFlx_ns; p.Fsr = a->SfcHFlx_sr; p.DFdT = a->DSfcHFlxDTs;
  p.U = a->WindU; p.V = a->WindV; p.Ta = a->SfcAirTemp; p.q1 = a->QVap1; p.SDw = a->SDwRFlx;
  p.LDw = a->LDwRFlx; p.C1 = a->ImplCplCoef1; p.C2 = a->ImplCplCoef2; p.Ts = a->SfcTemp;
  p.Alb = a->SfcAlbedo; p.Ice = a->SIceCon; p.Zs = a->SfcHeight; p.Ps = a->SfcPress;
  return p;
}

int launch(const Ptrs &p, const dccm_sfc_grid *g, double sig1, cudaStream_t s, const HostRows *hr = nullptr) {
  Geom geo;
  geo.plane = (int64_t)g->IA * g->JA;
  geo.IA = g->IA;
  geo.IS = g->IS;
  geo.JS = g->JS;
  geo.NI = g->IE - g->IS + 1;
  const int NJ = g->JE - g->JS + 1;
  if (geo.NI <= 0 || NJ <= 0) return DCCM_OK;
  geo.ncol = (int64_t)geo.NI * NJ;
  geo.sig1 = sig1;
  geo.sig1k = pow(sig1, (GasRUniv / MolWtDry) / CpDry);
  geo.hfac = (GasRUniv / MolWtDry) / Grav * (1.0 - sig1);
  const int threads = tunables().flux_threads > 0 ? tunables().flux_threads : 128;
  int64_t blocks = (geo.ncol + threads - 1) / threads;
  // In the coupling step the flux runs beside the transforms: fewer CTAs
  // leave them more issue slots (flux_ctas, chosen on whole-step timings).
  const int64_t cap = tunables().flux_ctas > 0 ? (int64_t)tunables().flux_ctas : (int64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  HostRows none;
  if (!hr) {
    memset(&none, 0, sizeof none);
    hr = &none;
  }
  if (hr->any)
    DCCM_CUDA(launch_surface(bulk_flux_column<true>, dim3((unsigned)blocks), dim3(threads), 0, s, p, geo, *hr));
  else
    DCCM_CUDA(launch_surface(bulk_flux_column<false>, dim3((unsigned)blocks), dim3(threads), 0, s, p, geo, *hr));
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

double *in_row(const dccm_sfc_bulk_flux_args &a, const dccm_sfc_grid &g, int k) {
  const void *base[NIN] = {a.SIceCon, a.SfcPress, a.SfcAirTemp, a.QVap1, a.WindU, a.WindV, a.SfcHeight,
                           a.SDwRFlx, a.LDwRFlx, a.SfcTemp, a.SfcTemp, a.SfcAlbedo, a.SfcAlbedo,
                           a.ImplCplCoef1, a.ImplCplCoef1, a.ImplCplCoef1, a.ImplCplCoef1,
                           a.ImplCplCoef2, a.ImplCplCoef2, a.ImplCplCoef2, a.ImplCplCoef2};
  int slot = 0;
  if (k >= I_TS && k < I_ALB) slot = k - I_TS;
  else if (k >= I_ALB && k < I_C1) slot = k - I_ALB;
  else if (k >= I_C1 && k < I_C2) slot = k - I_C1;
  else if (k >= I_C2) slot = k - I_C2;
  return row_start(base[k], g, slot);
}

double *out_row(const dccm_sfc_bulk_flux_args &a, const dccm_sfc_grid &g, int k) {
  if (k < O_FNS) return row_start(a.DelVarImplCPL, g, k - O_DELV);
  if (k < O_FSR) return row_start(a.SfcHFlx_ns, g, k - O_FNS);
  if (k < O_DFDT) return row_start(a.SfcHFlx_sr, g, k - O_FSR);
  if (k < O_WSX) return row_start(a.DSfcHFlxDTs, g, k - O_DFDT);
  if (k == O_TS3) return row_start(a.SfcTemp, g, 2);
  if (k == O_ALB3) return row_start(a.SfcAlbedo, g, 2);
  const void *three[10] = {a.WindStressX, a.WindStressY, a.SenHFlx, a.QVapMFlx, a.LatHFlx,
                           a.SfcVelTransCoef, a.SfcTempTransCoef, a.SfcQVapTransCoef, a.SUwRFlx, a.LUwRFlx};
  return row_start(three[(k - O_WSX) / 3], g, (k - O_WSX) % 3);
}

int launch_rows(const dccm_sfc_bulk_flux_args *a, const dccm_sfc_grid *g, const HostRows *h, cudaStream_t s) {
  DCCM_TRY(check_args(a));
  DCCM_TRY(check_grid(g));
  if (h && h->any && g->JE != g->JS) return DCCM_ERR_UNSUPPORTED;  // host rows: one interior row
  return launch(make_ptrs(a), g, a->a_Sig1Info[0], s, h);
}

// Host entry point state: one device staging area per process.
static DevBuf g_stage;
static cudaStream_t g_stream = nullptr;

}  // namespace flux
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_sfc_bulk_flux_get_dev(const dccm_sfc_bulk_flux_args *a,
                                          const dccm_sfc_grid *g, void *stream) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(flux::check_args(a));
  DCCM_TRY(flux::check_grid(g));
  return flux::launch(flux::make_ptrs(a), g, a->a_Sig1Info[0], as_stream(stream));
}

// Copy the interior IS..IE x JS..JE of nk planes between a host and a device
// (IA,JA,nk) array, starting at plane k0.
static int copy_interior(void *dst, const void *src, const dccm_sfc_grid *g, int k0, int nk,
                         cudaMemcpyKind kind, cudaStream_t s) {
  cudaMemcpy3DParms prm = {};
  const size_t pitch = (size_t)g->IA * sizeof(double);
  prm.srcPtr = make_cudaPitchedPtr(const_cast<void *>(src), pitch, g->IA, g->JA);
  prm.dstPtr = make_cudaPitchedPtr(dst, pitch, g->IA, g->JA);
  prm.srcPos = make_cudaPos((size_t)(g->IS - 1) * sizeof(double), g->JS - 1, k0);
  prm.dstPos = prm.srcPos;
  prm.extent = make_cudaExtent((size_t)(g->IE - g->IS + 1) * sizeof(double),
                               g->JE - g->JS + 1, nk);
  prm.kind = kind;
  DCCM_CUDA(cudaMemcpy3DAsync(&prm, s));
  return DCCM_OK;
}

extern "C" int dccm_sfc_bulk_flux_get(const dccm_sfc_bulk_flux_args *a, const dccm_sfc_grid *g) {
  DCCM_NVTX_FUNC();
  DCCM_TRY(flux::check_args(a));
  DCCM_TRY(flux::check_grid(g));
  if (g->IE < g->IS || g->JE < g->JS) return DCCM_OK;
  if (!flux::g_stream) DCCM_CUDA(cudaStreamCreateWithFlags(&flux::g_stream, cudaStreamNonBlocking));
  cudaStream_t s = flux::g_stream;
  const size_t plane = (size_t)g->IA * g->JA;
  // Device layout: 10 out x3, DelV x4, Fns/Fsr/DFdT x3, 6 in x1, C1/C2 x4,
  // Ts/Alb x3, Ice/Zs/Ps x1  -> 72 planes.
  DCCM_TRY(flux::g_stage.ensure(plane * sizeof(double) * 72));
  double *base = (double *)flux::g_stage.ptr;
  size_t off = 0;
  auto take = [&](int k) { double *q = base + off; off += plane * k; return q; };
  dccm_sfc_bulk_flux_args d = *a;
  d.WindStressX = take(3); d.WindStressY = take(3); d.SenHFlx = take(3); d.QVapMFlx = take(3);
  d.LatHFlx = take(3); d.SfcVelTransCoef = take(3); d.SfcTempTransCoef = take(3);
  d.SfcQVapTransCoef = take(3); d.DelVarImplCPL = take(4); d.SUwRFlx = take(3);
  d.LUwRFlx = take(3); d.SfcHFlx_ns = take(3); d.SfcHFlx_sr = take(3); d.DSfcHFlxDTs = take(3);
  double *U = take(1), *V = take(1), *Ta = take(1), *q1 = take(1), *SDw = take(1), *LDw = take(1);
  double *C1 = take(4), *C2 = take(4);
  d.SfcTemp = take(3); d.SfcAlbedo = take(3);
  double *Ice = take(1), *Zs = take(1), *Ps = take(1);
  d.WindU = U; d.WindV = V; d.SfcAirTemp = Ta; d.QVap1 = q1; d.SDwRFlx = SDw; d.LDwRFlx = LDw;
  d.ImplCplCoef1 = C1; d.ImplCplCoef2 = C2; d.SIceCon = Ice; d.SfcHeight = Zs; d.SfcPress = Ps;

  const cudaMemcpyKind H2D = cudaMemcpyHostToDevice, D2H = cudaMemcpyDeviceToHost;
  DCCM_TRY(copy_interior(U, a->WindU, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(V, a->WindV, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(Ta, a->SfcAirTemp, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(q1, a->QVap1, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(SDw, a->SDwRFlx, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(LDw, a->LDwRFlx, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(C1, a->ImplCplCoef1, g, 0, 4, H2D, s));
  DCCM_TRY(copy_interior(C2, a->ImplCplCoef2, g, 0, 4, H2D, s));
  DCCM_TRY(copy_interior(d.SfcTemp, a->SfcTemp, g, 0, 2, H2D, s));
  DCCM_TRY(copy_interior(d.SfcAlbedo, a->SfcAlbedo, g, 0, 2, H2D, s));
  DCCM_TRY(copy_interior(Ice, a->SIceCon, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(Zs, a->SfcHeight, g, 0, 1, H2D, s));
  DCCM_TRY(copy_interior(Ps, a->SfcPress, g, 0, 1, H2D, s));

  DCCM_TRY(flux::launch(flux::make_ptrs(&d), g, a->a_Sig1Info[0], s));

  DCCM_TRY(copy_interior(a->WindStressX, d.WindStressX, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->WindStressY, d.WindStressY, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->SenHFlx, d.SenHFlx, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->QVapMFlx, d.QVapMFlx, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->LatHFlx, d.LatHFlx, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->SfcVelTransCoef, d.SfcVelTransCoef, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->SfcTempTransCoef, d.SfcTempTransCoef, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->SfcQVapTransCoef, d.SfcQVapTransCoef, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->DelVarImplCPL, d.DelVarImplCPL, g, 0, 4, D2H, s));
  DCCM_TRY(copy_interior(a->SUwRFlx, d.SUwRFlx, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->LUwRFlx, d.LUwRFlx, g, 0, 3, D2H, s));
  DCCM_TRY(copy_interior(a->SfcHFlx_ns, d.SfcHFlx_ns, g, 0, 2, D2H, s));
  DCCM_TRY(copy_interior(a->SfcHFlx_sr, d.SfcHFlx_sr, g, 0, 2, D2H, s));
  DCCM_TRY(copy_interior(a->DSfcHFlxDTs, d.DSfcHFlxDTs, g, 0, 2, D2H, s));
  DCCM_TRY(copy_interior(a->SfcTemp, d.SfcTemp, g, 2, 1, D2H, s));
  DCCM_TRY(copy_interior(a->SfcAlbedo, d.SfcAlbedo, g, 2, 1, D2H, s));
  DCCM_CUDA(cudaStreamSynchronize(s));
  return DCCM_OK;
}
