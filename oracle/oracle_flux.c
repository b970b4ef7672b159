/*
 * Oracle (test infrastructure): FP64 restatement of the surface bulk flux,
 * DSFCM_Util_SfcBulkFlux_Get + BulkCoefL82
 * (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-572, limits :574-591).
 *
 * PARITY UNPINNED (the Fortran reference cannot be compiled here; see oracle.h).
 *
 * Loop structure is kept per column: every statement of the reference
 * touches only column (i,j), so evaluating the reference's loops column by
 * column gives the same values.  Expressions keep the reference's
 * left-to-right evaluation order; Fortran integer powers x**2, x**3, x**4
 * are written as products.
 *
 * Three places where the reference has no single defined result:
 *  D2  the final loop (:384-415) is an OpenMP collapse over (n, j) that
 *      writes the shared xy_CalcFlag(i,j) for every n.  Serial meaning used:
 *      the flag is evaluated for the n being processed.
 *  D3  :379 reads a_LatentHeatLocal(n) for n = 1..SFC_PROP_MAX = 3, but the
 *      array has extent 2 (:181, :200-201), so slot 3 reads past the array.
 *      Used here: slot 3 of LatHFlx after the implicit correction is the
 *      fraction-weighted merge of the corrected slots 1 and 2, with the
 *      same accumulation as :328.  With no sea ice this equals
 *      LatentHeat * QVapMFlx(:,:,3) exactly.
 *  --  BulkCoefL82 computes a Monin-Obukhov length (:545-550) and BetaW
 *      that DSFCM_Util_SfcBulkFlux_Get never returns; they are not computed.
 * Slot 3 of SfcHFlx_ns / SfcHFlx_sr / DSfcHFlxDTs is left untouched, as
 * in the reference (the final loop runs n = 1..2 only).
 */
#include <math.h>
#include "oracle.h"

/* Constants, sfc/DSFCM_Util_SfcBulkFlux_mod.f90:35-58. */
#define FKarm 0.4
#define GasRUniv 8.3144621
#define StB 5.670373e-8
#define Grav 9.8
#define MolWtDry 1.8e-2
#define MolWtWet 1.8e-2
#define CpDry 1616.0
#define LatentHeat 2425300.0
#define LatentHeatFusion 334000.0
#define RefPress 1e5
#define Es0 611.0
#define RoughLength 1e-4
#define RoughLenHeatFactor 1.0

/* read_config, :574-591. */
#define VelMinForRi 0.01
#define VelMinForVel 0.01
#define VelMinForTemp 0.01
#define VelMinForQVap 0.01
#define VelMaxForVel 1000.0
#define VelMaxForTemp 1000.0
#define VelMaxForQVap 1000.0
#define VelBulkCoefMin 0.0
#define TempBulkCoefMin 0.0
#define QVapBulkCoefMin 0.0
#define VelBulkCoefMax 1.0
#define TempBulkCoefMax 1.0
#define QVapBulkCoefMax 1.0

static inline double dmin(double a, double b) { return a < b ? a : b; }
static inline double dmax(double a, double b) { return a > b ? a : b; }

/* BulkCoefL82 for one column (:489-565, Monin-Obukhov length omitted). */
static void bulk_coef_l82(double Ri, double z0m, double z0h, double zs,
                          double z, double cmn, double chn, int flag,
                          double *cm, double *ch, double *cq) {
  double vm, th, qv;
  if (flag) {
    if (Ri > 0.0) {
      vm = cmn / (1.0 + 10.0 * Ri / sqrt(1.0 + 5.0 * Ri));
      th = chn / (1.0 + 15.0 * Ri * sqrt(1.0 + 5.0 * Ri));
      qv = th;
    } else {
      vm = cmn * (1.0 - 10.0 * Ri /
                            (1.0 + 75.0 * cmn * sqrt(-(z - zs + z0m) / z0m * Ri)));
      th = chn * (1.0 - 15.0 * Ri /
                            (1.0 + 75.0 * chn * sqrt(-(z - zs + z0h) / z0h * Ri)));
      qv = th;
    }
  } else {
    vm = 0.0;
    th = 0.0;
    qv = 0.0;
  }
  *cm = dmax(dmin(vm, VelBulkCoefMax), VelBulkCoefMin);
  *ch = dmax(dmin(th, TempBulkCoefMax), TempBulkCoefMin);
  *cq = dmax(dmin(qv, QVapBulkCoefMax), QVapBulkCoefMin);
}

void oracle_sfc_bulk_flux(double *const *a, int IA, int JA, int IS, int IE,
                          int JS, int JE) {
  const double GasRDry = GasRUniv / MolWtDry;
  const double GasRWet = GasRUniv / MolWtWet;
  const double EpsV = MolWtWet / MolWtDry;
  const double aL[2] = {LatentHeat, LatentHeat + LatentHeatFusion};
  const int64_t plane = (int64_t)IA * JA;
  const double sig1 = a[OF_Sig1Info][0];

#pragma omp parallel for collapse(2) schedule(static)
  for (int j = JS; j <= JE; ++j)
    for (int i = IS; i <= IE; ++i) {
      const int64_t c = (int64_t)(i - 1) + (int64_t)IA * (j - 1);
#define IN2(k) a[k][c]
#define A3(k, n) a[k][c + plane * ((n)-1)]
      const double SIceCon = IN2(OF_SIceCon);
      const double Ps = IN2(OF_SfcPress);
      const double Ta = IN2(OF_SfcAirTemp);
      const double q1 = IN2(OF_QVap1);
      const double U = IN2(OF_WindU), V = IN2(OF_WindV);
      const double zs = IN2(OF_SfcHeight);
      const double z0m = RoughLength;
      const double z0h = RoughLenHeatFactor * z0m;
      const double humd = 1.0; /* xya_SfcHumdCoef = 1 for all slots (:198) */

      /* :205-239 */
      double Frac[2], QVapSat[2], SfcVirTemp[2];
      Frac[0] = 1.0 - SIceCon;
      Frac[1] = SIceCon;
      for (int n = 1; n <= 2; ++n) {
        const double Ts = A3(OF_SfcTemp, n);
        QVapSat[n - 1] = EpsV * Es0 / Ps *
                         exp(aL[n - 1] / GasRWet * (1.0 / 273.0 - 1.0 / Ts));
        SfcVirTemp[n - 1] = Ts * (1.0 + (((1.0 / EpsV) - 1.0) * QVapSat[n - 1]));
      }
      const double VirTemp = Ta * (1.0 + (((1.0 / EpsV) - 1.0) * q1));
      const double Press1 = Ps * sig1;
      const double Exner = pow(Press1 / RefPress, GasRDry / CpDry);
      const double SfcExner = pow(Ps / RefPress, GasRDry / CpDry);
      const double VelAbs = sqrt(U * U + V * V);
      const double Height = zs + GasRDry / Grav * VirTemp * (1.0 - sig1);

      double WSX3 = 0.0, WSY3 = 0.0, Sen3 = 0.0, Lat3 = 0.0, QV3 = 0.0,
             SUw3 = 0.0, LUw3 = 0.0, Ts3 = 0.0, Alb3 = 0.0, CVel3 = 0.0,
             CTemp3 = 0.0, CQ3 = 0.0;

      double CVel[2], CTemp[2], CQ[2], WSX[2], WSY[2], Sen[2], QV[2], LatH[2],
          LUw[2], SUw[2];
      int flag[2];
      /* :244-348 */
      for (int n = 1; n <= 2; ++n) {
        const double tmp = (FKarm / log((Height - zs + z0m) / z0m));
        const double cmn = tmp * tmp;
        const double chn = tmp * (FKarm / log((Height - zs + z0h) / z0h));
        const double vmx = dmax(VelAbs, VelMinForRi);
        const double Ri = Grav / (SfcVirTemp[n - 1] / SfcExner) *
                          (VirTemp / Exner - SfcVirTemp[n - 1] / SfcExner) /
                          (vmx * vmx) * (Height - zs);
        const int f = (n == 1) ? 1 : (Frac[n - 1] > 1e-12);
        flag[n - 1] = f;
        double cm, ch, cq;
        bulk_coef_l82(Ri, z0m, z0h, zs, Height, cmn, chn, f, &cm, &ch, &cq);

        CVel[n - 1] = cm * Ps / (GasRDry * SfcVirTemp[n - 1]) *
                      dmin(dmax(VelAbs, VelMinForVel), VelMaxForVel);
        CTemp[n - 1] = ch * Ps / (GasRDry * SfcVirTemp[n - 1]) *
                       dmin(dmax(VelAbs, VelMinForTemp), VelMaxForTemp);
        CQ[n - 1] = cq * Ps / (GasRDry * SfcVirTemp[n - 1]) *
                    dmin(dmax(VelAbs, VelMinForQVap), VelMaxForQVap);

        const double Ts = A3(OF_SfcTemp, n);
        const double alb = A3(OF_SfcAlbedo, n);
        if (f) {
          WSX[n - 1] = -CVel[n - 1] * U;
          WSY[n - 1] = -CVel[n - 1] * V;
          Sen[n - 1] = -CpDry * SfcExner * CTemp[n - 1] * (Ta / Exner - Ts / SfcExner);
          QV[n - 1] = -humd * CQ[n - 1] * (q1 - QVapSat[n - 1]);
          LatH[n - 1] = aL[n - 1] * QV[n - 1];
          const double Ts2 = Ts * Ts;
          const double Ts4 = Ts2 * Ts2;
          LUw[n - 1] = StB * Ts4;
          SUw[n - 1] = alb * IN2(OF_SDwRFlx);

          Ts3 = Ts3 + Frac[n - 1] * Ts4;
          Alb3 = Alb3 + Frac[n - 1] * alb;
          WSX3 = WSX3 + Frac[n - 1] * WSX[n - 1];
          WSY3 = WSY3 + Frac[n - 1] * WSY[n - 1];
          Sen3 = Sen3 + Frac[n - 1] * Sen[n - 1];
          QV3 = QV3 + Frac[n - 1] * QV[n - 1];
          Lat3 = Lat3 + Frac[n - 1] * LatH[n - 1];
          LUw3 = LUw3 + Frac[n - 1] * LUw[n - 1];
          SUw3 = SUw3 + Frac[n - 1] * SUw[n - 1];
          CVel3 = CVel3 + Frac[n - 1] * CVel[n - 1];
          CTemp3 = CTemp3 + Frac[n - 1] * CTemp[n - 1];
          CQ3 = CQ3 + Frac[n - 1] * CQ[n - 1];
        } else {
          WSX[n - 1] = 0.0;
          WSY[n - 1] = 0.0;
          Sen[n - 1] = 0.0;
          QV[n - 1] = 0.0;
          LatH[n - 1] = 0.0;
          LUw[n - 1] = 0.0;
          SUw[n - 1] = 0.0;
        }
      }

      /* :355-382 implicit-coupling back-substitution */
      const double c1_1 = A3(OF_ImplCplCoef1, 1), c1_2 = A3(OF_ImplCplCoef1, 2),
                   c1_3 = A3(OF_ImplCplCoef1, 3), c1_4 = A3(OF_ImplCplCoef1, 4);
      const double c2_1 = A3(OF_ImplCplCoef2, 1), c2_2 = A3(OF_ImplCplCoef2, 2),
                   c2_3 = A3(OF_ImplCplCoef2, 3), c2_4 = A3(OF_ImplCplCoef2, 4);
      const double DFsDT1 = -CpDry * SfcExner * CTemp3 / Exner;
      const double g1 = 1.0 / (c1_1 + CVel3);
      const double g2 = 1.0 / (c1_2 + CVel3);
      const double g3 = 1.0 / (c1_3 - DFsDT1);
      const double g4 = 1.0 / (c1_4 + humd * CQ3);
      const double f1 = g1 * (WSX3 + c2_1);
      const double f2 = g2 * (WSY3 + c2_2);
      const double f3 = g3 * (Sen3 + c2_3);
      const double f4 = g4 * (QV3 + c2_4);
      A3(OF_DelVarImplCPL, 1) = f1;
      A3(OF_DelVarImplCPL, 2) = f2;
      A3(OF_DelVarImplCPL, 3) = f3;
      A3(OF_DelVarImplCPL, 4) = f4;

      double Lat3m = 0.0; /* D3: merged slot-3 latent heat flux */
      for (int n = 1; n <= 2; ++n) {
        WSX[n - 1] = WSX[n - 1] - CVel[n - 1] * f1;
        WSY[n - 1] = WSY[n - 1] - CVel[n - 1] * f2;
        Sen[n - 1] = Sen[n - 1] - CpDry * SfcExner / Exner * CTemp[n - 1] * f3;
        QV[n - 1] = QV[n - 1] - humd * CQ[n - 1] * f4;
        LatH[n - 1] = aL[n - 1] * QV[n - 1];
        if (flag[n - 1]) Lat3m = Lat3m + Frac[n - 1] * LatH[n - 1];
      }
      WSX3 = WSX3 - CVel3 * f1;
      WSY3 = WSY3 - CVel3 * f2;
      Sen3 = Sen3 - CpDry * SfcExner / Exner * CTemp3 * f3;
      QV3 = QV3 - humd * CQ3 * f4;
      (void)Lat3;
      Lat3 = Lat3m;

      /* :384-415 (serial meaning, D2) */
      for (int n = 1; n <= 2; ++n) {
        const int f = (n == 1) ? 1 : (Frac[n - 1] > 1e-12);
        const double Ts = A3(OF_SfcTemp, n);
        if (f) {
          A3(OF_SfcHFlx_ns, n) = +LUw[n - 1] - IN2(OF_LDwRFlx) + LatH[n - 1] + Sen[n - 1];
          A3(OF_SfcHFlx_sr, n) = SUw[n - 1] - IN2(OF_SDwRFlx);
          A3(OF_DSfcHFlxDTs, n) =
              +4.0 * StB * (Ts * Ts * Ts) + CpDry * CTemp[n - 1] +
              aL[n - 1] * humd * CQ[n - 1] *
                  (aL[n - 1] * QVapSat[n - 1] / (GasRWet * (Ts * Ts)));
        } else {
          A3(OF_SfcHFlx_ns, n) = 0.0;
          A3(OF_SfcHFlx_sr, n) = 0.0;
          A3(OF_DSfcHFlxDTs, n) = 0.0;
        }
      }

      for (int n = 1; n <= 2; ++n) {
        A3(OF_WindStressX, n) = WSX[n - 1];
        A3(OF_WindStressY, n) = WSY[n - 1];
        A3(OF_SenHFlx, n) = Sen[n - 1];
        A3(OF_QVapMFlx, n) = QV[n - 1];
        A3(OF_LatHFlx, n) = LatH[n - 1];
        A3(OF_SfcVelTransCoef, n) = CVel[n - 1];
        A3(OF_SfcTempTransCoef, n) = CTemp[n - 1];
        A3(OF_SfcQVapTransCoef, n) = CQ[n - 1];
        A3(OF_SUwRFlx, n) = SUw[n - 1];
        A3(OF_LUwRFlx, n) = LUw[n - 1];
      }
      A3(OF_WindStressX, 3) = WSX3;
      A3(OF_WindStressY, 3) = WSY3;
      A3(OF_SenHFlx, 3) = Sen3;
      A3(OF_QVapMFlx, 3) = QV3;
      A3(OF_LatHFlx, 3) = Lat3;
      A3(OF_SfcVelTransCoef, 3) = CVel3;
      A3(OF_SfcTempTransCoef, 3) = CTemp3;
      A3(OF_SfcQVapTransCoef, 3) = CQ3;
      A3(OF_SUwRFlx, 3) = SUw3;
      A3(OF_LUwRFlx, 3) = LUw3;
      A3(OF_SfcTemp, 3) = Ts3;
      A3(OF_SfcAlbedo, 3) = Alb3;
#undef IN2
#undef A3
    }
}
