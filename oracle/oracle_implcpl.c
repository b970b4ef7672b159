/*
 * Oracle (test infrastructure): implicit surface coupling of the vertical
 * diffusion, a plain-C FP64 restatement of
 *   SfcImplicitCoupling_VDiffForward   atm/dcpam_sfc_implicit_coupling_mod.f90:72-378
 *   Solve_TriDiagSystem_Forward        :380-405
 *   SfcImplicitCoupling_VDiffBackward  :25-70
 *   Solve_TriDiagSystem_Backward       :407-420
 * with every expression evaluated in the reference's order (Fortran
 * left-to-right for * and /, unary minus over the whole product), so that
 * with -ffp-contract=off the results are the reference's bit for bit.
 *
 * Layout (Fortran column-major, columns (i,j) flattened to c < ncol):
 *   half levels  x[c + ncol*k],  k = 0..kmax         (xyr_*)
 *   full levels  x[c + ncol*(k-1)], k = 1..kmax      (xyz_*)
 *   tracers      x[c + ncol*(k + (kmax+1)*(n-1))] / x[c + ncol*((k-1) + kmax*(n-1))]
 *   matrices     m[c + ncol*((k-1) + kmax*(d+1))],  d = -1, 0, 1   (xyza_*Mtx)
 *   coefficients x[c + ncol*(a-1)], a = 1..4         (xya_ImplCplCoef1/2)
 * The three matrices (UV, Temp, QMix) are the module state the backward
 * sweep reads.  Level 1 of the eliminated systems divides by the zero
 * sub-diagonal the reference sets at k = 1 (:199, :237, :272); the coupler
 * overwrites U, V, T and the vapour tracer at level 1 before the backward
 * sweep (atm/dccm_atm_mod.f90:832-835).  The IEEE results (infinities or
 * NaN) are reproduced as they come.
 */
#include <stddef.h>

#include "oracle.h"

#define H(a, k) a[c + ncol * (size_t)(k)]             /* half level k = 0..kmax */
#define F(a, k) a[c + ncol * (size_t)((k) - 1)]       /* full level k = 1..kmax */
#define MX(m, k, d) m[c + ncol * (size_t)(((k) - 1) + kmax * ((d) + 1))]

/* Solve_TriDiagSystem_Forward (:380-405): elimination from the top. */
static void solve_forward(double *m, double *rhs, size_t c, size_t ncol, int kmax) {
  int k = kmax;
  MX(m, k, 0) = MX(m, k, 0) / MX(m, k, -1);
  F(rhs, k) = F(rhs, k) / MX(m, k, -1);
  MX(m, k, -1) = 1.0;
  for (k = kmax - 1; k >= 1; --k) {
    MX(m, k, 0) = (MX(m, k, 0) * MX(m, k + 1, 0) - MX(m, k, 1)) / (MX(m, k, -1) * MX(m, k + 1, 0));
    F(rhs, k) = (F(rhs, k) * MX(m, k + 1, 0) - MX(m, k, 1) * F(rhs, k + 1)) / (MX(m, k, -1) * MX(m, k + 1, 0));
    MX(m, k, -1) = 1.0;
    MX(m, k, 1) = 0.0;
  }
}

/* Solve_TriDiagSystem_Backward (:407-420). */
static void solve_backward(const double *m, double *rhs, size_t c, size_t ncol, int kmax) {
  for (int k = 2; k <= kmax; ++k) F(rhs, k) = (F(rhs, k) - MX(m, k, -1) * F(rhs, k - 1)) / MX(m, k, 0);
}

void oracle_implcpl_forward(const double *const *in, double *const *out, double *uv, double *tm,
                            double *qm, int64_t ncol_, int kmax, int ncmax, int ih2o,
                            const double *consts) {
  const double *MomFluxX = in[OI_MomFluxX], *MomFluxY = in[OI_MomFluxY], *HeatFlux = in[OI_HeatFlux];
  const double *QMixFlux = in[OI_QMixFlux], *Press = in[OI_Press], *ExnerF = in[OI_ExnerFull];
  const double *ExnerH = in[OI_ExnerHalf], *VirTemp = in[OI_VirTemp], *Height = in[OI_Height];
  const double *VelDiff = in[OI_VelDiffCoef], *TempDiff = in[OI_TempDiffCoef];
  const double *QMixDiff = in[OI_QMixDiffCoef];
  double *DUDt = out[OO_DUDt], *DVDt = out[OO_DVDt], *DTempDt = out[OO_DTempDt];
  double *DQMixDt = out[OO_DQMixDt], *C1 = out[OO_ImplCplCoef1], *C2 = out[OO_ImplCplCoef2];
  const double Grav = consts[0], CpDry = consts[1], GasRDry = consts[2], DelTime = consts[3];
  const size_t ncol = (size_t)ncol_;
  const size_t lvl = ncol * (size_t)kmax;
#pragma omp parallel
  {
    double VTC[kmax + 1], TTC[kmax + 1], QTC[kmax + 1];
    double qsave[3 * kmax];
#pragma omp for schedule(static)
    for (size_t c = 0; c < ncol; ++c) {
      VTC[0] = VTC[kmax] = TTC[0] = TTC[kmax] = QTC[0] = QTC[kmax] = 0.0;
      for (int k = 1; k <= kmax - 1; ++k) {  // :188-195
        const double tmp = H(Press, k) / (GasRDry * H(VirTemp, k)) / (F(Height, k + 1) - F(Height, k));
        VTC[k] = H(VelDiff, k) * tmp;
        TTC[k] = H(TempDiff, k) * tmp;
        QTC[k] = H(QMixDiff, k) * tmp;
      }
      // UV matrix :199-221
      for (int k = 1; k <= kmax; ++k) {
        const double mass = -((H(Press, k) - H(Press, k - 1)) / Grav / (2.0 * DelTime));
        MX(uv, k, -1) = k == 1 ? 0.0 : -VTC[k - 1];
        if (k == 1) MX(uv, k, 0) = mass + VTC[k];
        else if (k < kmax) MX(uv, k, 0) = mass + VTC[k - 1] + VTC[k];
        else MX(uv, k, 0) = mass + VTC[k - 1];
        MX(uv, k, 1) = k == kmax ? 0.0 : -VTC[k];
      }
      // Temp matrix :225-256
      for (int k = 1; k <= kmax; ++k) {
        const double mass = -(CpDry * (H(Press, k) - H(Press, k - 1)) / Grav / (2.0 * DelTime));
        MX(tm, k, -1) = k == 1 ? 0.0 : -(CpDry * H(ExnerH, k - 1) / F(ExnerF, k - 1) * TTC[k - 1]);
        if (k == 1) MX(tm, k, 0) = mass + CpDry * H(ExnerH, k) / F(ExnerF, k) * TTC[k];
        else if (k < kmax)
          MX(tm, k, 0) = mass + CpDry * H(ExnerH, k - 1) / F(ExnerF, k) * TTC[k - 1] +
                         CpDry * H(ExnerH, k) / F(ExnerF, k) * TTC[k];
        else MX(tm, k, 0) = mass + CpDry * H(ExnerH, k - 1) / F(ExnerF, k) * TTC[k - 1];
        MX(tm, k, 1) = k == kmax ? 0.0 : -(CpDry * H(ExnerH, k) / F(ExnerF, k + 1) * TTC[k]);
      }
      // QMix matrix :260-291
      for (int k = 1; k <= kmax; ++k) {
        const double mass = -((H(Press, k) - H(Press, k - 1)) / Grav / (2.0 * DelTime));
        MX(qm, k, -1) = k == 1 ? 0.0 : -QTC[k - 1];
        if (k == 1) MX(qm, k, 0) = mass + QTC[k];
        else if (k < kmax) MX(qm, k, 0) = mass + QTC[k - 1] + QTC[k];
        else MX(qm, k, 0) = mass + QTC[k - 1];
        MX(qm, k, 1) = k == kmax ? 0.0 : -QTC[k];
      }
      // right-hand sides :295-308
      for (int k = 1; k <= kmax; ++k) {
        F(DUDt, k) = -(H(MomFluxX, k) - H(MomFluxX, k - 1));
        F(DVDt, k) = -(H(MomFluxY, k) - H(MomFluxY, k - 1));
        F(DTempDt, k) = -(H(HeatFlux, k) - H(HeatFlux, k - 1));
      }
      for (int n = 1; n <= ncmax; ++n)
        for (int k = 1; k <= kmax; ++k) {
          const size_t hk = c + ncol * (size_t)(k + (kmax + 1) * (n - 1));
          const size_t hk1 = c + ncol * (size_t)(k - 1 + (kmax + 1) * (n - 1));
          DQMixDt[c + ncol * (size_t)((k - 1) + kmax * (n - 1))] = -(QMixFlux[hk] - QMixFlux[hk1]);
        }
      C2[c + ncol * 0] = F(DUDt, 1);  // :310-313
      C2[c + ncol * 1] = F(DVDt, 1);
      C2[c + ncol * 2] = F(DTempDt, 1);
      C2[c + ncol * 3] = DQMixDt[c + ncol * (size_t)(kmax * (ih2o - 1))];
      // :322-331 (the V system uses a saved copy of the UV matrix: the same
      // elimination; the QMix system is reset from its copy for each tracer)
      double uvsave[3 * kmax];
      for (int d = -1; d <= 1; ++d)
        for (int k = 1; k <= kmax; ++k) uvsave[(k - 1) + kmax * (d + 1)] = MX(uv, k, d);
      solve_forward(uv, DUDt, c, ncol, kmax);
      {
        // the V solve on the saved copy: put the copy in place temporarily
        double uvdone[3 * kmax];
        for (int d = -1; d <= 1; ++d)
          for (int k = 1; k <= kmax; ++k) {
            uvdone[(k - 1) + kmax * (d + 1)] = MX(uv, k, d);
            MX(uv, k, d) = uvsave[(k - 1) + kmax * (d + 1)];
          }
        solve_forward(uv, DVDt, c, ncol, kmax);
        for (int d = -1; d <= 1; ++d)
          for (int k = 1; k <= kmax; ++k) MX(uv, k, d) = uvdone[(k - 1) + kmax * (d + 1)];
      }
      solve_forward(tm, DTempDt, c, ncol, kmax);
      for (int d = -1; d <= 1; ++d)
        for (int k = 1; k <= kmax; ++k) qsave[(k - 1) + kmax * (d + 1)] = MX(qm, k, d);
      for (int n = 1; n <= ncmax; ++n) {
        for (int d = -1; d <= 1; ++d)
          for (int k = 1; k <= kmax; ++k) MX(qm, k, d) = qsave[(k - 1) + kmax * (d + 1)];
        solve_forward(qm, DQMixDt + lvl * (size_t)(n - 1), c, ncol, kmax);
      }
      // :342-375
      const double Tmp = -((H(Press, 1) - H(Press, 0)) / Grav / (2.0 * DelTime));
      const double DFADUV1 = VTC[1], DFADUV2 = -VTC[1];
      C1[c + ncol * 0] = Tmp + DFADUV1 - DFADUV2 / MX(uv, 2, 0);
      C2[c + ncol * 0] = C2[c + ncol * 0] - DFADUV2 * F(DUDt, 2) / MX(uv, 2, 0);
      C1[c + ncol * 1] = Tmp + DFADUV1 - DFADUV2 / MX(uv, 2, 0);
      C2[c + ncol * 1] = C2[c + ncol * 1] - DFADUV2 * F(DVDt, 2) / MX(uv, 2, 0);
      const double DFADT1 = CpDry * H(ExnerH, 1) * TTC[1] / F(ExnerF, 1);
      const double DFADT2 = -(CpDry * H(ExnerH, 1) * TTC[1] / F(ExnerF, 2));
      C1[c + ncol * 2] = CpDry * Tmp + DFADT1 - DFADT2 / MX(tm, 2, 0);
      C2[c + ncol * 2] = C2[c + ncol * 2] - DFADT2 * F(DTempDt, 2) / MX(tm, 2, 0);
      const double DFADQ1 = QTC[1], DFADQ2 = -QTC[1];
      C1[c + ncol * 3] = Tmp + DFADQ1 - DFADQ2 / MX(qm, 2, 0);
      C2[c + ncol * 3] = C2[c + ncol * 3] -
                         DFADQ2 * DQMixDt[c + ncol * (size_t)(1 + kmax * (ih2o - 1))] / MX(qm, 2, 0);
    }
  }
}

void oracle_implcpl_backward(const double *uv, const double *tm, const double *qm, double *DUDt,
                             double *DVDt, double *DTempDt, double *DQMixDt, int64_t ncol_, int kmax,
                             int ncmax, double DelTime) {
  const size_t ncol = (size_t)ncol_;
  const size_t lvl = ncol * (size_t)kmax;
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < ncol; ++c) {
    solve_backward(uv, DUDt, c, ncol, kmax);  // :48-56
    solve_backward(uv, DVDt, c, ncol, kmax);
    solve_backward(tm, DTempDt, c, ncol, kmax);
    for (int k = 1; k <= kmax; ++k) {
      F(DUDt, k) = F(DUDt, k) / (2.0 * DelTime);
      F(DVDt, k) = F(DVDt, k) / (2.0 * DelTime);
      F(DTempDt, k) = F(DTempDt, k) / (2.0 * DelTime);
    }
    for (int n = 1; n <= ncmax; ++n) {  // :58-61
      double *q = DQMixDt + lvl * (size_t)(n - 1);
      solve_backward(qm, q, c, ncol, kmax);
      for (int k = 1; k <= kmax; ++k) F(q, k) = F(q, k) / (2.0 * DelTime);
    }
  }
}
