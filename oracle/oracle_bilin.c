/*
 * Oracle (test infrastructure): bilinear remap table and the surface
 * exchange grid, plain-C FP64 restatements of
 *   gen_gridmapfile_lonlat2lonlat      common/grid_mapping_util.f90:32-182
 *     (get_correspondID_latS :130-150, cal_coef :152-163,
 *      cal_coef_axisym :165-174)
 *   generate_surface_exchage_grid      tool/gmapgen/gmapgen_main.f90:336-405
 *     (sort :407-425)
 * Rows are (iR, jR, iS, jS, w), 1-based, in the order the reference writes
 * them.  One place is given a meaning: for a destination latitude north of
 * the last source latitude on a grid that is not axisymmetric, cal_coef
 * reads y_LatS(nys+1), past the end of the array (undefined).  There the
 * rows extrapolate linearly from the last two source latitudes, as the
 * reference does at the south edge (where latR <= y_LatS(1) uses rows 1
 * and 2 with a negative weight).  A single source latitude in that branch
 * has no such pair and returns -1.
 */
#include <math.h>
#include <stdlib.h>

#include "oracle.h"

/* get_correspondID_latS (:130-150): first j with y(j) < latR <= y(j+1). */
static int corresp_lat(double latR, const double *y, int nys, int *extp) {
  for (int j = 1; j <= nys - 1; ++j)
    if (y[j - 1] < latR && latR <= y[j]) {
      *extp = 0;
      return j;
    }
  *extp = 1;
  int id = 0;  // unassigned in the reference if neither test holds (NaN input)
  if (latR <= y[0]) id = 1;
  if (latR > y[nys - 1]) id = nys;
  return id;
}

int oracle_bilin_gen(const double *lonS, int nxs, const double *latS, int nys, const double *lonR, int nxr,
                     const double *latR, int nyr, int64_t cap, int32_t *iR, int32_t *jR, int32_t *iS,
                     int32_t *jS, double *w, int64_t *nrow) {
  int64_t n = 0;
  const double dlon_r = 360.0 / (double)nxr;  // :74-75 (degrees)
  const double dlon_s = 360.0 / (double)nxs;
#define ROW(a, b, c, d, e)        \
  do {                            \
    if (n < cap) {                \
      iR[n] = (a);                \
      jR[n] = (b);                \
      iS[n] = (c);                \
      jS[n] = (d);                \
      w[n] = (e);                 \
    }                             \
    ++n;                          \
  } while (0)
  for (int jr = 1; jr <= nyr; ++jr) {
    int extp;
    const int js = corresp_lat(latR[jr - 1], latS, nys, &extp);
    if (js == 0) return -2;
    if (nxr == 1) {  // :84-95
      if (!extp) {
        const double b1 = (latR[jr - 1] - latS[js - 1]) / (latS[js] - latS[js - 1]);
        const double c1 = (1.0 - b1) / nxs, c2 = b1 / nxs;
        for (int is = 1; is <= nxs; ++is) {
          ROW(1, jr, is, js, c1);
          ROW(1, jr, is, js % nys + 1, c2);
        }
      } else {
        for (int is = 1; is <= nxs; ++is) ROW(1, jr, is, js, 1.0 / nxs);
      }
    } else if (nxs == 1) {  // :96-106
      if (!extp) {
        const double b1 = (latR[jr - 1] - latS[js - 1]) / (latS[js] - latS[js - 1]);
        const double c1 = 1.0 - b1, c2 = b1;
        for (int ir = 1; ir <= nxr; ++ir) {
          ROW(ir, jr, 1, js, c1);
          ROW(ir, jr, 1, js % nys + 1, c2);
        }
      } else {
        for (int ir = 1; ir <= nxr; ++ir) ROW(ir, jr, 1, js, 1.0);
      }
    } else {  // :108-125
      if (nys < 2) return -1;
      const int jb = (extp && js == nys) ? nys - 1 : js;  // see the header
      for (int ir = 1; ir <= nxr; ++ir) {
        const int is = (int)(dlon_r * (ir - 1) / dlon_s) + 1;
        const double xc = lonR[ir - 1], yc = latR[jr - 1];
        const double x1 = lonS[is - 1], y1 = latS[jb - 1];
        const double x3 = lonS[is % nxs], y3 = latS[jb];
        const double a1 = (xc - x1) / (x3 - x1), a2 = 1.0 - a1;
        const double b1 = (yc - y1) / (y3 - y1), b2 = 1.0 - b1;
        ROW(ir, jr, is, jb, a2 * b2);
        ROW(ir, jr, is % nxs + 1, jb, a1 * b2);
        ROW(ir, jr, is % nxs + 1, jb % nys + 1, a1 * b1);
        ROW(ir, jr, is, jb % nys + 1, a2 * b1);
      }
    }
  }
#undef ROW
  *nrow = n;
  return n > cap ? 1 : 0;
}

/* generate_surface_exchage_grid (:336-405), latitudes only (longitudes and
 * their weights are the atmosphere's).  latX must hold JMA + JMO entries. */
int oracle_exchange_grid_lat(const double *latA, const double *wA, int JMA, const double *latO,
                             const double *wO, int JMO, double *latX, double *wX) {
  if (JMA == JMO) {  // :352-357
    for (int j = 0; j < JMA; ++j) {
      latX[j] = latA[j];
      wX[j] = wA[j];
    }
    return JMA;
  }
  const double PI = acos(-1.0);
  const int JMS_ = JMO + JMA - 1;
  double *FJA = malloc(sizeof(double) * (JMA + 1)), *FJO = malloc(sizeof(double) * (JMO + 1));
  double *FJS = malloc(sizeof(double) * (JMS_ + 1));
  FJA[0] = -PI / 2.0;  // :361-365
  for (int j = 1; j <= JMA; ++j) FJA[j] = asin(wA[j - 1] + sin(FJA[j - 1]));
  FJA[JMA] = PI / 2.0;
  FJO[0] = -PI / 2.0;  // :367-371
  for (int j = 1; j <= JMO - 1; ++j) FJO[j] = asin(wO[j - 1] + sin(FJO[j - 1]));
  FJO[JMO] = PI / 2.0;
  for (int j = 0; j <= JMA - 1; ++j) FJS[j] = FJA[j];  // :373-374
  for (int j = 1; j <= JMO; ++j) FJS[JMA - 1 + j] = FJO[j];
  const int N = JMS_ + 1;  // sort (:407-425): exchange sort, ascending
  for (int i = 0; i < N - 1; ++i)
    for (int j = i + 1; j < N; ++j)
      if (FJS[i] > FJS[j]) {
        const double t = FJS[i];
        FJS[i] = FJS[j];
        FJS[j] = t;
      }
  (void)latO;
  int JMS = 0;  // :380-388
  for (int j = 1; j <= JMS_; ++j) {
    const double intWt = sin(FJS[j]) - sin(FJS[j - 1]);
    if (fabs(intWt) > 1e-12) {
      latX[JMS] = 0.5 * (FJS[j - 1] + FJS[j]);
      wX[JMS] = intWt;
      ++JMS;
    }
  }
  free(FJA);
  free(FJO);
  free(FJS);
  return JMS;
}
