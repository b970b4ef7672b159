/*
 * Oracle (test infrastructure): Jones-99 first/second-order remap table
 * generator, table reader and COO apply, restated from
 *   common/grid_mapping_util_jones99.f90:35-442 (generator),
 *   common/grid_mapping_util_jones99.f90:446-506 (reader),
 *   common/interpolation_data_latlon_mod.f90:274-306 (apply).
 *
 * PARITY UNPINNED (the Fortran reference cannot be compiled here; see oracle.h).
 *
 * Reference behaviour kept on purpose (mode 0, "REF"):
 *  - the longitude weight of every source column in the overlap range is
 *    2*pi/NXD whatever the true overlap (:325-332, :347-350);
 *  - search_OverwrapRange (:384-440) resets only SrcRangeX(1) and
 *    SrcRangeY(2); SrcRangeX(2) and SrcRangeY(1) keep the value of the
 *    previous call when no source cell matches (intent(out) dummies that
 *    the reference does not assign).  The first call has no previous value:
 *    a table that would need one is reported as an error (-2);
 *  - X1 is not checked: an unmatched left edge leaves SrcRangeX(1) = -1 and
 *    the row is written with source index <= 0 (:402, :433);
 *  - the |w| > 1e-14 filter (:245, :262).
 * Mode 1 ("CONSERVE") is this project's conservative variant: the same
 * latitude segments, but each source column's longitude weight is its true
 * periodic overlap with the destination cell, so row sums are 1 and
 * area-weighted integrals are conserved whatever NXS and NXD are.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define UNSET (-2147483647)

typedef struct {
  int nx, ny;  /* interior sizes */
  double *x;   /* centres with halo, 1-based: x[1..nx+2] */
  double *u;   /* edges u[1..nx+1] (u[i] = east edge of cell i, i=IS-1..IE) */
  double *y;   /* centres, 1-based y[2..ny+1] */
  double *v;   /* edges v[1..ny+1] */
} halo_grid;

static const double PI_ = 3.141592653589793238462643383279502884;

/* gen_gridmapfile_lonlat2lonlat + calc_edge_coordinate (:78-152). */
static void make_grid(halo_grid *g, const double *lon, int nx, const double *lat,
                      int ny, const double *latwt) {
  const double PI = acos(-1.0);
  const int IA = nx + 2, IS = 2, IE = IA - 1;
  const int JA = ny + 2, JS = 2, JE = JA - 1;
  g->nx = nx;
  g->ny = ny;
  g->x = (double *)calloc((size_t)IA + 2, sizeof(double));
  g->u = (double *)calloc((size_t)IA + 2, sizeof(double));
  g->y = (double *)calloc((size_t)JA + 2, sizeof(double));
  g->v = (double *)calloc((size_t)JA + 2, sizeof(double));
  for (int i = IS; i <= IE; ++i) g->x[i] = lon[i - IS];
  for (int j = JS; j <= JE; ++j) g->y[j] = lat[j - JS];
  g->x[IS - 1] = g->x[IE] - 2.0 * PI;
  g->x[IE + 1] = g->x[IS] + 2.0 * PI;
  for (int i = IS - 1; i <= IE; ++i) g->u[i] = 0.5 * (g->x[i] + g->x[i + 1]);
  g->v[JS - 1] = -PI / 2.0;
  for (int j = JS; j <= JE - 1; ++j)
    g->v[j] = asin(latwt[j - JS] + sin(g->v[j - 1]));
  g->v[JE] = PI / 2.0;
}

static void free_grid(halo_grid *g) {
  free(g->x);
  free(g->u);
  free(g->y);
  free(g->v);
}

/* Row emitter with capacity check. */
typedef struct {
  int64_t n, cap;
  int32_t *iD, *jD, *iS, *jS;
  double *w;
} rows_t;

static void emit(rows_t *r, int iD, int jD, int iS, int jS, double w) {
  if (r->n < r->cap) {
    r->iD[r->n] = iD;
    r->jD[r->n] = jD;
    r->iS[r->n] = iS;
    r->jS[r->n] = jS;
    r->w[r->n] = w;
  }
  r->n++;
}

/* Periodic overlap length of [a1,a2] with [b1,b2] (mode 1 only). */
static double lon_overlap(double a1, double a2, double b1, double b2) {
  double tot = 0.0;
  for (int s = -1; s <= 1; ++s) {
    const double sh = 2.0 * PI_ * s;
    const double lo = a1 > b1 + sh ? a1 : b1 + sh;
    const double hi = a2 < b2 + sh ? a2 : b2 + sh;
    if (hi > lo) tot += hi - lo;
  }
  return tot;
}

int oracle_j99_gen(const double *lonS, int nxs, const double *latS, int nys,
                   const double *lonD, int nxd, const double *latD, int nyd,
                   const double *latwtS, const double *latwtD, int order,
                   int mode, int64_t cap, int32_t *oiD, int32_t *ojD,
                   int32_t *oiS, int32_t *ojS, double *ow, int64_t *nrow) {
  const double PI = acos(-1.0);
  halo_grid S, D;
  make_grid(&S, lonS, nxs, latS, nys, latwtS);
  make_grid(&D, lonD, nxd, latD, nyd, latwtD);
  const int ISS = 2, IES = nxs + 1, JSS = 2, JES = nys + 1;
  const int ISD = 2, IED = nxd + 1, JSD = 2, JED = nyd + 1;
  const int NXD = IED - ISD + 1, NXS = IES - ISS + 1, NYS = JES - JSS + 1;
  rows_t R = {0, cap, oiD, ojD, oiS, ojS, ow};
  int rx[2] = {UNSET, UNSET}, ry[2] = {UNSET, UNSET};
  int status = 0;
  double *seg = (double *)malloc(sizeof(double) * ((size_t)NYS + 2));
  double *ovl = (double *)malloc(sizeof(double) * ((size_t)NXS + 2));
  int *ovi = (int *)malloc(sizeof(int) * ((size_t)NXS + 2));

  for (int jD = JSD; jD <= JED && status == 0; ++jD) {
    for (int iD = ISD; iD <= IED; ++iD) {
      const double DX1 = D.u[iD - 1], DX2 = D.u[iD];
      const double DY1 = D.v[jD - 1], DY2 = D.v[jD];
      /* search_OverwrapRange, :402-438 */
      rx[0] = -1;
      ry[1] = -1;
      if (NXS == 1 && NXD != 1) {
        rx[0] = ISS;
        rx[1] = ISS;
      } else if (NXS != 1 && NXD == 1) {
        rx[0] = ISS;
        rx[1] = IES;
      } else {
        for (int i = ISS; i <= IES; ++i) {
          if (S.u[i - 1] <= DX1 && DX1 <= S.u[i]) rx[0] = i;
          if (S.u[i - 1] <= DX2 && DX2 <= S.u[i]) {
            rx[1] = i;
            break;
          }
        }
      }
      for (int j = JSS; j <= JES; ++j) {
        if (S.v[j - 1] <= DY1 && DY1 <= S.v[j]) ry[0] = j;
        if (S.v[j - 1] <= DY2 && DY2 <= S.v[j]) {
          ry[1] = j;
          break;
        }
      }
      if (ry[0] == UNSET || rx[1] == UNSET) { /* value the reference never set */
        status = -2;
        break;
      }
      if (ry[0] < 0 || ry[1] < 0) { /* the reference stops (:433-438) */
        status = -1;
        break;
      }

      /* calc_RemappingWeight, :314-365 */
      const int NXr = rx[1] - rx[0] + 1;
      const int NYr = ry[1] - ry[0] + 1;
      if ((mode == 0 && NXr <= 0) || NYr <= 0) continue;
      double DLon_k = 2.0 * PI / (double)NXD, DLon_nk, DLon_n;
      if (NXD == 1) {
        DLon_nk = 2.0 * PI / (double)NXS;
        DLon_n = DLon_nk;
      } else {
        DLon_nk = 2.0 * PI / (double)NXD;
        DLon_n = 2.0 * PI;
      }
      seg[0] = D.v[jD - 1];
      for (int j = 1; j <= NYr - 1; ++j) seg[j] = S.v[ry[0] + j - 1];
      seg[NYr] = D.v[jD];
      const double lat1_k = D.v[jD - 1], lat2_k = D.v[jD];

      if (mode == 0) {
        const double Ak = (sin(lat2_k) - sin(lat1_k)) * DLon_k;
        for (int m = 1; m <= NXr; ++m) {
          const int iS = rx[0] + m - 1;
          for (int n = 1; n <= NYr; ++n) {
            const int jS = ry[0] + n - 1;
            const double w1 = DLon_nk * (sin(seg[n]) - sin(seg[n - 1])) / Ak;
            if (fabs(w1) > 1e-14)
              emit(&R, iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, jS - JSS + 1, w1);
            if (order > 1) {
              /* :253-267 second-order terms */
              const double lat1_nk = seg[n - 1], lat2_nk = seg[n];
              const double lat1_n = S.v[ry[0] + n - 2], lat2_n = S.v[ry[0] + n - 1];
              const double An = (sin(lat2_n) - sin(lat1_n)) * DLon_n;
              const double w2 =
                  ((cos(lat2_nk) + lat2_nk * sin(lat2_nk)) -
                   (cos(lat1_nk) + lat1_nk * sin(lat1_nk))) * DLon_nk / Ak -
                  ((cos(lat2_n) + lat2_n * sin(lat2_n)) -
                   (cos(lat1_n) + lat1_n * sin(lat1_n))) * DLon_n * w1 / An;
              int j1, j2;
              if (jS == JSS) {
                j1 = jS;
                j2 = jS + 1;
              } else if (jS == JES) {
                j1 = jS - 1;
                j2 = jS;
              } else {
                j1 = jS - 1;
                j2 = jS + 1;
              }
              const double DLat = S.y[j2] - S.y[j1];
              if (fabs(w2) > 1e-14) {
                emit(&R, iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, j1 - JSS + 1, -w2 / DLat);
                emit(&R, iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, j2 - JSS + 1, +w2 / DLat);
              }
            }
          }
        }
      } else {
        /* Conservative variant: true periodic longitude overlaps, ascending
         * source index; latitude segments as above. */
        const double dlon_k = DX2 - DX1;
        const double Ak = (sin(lat2_k) - sin(lat1_k)) * dlon_k;
        int nov = 0;
        if (NXS == 1) {
          ovi[0] = ISS;
          ovl[0] = dlon_k;
          nov = 1;
        } else {
          for (int i = ISS; i <= IES; ++i) {
            const double o = lon_overlap(DX1, DX2, S.u[i - 1], S.u[i]);
            if (o > 0.0) {
              ovi[nov] = i;
              ovl[nov] = o;
              nov++;
            }
          }
        }
        for (int m = 0; m < nov; ++m) {
          for (int n = 1; n <= NYr; ++n) {
            const int jS = ry[0] + n - 1;
            const double w1 = ovl[m] * (sin(seg[n]) - sin(seg[n - 1])) / Ak;
            if (fabs(w1) > 1e-14)
              emit(&R, iD - ISD + 1, jD - JSD + 1, ovi[m] - ISS + 1, jS - JSS + 1, w1);
          }
        }
      }
    }
  }
  free(seg);
  free(ovl);
  free(ovi);
  free_grid(&S);
  free_grid(&D);
  *nrow = R.n;
  if (status) return status;
  return R.n > cap ? 1 : 0;
}

/* set_mappingTable_interpCoef, :496-501. */
void oracle_table_to_index(int64_t n, const int32_t *iD, const int32_t *jD,
                           const int32_t *iS, const int32_t *jS, int GNXS,
                           int GNXR, int32_t *send_index, int32_t *recv_index) {
  for (int64_t k = 0; k < n; ++k) {
    recv_index[k] = iD[k] + GNXR * (jD[k] - 1);
    send_index[k] = iS[k] + GNXS * (jS[k] - 1);
  }
}

/* interpolate_data_latlon, :293-302. */
int oracle_remap_apply(int64_t nop, const int32_t *send_index,
                       const int32_t *recv_index, const double *coef,
                       int64_t sn1, const double *send, int64_t rn1,
                       double *recv, int num_of_data) {
  for (int64_t k = 0; k < nop; ++k)
    if (send_index[k] < 1 || send_index[k] > sn1 || recv_index[k] < 1 ||
        recv_index[k] > rn1)
      return -1;
  memset(recv, 0, sizeof(double) * (size_t)rn1 * (size_t)num_of_data);
#pragma omp parallel for schedule(static)
  for (int d = 0; d < num_of_data; ++d) {
    const double *s = send + (int64_t)d * sn1;
    double *r = recv + (int64_t)d * rn1;
    for (int64_t k = 0; k < nop; ++k) {
      const int64_t sp = send_index[k] - 1, rp = recv_index[k] - 1;
      r[rp] = r[rp] + s[sp] * coef[k];
    }
  }
  return 0;
}

/* Neumaier compensated sum of f*area (global area integral). */
double oracle_area_integral(int64_t n, const double *f, const double *area) {
  double s = 0.0, c = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double x = f[i] * area[i];
    const double t = s + x;
    if (fabs(s) >= fabs(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  return s + c;
}
