/*
 * Oracle (test infrastructure): FP64 spherical-harmonic transform pair on
 * the Gaussian grid, with Gauss-Legendre nodes by Newton iteration and the
 * normalised associated Legendre functions by the three-term recurrence.
 *
 * The reference does not contain this code: its atmosphere calls SPML
 * (w_module / wa_module over ISPACK), an external library that is not
 * vendored and whose version is not pinned (Mkinclude:15-21).  The call
 * sites are atm/dcpam_main_mod.f90:2173-2180 (dynamics through libdcpam5)
 * and tool/gmapgen/gmapgen_main.f90:262-305 (w_Initial, xy_Lon, xy_Lat,
 * x_Lon_Weight, y_Lat_Weight).  PARITY UNPINNED for this part: the oracle
 * restates the published mathematics and fixes its own convention:
 *
 *  - latitudes ascending south to north, mu_j = sin(lat_j) the roots of
 *    P_J, weights w_j with sum 2 (the reference's edge builder starts at
 *    -pi/2, common/grid_mapping_util_jones99.f90:147-151, and gmapgen
 *    prints sum(w) = 2, tool/gmapgen/gmapgen_main.f90:403);
 *  - longitudes lon_i = 2 pi i / I, i = 0..I-1;
 *  - Pbar_n^m normalised so that integral_{-1}^{1} Pbar^2 dmu = 2 (mean
 *    square 1 over the sphere for Pbar e^{i m lon}); no Condon-Shortley
 *    phase;  triangular truncation n <= N;
 *  - coefficients s_n^m complex, m = 0..N, n = m..N, stored m-major:
 *    idx(m,n) = m(N+1) - m(m-1)/2 + (n-m);
 *  - inverse:  g = Re F_0 + 2 Re sum_{m>=1} F_m e^{i m lon},
 *              F_m(mu) = sum_n s_n^m Pbar_n^m(mu);
 *  - forward:  G_m(mu_j) = (1/I) sum_i g_ij e^{-i m lon_i},
 *              s_n^m = (1/2) sum_j w_j Pbar_n^m(mu_j) G_m(mu_j).
 * The Legendre sums use the equatorial fold
 * Pbar_n^m(-mu) = (-1)^(n+m) Pbar_n^m(mu).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

static int g_threads = 0;
void oracle_set_threads(int n) {
  g_threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}
int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int64_t idx_mn(int N, int m, int n) {
  return (int64_t)m * (N + 1) - (int64_t)m * (m - 1) / 2 + (n - m);
}

/* Gauss-Legendre nodes (ascending) and weights by Newton iteration. */
void oracle_gauss_nodes(int J, double *mu, double *w) {
  const double PI = acos(-1.0);
  for (int k = 0; k < J / 2; ++k) {
    double x = cos(PI * (k + 0.75) / (J + 0.5));
    double dp = 0.0;
    int last = 0;
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
      if (last) break; /* one more step after |dx| <= 1e-15 |x| (quadratic convergence) */
      if (fabs(dx) <= 1e-15 * fabs(x)) last = 1;
    }
    {
      double p0 = 1.0, p1 = x;
      for (int l = 2; l <= J; ++l) {
        const double p2 = ((2.0 * l - 1.0) * x * p1 - (l - 1.0) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      dp = J * (x * p1 - p0) / (x * x - 1.0);
    }
    mu[J - 1 - k] = x;
    mu[k] = -x;
    w[J - 1 - k] = w[k] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
}

/* Normalised associated Legendre functions by recurrence in n. */
void oracle_pnm(int N, int J, const double *mu, double *p) {
  for (int j = 0; j < J; ++j) {
    const double x = mu[j];
    const double sx = sqrt((1.0 - x) * (1.0 + x));
    double pmm = 1.0;
    for (int m = 0; m <= N; ++m) {
      if (m > 0) pmm = pmm * sqrt((2.0 * m + 1.0) / (2.0 * m)) * sx;
      p[idx_mn(N, m, m) * J + j] = pmm;
      if (m + 1 <= N) {
        double pa = pmm, pb = sqrt(2.0 * m + 3.0) * x * pmm;
        p[idx_mn(N, m, m + 1) * J + j] = pb;
        for (int n = m + 2; n <= N; ++n) {
          const double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
          const double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) /
                                (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
          const double pc = a * (x * pb - b * pa);
          p[idx_mn(N, m, n) * J + j] = pc;
          pa = pb;
          pb = pc;
        }
      }
    }
  }
}

/* ------------------------------------------------------ mixed-radix FFT */
typedef struct {
  double re, im;
} cplx;

/* out[k] = sum_j x[j*xs] * exp(sign * 2 pi i j k / n); tw[t] = exp(-2 pi i t/I). */
static void dft_rec(int n, const cplx *x, int64_t xs, cplx *out, const cplx *tw,
                    int I, int sign) {
  if (n == 1) {
    out[0] = x[0];
    return;
  }
  int p;
  if (n % 4 == 0) p = 4;
  else if (n % 2 == 0) p = 2;
  else if (n % 3 == 0) p = 3;
  else if (n % 5 == 0) p = 5;
  else p = n;
  const int m = n / p;
  for (int r = 0; r < p; ++r) dft_rec(m, x + r * xs, xs * p, out + r * m, tw, I, sign);
  const int tstep = I / n;
  cplx t[p];
  for (int k = 0; k < m; ++k) {
    for (int r = 0; r < p; ++r) {
      const cplx a = out[r * m + k];
      const int64_t e = ((int64_t)r * k * tstep) % I;
      const double c = tw[e].re, s = sign < 0 ? tw[e].im : -tw[e].im;
      t[r].re = a.re * c - a.im * s;
      t[r].im = a.re * s + a.im * c;
    }
    for (int q = 0; q < p; ++q) {
      double sr = 0.0, si = 0.0;
      for (int r = 0; r < p; ++r) {
        const int64_t e = ((int64_t)r * q * (I / p)) % I;
        const double c = tw[e].re, s = sign < 0 ? tw[e].im : -tw[e].im;
        sr += t[r].re * c - t[r].im * s;
        si += t[r].re * s + t[r].im * c;
      }
      out[k + q * m].re = sr;
      out[k + q * m].im = si;
    }
  }
}

static cplx *make_twiddles(int I) {
  const double PI = acos(-1.0);
  cplx *tw = (cplx *)malloc(sizeof(cplx) * (size_t)I);
  for (int t = 0; t < I; ++t) {
    const double ang = 2.0 * PI * (double)t / (double)I;
    tw[t].re = cos(ang);
    tw[t].im = -sin(ang);
  }
  return tw;
}

void oracle_rfft_row(int I, const double *g, int M, double *out) {
  cplx *tw = make_twiddles(I);
  cplx *x = (cplx *)malloc(sizeof(cplx) * (size_t)I);
  cplx *y = (cplx *)malloc(sizeof(cplx) * (size_t)I);
  for (int i = 0; i < I; ++i) {
    x[i].re = g[i];
    x[i].im = 0.0;
  }
  dft_rec(I, x, 1, y, tw, I, -1);
  for (int m = 0; m < M; ++m) {
    out[2 * m] = y[m].re / I;
    out[2 * m + 1] = y[m].im / I;
  }
  free(tw);
  free(x);
  free(y);
}

/* Gauss nodes, weights and Pbar tables, computed once per (N, J) and kept
 * (as a transform library keeps them from its initialisation, SPML's
 * w_Initial).  Called outside parallel regions. */
typedef struct {
  int N, J;
  double *mu, *w, *p;
} tables_t;
static tables_t g_tab[8];
static int g_ntab = 0;

static void tables_for(int N, int J, const double **mu, const double **w, const double **p) {
  for (int k = 0; k < g_ntab; ++k)
    if (g_tab[k].N == N && g_tab[k].J == J) {
      *mu = g_tab[k].mu;
      *w = g_tab[k].w;
      *p = g_tab[k].p;
      return;
    }
  const int64_t ncoef = (int64_t)(N + 1) * (N + 2) / 2;
  tables_t t = {N, J, (double *)malloc(sizeof(double) * J), (double *)malloc(sizeof(double) * J),
                (double *)malloc(sizeof(double) * ncoef * J)};
  oracle_gauss_nodes(J, t.mu, t.w);
  oracle_pnm(N, J, t.mu, t.p);
  if (g_ntab == 8) { /* evict the oldest */
    free(g_tab[0].mu);
    free(g_tab[0].w);
    free(g_tab[0].p);
    for (int k = 1; k < 8; ++k) g_tab[k - 1] = g_tab[k];
    g_ntab = 7;
  }
  g_tab[g_ntab++] = t;
  *mu = t.mu;
  *w = t.w;
  *p = t.p;
}

/* ------------------------------------------------------------ transforms */
void oracle_sht_inverse(int N, int I, int J, int batch, const double *spec,
                        double *grid) {
  const int64_t ncoef = (int64_t)(N + 1) * (N + 2) / 2;
  const int Jh = J / 2;
  const double *mu, *w, *p;
  tables_for(N, J, &mu, &w, &p);
  (void)mu;
  cplx *tw = make_twiddles(I);
#pragma omp parallel
  {
    cplx *Z = (cplx *)malloc(sizeof(cplx) * (size_t)I);
    cplx *z = (cplx *)malloc(sizeof(cplx) * (size_t)I);
    cplx *Fn = (cplx *)malloc(sizeof(cplx) * (size_t)(N + 1));
    cplx *Fs = (cplx *)malloc(sizeof(cplx) * (size_t)(N + 1));
#pragma omp for collapse(2) schedule(static)
    for (int b = 0; b < batch; ++b)
      for (int jj = 0; jj < Jh; ++jj) {
        const double *s = spec + (int64_t)b * ncoef * 2;
        const int jn = J - 1 - jj, js = jj; /* northern row uses mu > 0 */
        for (int m = 0; m <= N; ++m) {
          double er = 0, ei = 0, orr = 0, oi = 0;
          for (int n = m; n <= N; ++n) {
            const int64_t c = idx_mn(N, m, n);
            const double pv = p[c * J + jn];
            if (((n - m) & 1) == 0) {
              er += s[2 * c] * pv;
              ei += s[2 * c + 1] * pv;
            } else {
              orr += s[2 * c] * pv;
              oi += s[2 * c + 1] * pv;
            }
          }
          Fn[m].re = er + orr;
          Fn[m].im = ei + oi;
          Fs[m].re = er - orr;
          Fs[m].im = ei - oi;
        }
        /* Two real rows through one complex inverse DFT:
         * Z_k = A_k + i B_k with A, B Hermitian spectra of rows jn, js. */
        for (int k = 0; k < I; ++k) Z[k].re = Z[k].im = 0.0;
        for (int m = 0; m <= N; ++m) {
          const double ar = m == 0 ? Fn[0].re : Fn[m].re, ai = m == 0 ? 0.0 : Fn[m].im;
          const double br = m == 0 ? Fs[0].re : Fs[m].re, bi = m == 0 ? 0.0 : Fs[m].im;
          Z[m].re += ar - bi;
          Z[m].im += ai + br;
          if (m > 0) { /* conj(A_m) + i conj(B_m) at I-m */
            Z[I - m].re += ar + bi;
            Z[I - m].im += -ai + br;
          }
        }
        dft_rec(I, Z, 1, z, tw, I, +1);
        double *gn = grid + ((int64_t)b * J + jn) * I;
        double *gs = grid + ((int64_t)b * J + js) * I;
        for (int i = 0; i < I; ++i) {
          gn[i] = z[i].re;
          gs[i] = z[i].im;
        }
      }
    free(Z);
    free(z);
    free(Fn);
    free(Fs);
  }
  free(tw);
}

void oracle_sht_forward(int N, int I, int J, int batch, const double *grid,
                        double *spec) {
  const int64_t ncoef = (int64_t)(N + 1) * (N + 2) / 2;
  const int Jh = J / 2;
  const double *mu, *w, *p;
  tables_for(N, J, &mu, &w, &p);
  (void)mu;
  cplx *tw = make_twiddles(I);
#pragma omp parallel
  {
    cplx *z = (cplx *)malloc(sizeof(cplx) * (size_t)I);
    cplx *Z = (cplx *)malloc(sizeof(cplx) * (size_t)I);
    /* E/O folded Fourier coefficients for all lat pairs: [Jh][N+1] */
    cplx *E = (cplx *)malloc(sizeof(cplx) * (size_t)Jh * (N + 1));
    cplx *O = (cplx *)malloc(sizeof(cplx) * (size_t)Jh * (N + 1));
#pragma omp for schedule(static)
    for (int b = 0; b < batch; ++b) {
      for (int jj = 0; jj < Jh; ++jj) {
        const int jn = J - 1 - jj, js = jj;
        const double *gn = grid + ((int64_t)b * J + jn) * I;
        const double *gs = grid + ((int64_t)b * J + js) * I;
        for (int i = 0; i < I; ++i) {
          z[i].re = gn[i];
          z[i].im = gs[i];
        }
        dft_rec(I, z, 1, Z, tw, I, -1);
        for (int m = 0; m <= N; ++m) {
          const cplx zm = Z[m];
          const cplx zc = Z[(I - m) % I];
          /* A = (Z_m + conj Z_{I-m})/2 (north), B = (Z_m - conj Z_{I-m})/(2i) */
          const double ar = 0.5 * (zm.re + zc.re), ai = 0.5 * (zm.im - zc.im);
          const double br = 0.5 * (zm.im + zc.im), bi = -0.5 * (zm.re - zc.re);
          E[(int64_t)jj * (N + 1) + m].re = (ar + br) / I;
          E[(int64_t)jj * (N + 1) + m].im = (ai + bi) / I;
          O[(int64_t)jj * (N + 1) + m].re = (ar - br) / I;
          O[(int64_t)jj * (N + 1) + m].im = (ai - bi) / I;
        }
      }
      double *s = spec + (int64_t)b * ncoef * 2;
      for (int m = 0; m <= N; ++m)
        for (int n = m; n <= N; ++n) {
          const int64_t c = idx_mn(N, m, n);
          const cplx *X = (((n - m) & 1) == 0) ? E : O;
          double sr = 0.0, si = 0.0;
          for (int jj = 0; jj < Jh; ++jj) {
            const int jn = J - 1 - jj;
            const double pw = 0.5 * w[jn] * p[c * J + jn];
            sr += pw * X[(int64_t)jj * (N + 1) + m].re;
            si += pw * X[(int64_t)jj * (N + 1) + m].im;
          }
          s[2 * c] = sr;
          s[2 * c + 1] = m == 0 ? 0.0 : si;
        }
    }
    free(z);
    free(Z);
    free(E);
    free(O);
  }
  free(tw);
}
