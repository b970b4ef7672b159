/* Oracle (test infrastructure): spectral-space operators, plain loops over
 * (m, n).  The reference applies ∇² and hyperdiffusion inside
 * DynamicsHSplVAS83 (atm/dcpam_main_mod.f90:2173-2180, external dcpam5
 * library, not in the source tree; HDOrder = 8 and the e-folding time of
 * the largest wavenumber: exp/APEI07Couple/common/dcpam/
 * dcpam_APEI07Couple_T21L16.conf:205-227).  With the code absent this is a
 * restatement of the mathematics: parity unpinned.
 *
 *   Laplacian          f_n = -n(n+1)/a^2
 *   inverse Laplacian  f_n = -a^2/(n(n+1)), f_0 = 0
 *   hyperdiffusion     D_n = nu (K_n - c), K_n = (n(n+1)/a^2)^(order/2),
 *                      c = K_1 (rotation correction) or 0, D_0 = 0,
 *                      nu = 1/(tau (K_N - c))
 *     tendency         f_n = -D_n;  implicit step  f_n = 1/(1 + dt D_n)
 */
#include "oracle.h"

static double kpow(double n, double a2, int p) {
  double r = 1.0;
  for (int i = 0; i < p; ++i) r *= n * (n + 1.0) / a2;
  return r;
}

int oracle_spec_apply(int N, int kind, double radius, int order, double efold_time, double dt,
                      int rotation_correction, int batch, const double *in, double *out) {
  if (N < 0 || radius <= 0.0 || kind < 0 || kind > 3) return -1;
  const double a2 = radius * radius;
  int p = 0;
  double nu = 0.0, c = 0.0;
  if (kind >= 2) {
    if (order < 2 || order % 2 || order > 32 || efold_time <= 0.0 || N < 2) return -1;
    p = order / 2;
    c = rotation_correction ? kpow(1.0, a2, p) : 0.0;
    nu = 1.0 / (efold_time * (kpow((double)N, a2, p) - c));
  }
  const long nc = (long)(N + 1) * (N + 2) / 2;
  for (int m = 0; m <= N; ++m)
    for (int n = m; n <= N; ++n) {
      const long k = (long)m * (N + 1) - (long)m * (m - 1) / 2 + (n - m);
      const double nn = (double)n * (double)(n + 1);
      double f;
      if (kind == 0) f = -nn / a2;
      else if (kind == 1) f = n == 0 ? 0.0 : -a2 / nn;
      else {
        double r = 1.0;
        for (int i = 0; i < p; ++i) r *= nn / a2;
        const double d = n == 0 ? 0.0 : nu * (r - c);
        f = kind == 2 ? -d : 1.0 / (1.0 + dt * d);
      }
      for (int b = 0; b < batch; ++b) {
        out[2 * (b * nc + k)] = f * in[2 * (b * nc + k)];
        out[2 * (b * nc + k) + 1] = f * in[2 * (b * nc + k) + 1];
      }
    }
  return 0;
}
