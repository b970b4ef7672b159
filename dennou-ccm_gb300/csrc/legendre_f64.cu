// Plain FP64 Legendre transforms on the CUDA cores (the FP64 GPU path).
//
// Both directions are per-zonal-wavenumber dense contractions folded by
// equatorial symmetry, Pbar_n^m(-mu) = (-1)^(n+m) Pbar_n^m(mu):
//   inverse  E[jj][c] = sum_{n-m even} Pbar(m,n,jj) s_n^m[c],
//            O[jj][c] = sum_{n-m odd}  ...,  F(jn) = E + O,  F(js) = E - O;
//   forward  s_n^m[c] = sum_jj (w_jj/2) Pbar(m,n,jj) X_p[jj][c],
//            X_0 = E-fold, X_1 = O-fold of the Fourier coefficients.
// Each CTA computes a 64 x 64 output tile (4 x 4 per thread, FMA in FP64)
// from 16-deep slabs of both operands staged in shared memory.
#include "sht_plan.cuh"

namespace dccm {
namespace sht {

constexpr int TT = 64;  // output tile edge
constexpr int TK = 16;  // k slab depth

// grid: (N+1, ceil(2B/64), ceil(Jh/64)); block 256.
__global__ void __launch_bounds__(256)
leg_inv_f64(int N, int Jh, int batch, int64_t ncoef, const double *__restrict__ spec,
            const double *__restrict__ pnm, double *__restrict__ F) {
  const int m = blockIdx.x;
  const int c0 = blockIdx.y * TT, j0 = blockIdx.z * TT;
  const int C2B = 2 * batch, J = 2 * Jh;
  __shared__ double Ss[TK][TT];
  __shared__ double Ps[TK][TT];
  const int tc = threadIdx.x % 16, tj = threadIdx.x / 16;
  double acc[2][4][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[p][a][b] = 0.0;
  for (int p = 0; p < 2; ++p) {
    const int K = count_np(N, m, p);
    for (int k0 = 0; k0 < K; k0 += TK) {
      for (int t = threadIdx.x; t < TK * TT; t += blockDim.x) {
        const int kk = t / TT, cc = t % TT;
        const int k = k0 + kk, c = c0 + cc, jj = j0 + cc;
        double sv = 0.0, pv = 0.0;
        if (k < K) {
          const int n = m + p + 2 * k;
          const int64_t id = idx_mn(N, m, n);
          if (c < C2B) sv = spec[((int64_t)(c >> 1) * ncoef + id) * 2 + (c & 1)];
          if (jj < Jh) pv = pnm[id * Jh + jj];
        }
        Ss[kk][cc] = sv;
        Ps[kk][cc] = pv;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < TK; ++kk) {
        double sv[4], pv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) pv[a] = Ps[kk][tj * 4 + a];
#pragma unroll
        for (int b = 0; b < 4; ++b) sv[b] = Ss[kk][tc * 4 + b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[p][a][b] = fma(pv[a], sv[b], acc[p][a][b]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int jj = j0 + tj * 4 + a;
    if (jj >= Jh) continue;
    const int jn = Jh + jj, js = Jh - 1 - jj;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int c = c0 + tc * 4 + b;
      if (c >= C2B) continue;
      F[((int64_t)m * J + jn) * C2B + c] = acc[0][a][b] + acc[1][a][b];
      F[((int64_t)m * J + js) * C2B + c] = acc[0][a][b] - acc[1][a][b];
    }
  }
}

// grid: (N+1, ceil(2B/64), 2 * ceil(Kmax/64)) with z = ktile*2 + p; block 256.
__global__ void __launch_bounds__(256)
leg_fwd_f64(int N, int Jh, int batch, int64_t ncoef, const double *__restrict__ G,
            const double *__restrict__ pnm, const double *__restrict__ w,
            double *__restrict__ spec) {
  const int m = blockIdx.x;
  const int p = blockIdx.z & 1, kt = blockIdx.z >> 1;
  const int K = count_np(N, m, p);
  const int n0 = kt * TT;
  if (n0 >= K) return;
  const int c0 = blockIdx.y * TT;
  const int C2B = 2 * batch;
  __shared__ double Gs[TK][TT];
  __shared__ double Ps[TK][TT];
  const int tc = threadIdx.x % 16, tk = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  const double *Gp = G + ((int64_t)m * 2 + p) * Jh * C2B;
  for (int j0 = 0; j0 < Jh; j0 += TK) {
    for (int t = threadIdx.x; t < TK * TT; t += blockDim.x) {
      const int jl = t / TT, cc = t % TT;
      const int jj = j0 + jl, c = c0 + cc;
      Gs[jl][cc] = (jj < Jh && c < C2B) ? Gp[(int64_t)jj * C2B + c] : 0.0;
    }
    for (int t = threadIdx.x; t < TK * TT; t += blockDim.x) {
      const int kl = t / TK, jl = t % TK;  // jj fastest: coalesced table reads
      const int k = n0 + kl, jj = j0 + jl;
      double v = 0.0;
      if (k < K && jj < Jh) {
        const int n = m + p + 2 * k;
        v = (0.5 * w[Jh + jj]) * pnm[idx_mn(N, m, n) * Jh + jj];
      }
      Ps[jl][kl] = v;
    }
    __syncthreads();
#pragma unroll
    for (int jl = 0; jl < TK; ++jl) {
      double gv[4], pv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) pv[a] = Ps[jl][tk * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) gv[b] = Gs[jl][tc * 4 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(pv[a], gv[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int k = n0 + tk * 4 + a;
    if (k >= K) continue;
    const int n = m + p + 2 * k;
    const int64_t id = idx_mn(N, m, n);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int c = c0 + tc * 4 + b;
      if (c >= C2B) continue;
      spec[((int64_t)(c >> 1) * ncoef + id) * 2 + (c & 1)] = (m == 0 && (c & 1)) ? 0.0 : acc[a][b];
    }
  }
}

int legendre_inv_f64(const Plan &P, int batch, const double *spec, double *F, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  dim3 grd(P.N + 1, (2 * batch + TT - 1) / TT, (P.Jh + TT - 1) / TT);
  leg_inv_f64<<<grd, 256, 0, s>>>(P.N, P.Jh, batch, P.ncoef, spec, P.d_pnm, F);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int legendre_fwd_f64(const Plan &P, int batch, const double *G, double *spec, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  const int kmax = count_np(P.N, 0, 0);
  dim3 grd(P.N + 1, (2 * batch + TT - 1) / TT, 2 * ((kmax + TT - 1) / TT));
  leg_fwd_f64<<<grd, 256, 0, s>>>(P.N, P.Jh, batch, P.ncoef, G, P.d_pnm, P.d_w, spec);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

}  // namespace sht
}  // namespace dccm
