// Longitude FFT of the plain FP64 path: self-sorting Stockham radix-4/3/2
// in shared memory, one warp per pair of latitude rows.
//
// On GB300 the FP64 pipe is the limit of this path, so it uses the
// transform with the fewest FP64 operations per point: radix-4 stages
// (multiplications by +-i are swaps) with table twiddles, about half the
// multiplications of the register/shuffle factorisation that the FP32 path
// uses (fft.cu).  Rows pair up as in fft.cu (z = g(jn) + i g(js)), and the
// data layouts (F[m][j][c] in, G[m][p][jj][c] out) are the same.
#include "sht_plan.cuh"

namespace dccm {
namespace sht {
namespace f64 {

constexpr int MAX_STAGES = 12;

struct Radix {
  int I, nst;
  int r[MAX_STAGES];
};

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmuli(double2 a, int s) { return make_double2(-a.y * s, a.x * s); }

// Stockham autosort FFT of one complex row by one warp.  sign = -1 forward,
// +1 inverse (unnormalised).  Returns the buffer holding the result.
__device__ double2 *warp_stockham(double2 *x, double2 *y, const double2 *__restrict__ tw, const Radix &a,
                                  int sign, int lane) {
  const int I = a.I;
  int Ns = 1;
  for (int st = 0; st < a.nst; ++st) {
    const int R = a.r[st];
    const int nb = I / R;
    const int tstep = I / (Ns * R);
    for (int j = lane; j < nb; j += 32) {
      const int k = j % Ns;
      const int base = (j / Ns) * Ns * R + k;
      double2 v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (r < R) {
          double2 t = x[j + r * nb];
          if (r > 0 && k > 0) {
            double2 w = tw[k * r * tstep];
            if (sign > 0) w.y = -w.y;
            t = cmul(t, w);
          }
          v[r] = t;
        }
      if (R == 4) {
        const double2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
        const double2 s1 = cadd(v[1], v[3]), d1 = cmuli(csub(v[1], v[3]), sign);
        y[base] = cadd(s0, s1);
        y[base + Ns] = cadd(d0, d1);
        y[base + 2 * Ns] = csub(s0, s1);
        y[base + 3 * Ns] = csub(d0, d1);
      } else if (R == 2) {
        y[base] = cadd(v[0], v[1]);
        y[base + Ns] = csub(v[0], v[1]);
      } else {  // R == 3
        const double2 t1 = cadd(v[1], v[2]);
        const double2 t2 = cmuli(csub(v[1], v[2]), sign);
        const double h = 0.86602540378443864676;  // sqrt(3)/2
        const double2 m = make_double2(v[0].x - 0.5 * t1.x, v[0].y - 0.5 * t1.y);
        const double2 q = make_double2(t2.x * h, t2.y * h);
        y[base] = cadd(v[0], t1);
        y[base + Ns] = cadd(m, q);
        y[base + 2 * Ns] = csub(m, q);
      }
    }
    __syncwarp();
    double2 *t = x;
    x = y;
    y = t;
    Ns *= R;
  }
  return x;
}

__global__ void __launch_bounds__(512)
fft64_inverse_kernel(Radix a, int N, int J, int batch, int BB, const double *__restrict__ F,
                     double *__restrict__ grid, const double2 *__restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int I = a.I, Jh = J / 2;
  const int jj = blockIdx.x;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = blockIdx.y * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  double *stA = reinterpret_cast<double *>(smem_raw);
  double *stB = stA + (size_t)(N + 1) * cw;
  double2 *tw = reinterpret_cast<double2 *>(stB + (size_t)(N + 1) * cw);
  double2 *bufs = tw + I;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = twg[t];
  for (int t = threadIdx.x; t < (N + 1) * cw; t += blockDim.x) {
    const int m = t / cw, c = t % cw;
    double va = 0, vb = 0;
    if (c < 2 * nb) {
      va = F[((int64_t)m * J + jn) * C2B + 2LL * b0 + c];
      vb = F[((int64_t)m * J + js) * C2B + 2LL * b0 + c];
    }
    stA[t] = va;
    stB[t] = vb;
  }
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nw = blockDim.x / 32;
  double2 *x = bufs + (size_t)warp * 2 * I;
  double2 *y = x + I;
  for (int bl = warp; bl < nb; bl += nw) {
    for (int k = lane; k < I; k += 32) x[k] = make_double2(0.0, 0.0);
    __syncwarp();
    for (int m = lane; m <= N; m += 32) {
      const double ar = stA[m * cw + 2 * bl], ai = m ? stA[m * cw + 2 * bl + 1] : 0.0;
      const double br = stB[m * cw + 2 * bl], bi = m ? stB[m * cw + 2 * bl + 1] : 0.0;
      x[m] = make_double2(ar - bi, ai + br);
      if (m > 0) x[I - m] = make_double2(ar + bi, br - ai);
    }
    __syncwarp();
    double2 *z = warp_stockham(x, y, tw, a, +1, lane);
    double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
    for (int i = lane; i < I; i += 32) {
      gn[i] = z[i].x;
      gs[i] = z[i].y;
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(512)
fft64_forward_kernel(Radix a, int N, int J, int batch, int BB, const double *__restrict__ grid,
                     double *__restrict__ G, const double2 *__restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int I = a.I, Jh = J / 2;
  const int jj = blockIdx.x;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = blockIdx.y * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  double *stE = reinterpret_cast<double *>(smem_raw);
  double *stO = stE + (size_t)(N + 1) * cw;
  double2 *tw = reinterpret_cast<double2 *>(stO + (size_t)(N + 1) * cw);
  double2 *bufs = tw + I;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = twg[t];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nw = blockDim.x / 32;
  double2 *x = bufs + (size_t)warp * 2 * I;
  double2 *y = x + I;
  const double invI = 1.0 / (double)I;
  for (int bl = warp; bl < nb; bl += nw) {
    const double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    const double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
    for (int i = lane; i < I; i += 32) x[i] = make_double2(gn[i], gs[i]);
    __syncwarp();
    double2 *Z = warp_stockham(x, y, tw, a, -1, lane);
    for (int m = lane; m <= N; m += 32) {
      const double2 zm = Z[m], zc = Z[(I - m) % I];
      const double ar = 0.5 * (zm.x + zc.x), ai = 0.5 * (zm.y - zc.y);
      const double br = 0.5 * (zm.y + zc.y), bi = -0.5 * (zm.x - zc.x);
      stE[m * cw + 2 * bl] = (ar + br) * invI;
      stE[m * cw + 2 * bl + 1] = m ? (ai + bi) * invI : 0.0;
      stO[m * cw + 2 * bl] = (ar - br) * invI;
      stO[m * cw + 2 * bl + 1] = m ? (ai - bi) * invI : 0.0;
    }
    __syncwarp();
  }
  __syncthreads();
  for (int t = threadIdx.x; t < (N + 1) * cw; t += blockDim.x) {
    const int m = t / cw, c = t % cw;
    if (c < 2 * nb) {
      G[(((int64_t)m * 2 + 0) * Jh + jj) * C2B + 2LL * b0 + c] = stE[t];
      G[(((int64_t)m * 2 + 1) * Jh + jj) * C2B + 2LL * b0 + c] = stO[t];
    }
  }
}

static bool radix_plan(int I, Radix &a) {
  a.I = I;
  a.nst = 0;
  int n = I;
  while (n % 4 == 0 && a.nst < MAX_STAGES) { a.r[a.nst++] = 4; n /= 4; }
  while (n % 2 == 0 && a.nst < MAX_STAGES) { a.r[a.nst++] = 2; n /= 2; }
  while (n % 3 == 0 && a.nst < MAX_STAGES) { a.r[a.nst++] = 3; n /= 3; }
  return n == 1;
}

static int pick_bb(const Plan &P, int batch, size_t *smem) {
  const size_t budget = 160 * 1024;
  int BB = 16;
  auto need = [&](int bb) {
    return (size_t)(P.N + 1) * 2 * bb * 2 * sizeof(double) + (size_t)P.I * sizeof(double2) * (1 + 2 * (size_t)bb);
  };
  while (BB > 1 && need(BB) > budget) BB /= 2;
  if (BB > batch) BB = batch < 1 ? 1 : batch;
  *smem = need(BB);
  return BB;
}

}  // namespace f64

int fft_inverse_f64(const Plan &P, int batch, const double *F, double *grid, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  f64::Radix a;
  if (!f64::radix_plan(P.I, a)) return DCCM_ERR_UNSUPPORTED;
  size_t smem;
  const int BB = f64::pick_bb(P, batch, &smem);
  DCCM_CUDA(cudaFuncSetAttribute(f64::fft64_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  f64::fft64_inverse_kernel<<<dim3(P.Jh, (batch + BB - 1) / BB), 32 * BB, smem, s>>>(a, P.N, P.J, batch, BB, F,
                                                                                     grid, P.d_tw64);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int fft_forward_f64(const Plan &P, int batch, const double *grid, double *G, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  f64::Radix a;
  if (!f64::radix_plan(P.I, a)) return DCCM_ERR_UNSUPPORTED;
  size_t smem;
  const int BB = f64::pick_bb(P, batch, &smem);
  DCCM_CUDA(cudaFuncSetAttribute(f64::fft64_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  f64::fft64_forward_kernel<<<dim3(P.Jh, (batch + BB - 1) / BB), 32 * BB, smem, s>>>(a, P.N, P.J, batch, BB, grid,
                                                                                     G, P.d_tw64);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

}  // namespace sht
}  // namespace dccm
