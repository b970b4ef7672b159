// Longitude FFT of the spherical-harmonic transform (FP32 for the mixed
// path, FP64 for the plain path).
//
// Two real latitude rows that mirror each other about the equator (jn, js)
// travel through one complex FFT of length I: z = g(jn) + i g(js).  One warp
// owns one field-level's pair of rows and runs a self-sorting Stockham FFT
// (radix 4, 3 and 2 stages; I = 64, 128, 192, 256, 512, 1024, ...) in its own
// two shared-memory buffers, synchronising with __syncwarp only.  Twiddles
// come from a table e^{-2 pi i t / I} evaluated in FP64 on the host.
//
// Inverse: the CTA stages the Fourier coefficients m = 0..N of its block of
// field-levels for rows jn and js (coalesced along c), each warp assembles
// the Hermitian spectrum of both rows into one complex array and transforms
// it; Re and Im of the result are the two grid rows.
// Forward: each warp loads its two rows, transforms, separates the two real
// spectra (A_m = (Z_m + conj Z_{I-m})/2, B_m = (Z_m - conj Z_{I-m})/(2i)),
// folds them into E = (A + B)/I and O = (A - B)/I, stages them, and the CTA
// writes G[m][p][jj][c] coalesced along c.
#include "fp_conv.cuh"
#include "sht_plan.cuh"

namespace dccm {
namespace sht {

template <typename T> struct Cx;
template <> struct Cx<float> { using t = float2; };
template <> struct Cx<double> { using t = double2; };

// Grid values are FP64 in memory; the FP32 transform converts on the integer pipes.
__device__ __forceinline__ float from_f64(double x, float) { return f64_to_f32_rn(x); }
__device__ __forceinline__ double from_f64(double x, double) { return x; }
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64(x); }
__device__ __forceinline__ double to_f64(double x) { return x; }

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) x, decltype(C::x) y) {
  C r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// multiply by i*s (s = +1 or -1)
template <typename C> __device__ __forceinline__ C cmuli(C a, int s) {
  C r;
  r.x = -a.y * s;
  r.y = a.x * s;
  return r;
}

struct FftArgs {
  int I, nst;
  int radix[MAX_STAGES];
};

// Stockham autosort FFT of one complex row by one warp.  sign = -1 forward,
// +1 inverse (unnormalised).  Returns the buffer holding the result.
template <typename C>
__device__ C *warp_fft(C *x, C *y, const C *__restrict__ tw, const FftArgs &a, int sign, int lane) {
  const int I = a.I;
  int Ns = 1;
  for (int st = 0; st < a.nst; ++st) {
    const int R = a.radix[st];
    const int nb = I / R;
    const int tstep = I / (Ns * R);
    for (int j = lane; j < nb; j += 32) {
      const int k = j % Ns;
      const int base = (j / Ns) * Ns * R + k;
      C v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (r < R) {
          C t = x[j + r * nb];
          if (r > 0 && k > 0) {
            C w = tw[k * r * tstep];
            if (sign > 0) w.y = -w.y;
            t = cmul(t, w);
          }
          v[r] = t;
        }
      if (R == 4) {
        const C s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
        const C s1 = cadd(v[1], v[3]), d1 = cmuli(csub(v[1], v[3]), sign);
        y[base] = cadd(s0, s1);
        y[base + Ns] = cadd(d0, d1);
        y[base + 2 * Ns] = csub(s0, s1);
        y[base + 3 * Ns] = csub(d0, d1);
      } else if (R == 2) {
        y[base] = cadd(v[0], v[1]);
        y[base + Ns] = csub(v[0], v[1]);
      } else {  // R == 3
        const C t1 = cadd(v[1], v[2]);
        const C t2 = cmuli(csub(v[1], v[2]), sign);
        using R_ = decltype(t1.x);
        const R_ h = (R_)0.86602540378443864676;  // sqrt(3)/2
        C m;
        m.x = v[0].x - (R_)0.5 * t1.x;
        m.y = v[0].y - (R_)0.5 * t1.y;
        C q;
        q.x = t2.x * h;
        q.y = t2.y * h;
        y[base] = cadd(v[0], t1);
        y[base + Ns] = cadd(m, q);
        y[base + 2 * Ns] = csub(m, q);
      }
    }
    __syncwarp();
    C *t = x;
    x = y;
    y = t;
    Ns *= R;
  }
  return x;
}

// ------------------------------------------------------------- inverse
template <typename T>
__global__ void __launch_bounds__(512)
fft_inverse_kernel(FftArgs a, int N, int J, int batch, int BB, const T *__restrict__ F,
                   double *__restrict__ grid, const typename Cx<T>::t *__restrict__ twg) {
  using C = typename Cx<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int I = a.I, Jh = J / 2;
  const int jj = blockIdx.x;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = blockIdx.y * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  T *stA = reinterpret_cast<T *>(smem_raw);      // [N+1][2BB] row jn
  T *stB = stA + (size_t)(N + 1) * cw;           // [N+1][2BB] row js
  C *tw = reinterpret_cast<C *>(stB + (size_t)(N + 1) * cw);
  C *bufs = tw + I;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = twg[t];
  for (int t = threadIdx.x; t < (N + 1) * cw; t += blockDim.x) {
    const int m = t / cw, c = t % cw;
    T va = 0, vb = 0;
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
  C *x = bufs + (size_t)warp * 2 * I;
  C *y = x + I;
  for (int bl = warp; bl < nb; bl += nw) {
    for (int k = lane; k < I; k += 32) x[k] = cmk<C>(0, 0);
    __syncwarp();
    for (int m = lane; m <= N; m += 32) {
      const T ar = stA[m * cw + 2 * bl], ai = m ? stA[m * cw + 2 * bl + 1] : (T)0;
      const T br = stB[m * cw + 2 * bl], bi = m ? stB[m * cw + 2 * bl + 1] : (T)0;
      x[m] = cmk<C>(ar - bi, ai + br);
      if (m > 0) x[I - m] = cmk<C>(ar + bi, br - ai);
    }
    __syncwarp();
    C *z = warp_fft<C>(x, y, tw, a, +1, lane);
    double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
    for (int i = lane; i < I; i += 32) {
      const C v = z[i];
      gn[i] = to_f64(v.x);
      gs[i] = to_f64(v.y);
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------- forward
template <typename T>
__global__ void __launch_bounds__(512)
fft_forward_kernel(FftArgs a, int N, int J, int batch, int BB, const double *__restrict__ grid,
                   T *__restrict__ G, const typename Cx<T>::t *__restrict__ twg) {
  using C = typename Cx<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int I = a.I, Jh = J / 2;
  const int jj = blockIdx.x;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = blockIdx.y * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  T *stE = reinterpret_cast<T *>(smem_raw);  // [N+1][2BB]
  T *stO = stE + (size_t)(N + 1) * cw;
  C *tw = reinterpret_cast<C *>(stO + (size_t)(N + 1) * cw);
  C *bufs = tw + I;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = twg[t];
  for (int t = threadIdx.x; t < (N + 1) * cw; t += blockDim.x) {
    stE[t] = 0;
    stO[t] = 0;
  }
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nw = blockDim.x / 32;
  C *x = bufs + (size_t)warp * 2 * I;
  C *y = x + I;
  const T invI = (T)(1.0 / (double)I);
  for (int bl = warp; bl < nb; bl += nw) {
    const double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    const double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
    for (int i = lane; i < I; i += 32) {
      C v;
      v.x = from_f64(gn[i], T());
      v.y = from_f64(gs[i], T());
      x[i] = v;
    }
    __syncwarp();
    C *Z = warp_fft<C>(x, y, tw, a, -1, lane);
    for (int m = lane; m <= N; m += 32) {
      const C zm = Z[m], zc = Z[(I - m) % I];
      // A = (Z_m + conj Z_{I-m})/2, B = (Z_m - conj Z_{I-m})/(2i)
      const T ar = (T)0.5 * (zm.x + zc.x), ai = (T)0.5 * (zm.y - zc.y);
      const T br = (T)0.5 * (zm.y + zc.y), bi = (T)-0.5 * (zm.x - zc.x);
      stE[m * cw + 2 * bl] = (ar + br) * invI;
      stE[m * cw + 2 * bl + 1] = m ? (ai + bi) * invI : (T)0;
      stO[m * cw + 2 * bl] = (ar - br) * invI;
      stO[m * cw + 2 * bl + 1] = m ? (ai - bi) * invI : (T)0;
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

template <typename T>
static int pick_bb(const Plan &P, int batch, size_t *smem, int *threads) {
  using C = typename Cx<T>::t;
  const size_t budget = 160 * 1024;
  int BB = 16;
  for (; BB > 1; BB /= 2) {
    const size_t st = (size_t)(P.N + 1) * 2 * BB * 2 * sizeof(T);
    const size_t bu = (size_t)P.I * sizeof(C) * (1 + 2 * (size_t)BB);
    if (st + bu <= budget) break;
  }
  if (BB > batch) BB = batch < 1 ? 1 : batch;
  *smem = (size_t)(P.N + 1) * 2 * BB * 2 * sizeof(T) + (size_t)P.I * sizeof(C) * (1 + 2 * (size_t)BB);
  *threads = 32 * BB;
  return BB;
}

static FftArgs fft_args(const Plan &P) {
  FftArgs a;
  a.I = P.fft.I;
  a.nst = P.fft.nst;
  for (int k = 0; k < MAX_STAGES; ++k) a.radix[k] = P.fft.radix[k];
  return a;
}

template <typename T>
static int launch_inv(const Plan &P, int batch, const void *F, double *grid, cudaStream_t s) {
  size_t smem;
  int threads;
  const int BB = pick_bb<T>(P, batch, &smem, &threads);
  DCCM_CUDA(cudaFuncSetAttribute(fft_inverse_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  dim3 grd(P.Jh, (batch + BB - 1) / BB);
  const void *tw = std::is_same<T, float>::value ? (const void *)P.d_tw32 : (const void *)P.d_tw64;
  fft_inverse_kernel<T><<<grd, threads, smem, s>>>(fft_args(P), P.N, P.J, batch, BB, (const T *)F, grid,
                                                   (const typename Cx<T>::t *)tw);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

template <typename T>
static int launch_fwd(const Plan &P, int batch, const double *grid, void *G, cudaStream_t s) {
  size_t smem;
  int threads;
  const int BB = pick_bb<T>(P, batch, &smem, &threads);
  DCCM_CUDA(cudaFuncSetAttribute(fft_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  dim3 grd(P.Jh, (batch + BB - 1) / BB);
  const void *tw = std::is_same<T, float>::value ? (const void *)P.d_tw32 : (const void *)P.d_tw64;
  fft_forward_kernel<T><<<grd, threads, smem, s>>>(fft_args(P), P.N, P.J, batch, BB, grid, (T *)G,
                                                   (const typename Cx<T>::t *)tw);
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int fft_inverse(const Plan &P, int batch, bool fp32, const void *F, double *grid, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  return fp32 ? launch_inv<float>(P, batch, F, grid, s) : launch_inv<double>(P, batch, F, grid, s);
}

int fft_forward(const Plan &P, int batch, bool fp32, const double *grid, void *G, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  return fp32 ? launch_fwd<float>(P, batch, grid, G, s) : launch_fwd<double>(P, batch, grid, G, s);
}

}  // namespace sht
}  // namespace dccm
