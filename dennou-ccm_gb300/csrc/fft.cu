// Longitude FFT of the spherical-harmonic transform, FP32 (mixed path), one
// warp per pair of latitude rows.  The plain FP64 path has its own
// transform in fft_f64.cu.
//
// Two real latitude rows that mirror each other about the equator (jn, js)
// travel through one complex FFT of length I = 32 R: z = g(jn) + i g(js).
// Lane l holds the R samples z[32 r + l] in registers, and the transform is
// the four-step factorisation I = R x 32:
//   forward  (1) length-R DFT over r in registers,
//            (2) twiddle e^{-2 pi i l k1 / I},
//            (3) length-32 radix-2 decimation-in-frequency across the lanes
//                with __shfl_xor; lane l ends with Z[k1 + R brev5(l)];
//   inverse  the same steps mirrored (decimation in time across lanes from
//            bit-reversed input, conjugate twiddles, register DFT last), so
//            lane l ends with z[32 r + l] and the row stores are coalesced.
// Rows are read and written straight from/to global memory (lanes along
// longitude); shared memory only stages the Fourier coefficients of the
// CTA's block of field-levels (coalesced along c) and, in the forward
// direction, the spectrum for separating the two real rows.  Twiddles come
// from a table e^{-2 pi i t / I} evaluated in FP64 on the host.  Supported
// lengths: R in {2, 3, 4, 6, 8, 12, 16, 24, 32}, i.e. I = 64 ... 1024.
//
// Inverse: Z_m = A_m + i B_m and Z_{I-m} = conj(A_m) + i conj(B_m) from the
// Fourier coefficients A (row jn) and B (row js); Re z and Im z are the rows.
// Forward: A_m = (Z_m + conj Z_{I-m})/2, B_m = (Z_m - conj Z_{I-m})/(2i),
// folded into E = (A + B)/I and O = (A - B)/I and written as G[m][p][jj][c].
#include <string.h>

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
// twiddle tw[t] = e^{-2 pi i t / I}; sign +1 uses its conjugate
template <typename C> __device__ __forceinline__ C twid(const C *tw, int t, int sign) {
  C w = tw[t];
  if (sign > 0) w.y = -w.y;
  return w;
}
template <typename C> __device__ __forceinline__ C shfl_xor_c(C v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

// In-register DFT of length R: v[k] <- sum_r v[r] e^{sign 2 pi i r k / R}.
// Even lengths split into two halves (decimation in time), 3 is direct.
template <int R> struct RegDft {
  template <typename C> __device__ __forceinline__ static void run(C *v, const C *tw, int I, int sign) {
    if constexpr (R == 1) {
      return;
    } else if constexpr (R == 2) {
      const C a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else if constexpr (R == 3) {
      using S = decltype(v[0].x);
      const C t1 = cadd(v[1], v[2]);
      const C d = csub(v[1], v[2]);
      const S h = (S)0.86602540378443864676 * (S)sign;  // sign * sqrt(3)/2
      C mm, q;
      mm.x = v[0].x - (S)0.5 * t1.x;
      mm.y = v[0].y - (S)0.5 * t1.y;
      q.x = -d.y * h;  // i * sign * sqrt(3)/2 * d
      q.y = d.x * h;
      v[0] = cadd(v[0], t1);
      v[1] = cadd(mm, q);
      v[2] = csub(mm, q);
    } else {
      static_assert(R % 2 == 0, "length");
      constexpr int H = R / 2;
      C e[H], o[H];
#pragma unroll
      for (int i = 0; i < H; ++i) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
      }
      RegDft<H>::run(e, tw, I, sign);
      RegDft<H>::run(o, tw, I, sign);
#pragma unroll
      for (int k = 0; k < H; ++k) {
        const C t = k == 0 ? o[0] : cmul(o[k], twid(tw, k * (I / R), sign));
        v[k] = cadd(e[k], t);
        v[k + H] = csub(e[k], t);
      }
    }
  }
};

// Forward complex FFT of one row held as v[r] = z[32 r + lane];
// on return v[k1] = Z[k1 + R brev5(lane)].
template <int R, typename C>
__device__ __forceinline__ void warp_fft_fwd(C (&v)[R], const C *tw, int lane) {
  constexpr int I = 32 * R;
  RegDft<R>::run(v, tw, I, -1);
#pragma unroll
  for (int k = 1; k < R; ++k)
    if (lane) v[k] = cmul(v[k], twid(tw, lane * k, -1));
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool upper = lane & h;
    const C w = twid(tw, (lane & (h - 1)) * (I / (2 * h)), -1);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const C p = shfl_xor_c(v[k], h);
      v[k] = upper ? cmul(csub(p, v[k]), w) : cadd(v[k], p);
    }
  }
}

// Inverse (unnormalised) FFT of one row held as v[k1] = Z[k1 + R brev5(lane)];
// on return v[r] = z[32 r + lane].
template <int R, typename C>
__device__ __forceinline__ void warp_fft_inv(C (&v)[R], const C *tw, int lane) {
  constexpr int I = 32 * R;
#pragma unroll
  for (int h = 1; h <= 16; h <<= 1) {
    const bool upper = lane & h;
    const C w = twid(tw, (lane & (h - 1)) * (I / (2 * h)), +1);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const C p = shfl_xor_c(v[k], h);
      // top = a + w b, bottom = a - w b, with a the lower lane's value
      v[k] = upper ? csub(p, cmul(v[k], w)) : cadd(v[k], cmul(p, w));
    }
  }
#pragma unroll
  for (int k = 1; k < R; ++k)
    if (lane) v[k] = cmul(v[k], twid(tw, lane * k, +1));
  RegDft<R>::run(v, tw, I, +1);
}

// ------------------------------------------------------------- inverse
// One CTA: latitude pair jj, field-levels [by*BB, by*BB + BB).
template <typename T, int R>
__device__ __forceinline__ void fft_inv_block(int N, int J, int batch, int BB, const T *__restrict__ F,
                                              double *__restrict__ grid, const typename Cx<T>::t *__restrict__ twg,
                                              int jj, int by, unsigned char *smem_raw) {
  using C = typename Cx<T>::t;
  constexpr int I = 32 * R;
  const int Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  C *tw = reinterpret_cast<C *>(smem_raw);
  T *stA = reinterpret_cast<T *>(tw + I);  // [N+1][2BB] row jn
  T *stB = stA + (size_t)(N + 1) * cw;     // [N+1][2BB] row js
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
  const int k2 = brev5(lane);
  for (int bl = warp; bl < nb; bl += nw) {
    C v[R];
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
      const int k = k1 + R * k2;
      C z = cmk<C>(0, 0);
      if (k <= N) {
        const T ar = stA[k * cw + 2 * bl], ai = k ? stA[k * cw + 2 * bl + 1] : (T)0;
        const T br = stB[k * cw + 2 * bl], bi = k ? stB[k * cw + 2 * bl + 1] : (T)0;
        z = cmk<C>(ar - bi, ai + br);
      } else if (k >= I - N) {
        const int m = I - k;
        const T ar = stA[m * cw + 2 * bl], ai = stA[m * cw + 2 * bl + 1];
        const T br = stB[m * cw + 2 * bl], bi = stB[m * cw + 2 * bl + 1];
        z = cmk<C>(ar + bi, br - ai);
      }
      v[k1] = z;
    }
    warp_fft_inv<R>(v, tw, lane);
    double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      gn[32 * r + lane] = to_f64(v[r].x);
      gs[32 * r + lane] = to_f64(v[r].y);
    }
  }
}

// ------------------------------------------------------------- forward
template <typename T, int R>
__device__ __forceinline__ void fft_fwd_block(int N, int J, int batch, int BB, const double *__restrict__ grid,
                                              T *__restrict__ G, const typename Cx<T>::t *__restrict__ twg,
                                              int jj, int by, unsigned char *smem_raw) {
  using C = typename Cx<T>::t;
  constexpr int I = 32 * R;
  const int Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * BB;
  const int nb = min(BB, batch - b0);
  const int64_t C2B = 2LL * batch;
  const int cw = 2 * BB;
  const int nw = blockDim.x / 32;
  C *tw = reinterpret_cast<C *>(smem_raw);
  C *zb = tw + I;                                        // [nw][I] spectra
  T *stE = reinterpret_cast<T *>(zb + (size_t)nw * I);  // [N+1][2BB]
  T *stO = stE + (size_t)(N + 1) * cw;
  for (int t = threadIdx.x; t < I; t += blockDim.x) tw[t] = twg[t];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  C *Z = zb + (size_t)warp * I;
  const int k2 = brev5(lane);
  const T invI = (T)1 / (T)I;
  for (int bl = warp; bl < nb; bl += nw) {
    const double *gn = grid + ((int64_t)(b0 + bl) * J + jn) * I;
    const double *gs = grid + ((int64_t)(b0 + bl) * J + js) * I;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r].x = from_f64(gn[32 * r + lane], T());
      v[r].y = from_f64(gs[32 * r + lane], T());
    }
    warp_fft_fwd<R>(v, tw, lane);
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) Z[k1 + R * k2] = v[k1];
    __syncwarp();
    for (int m = lane; m <= N; m += 32) {
      const C zm = Z[m], zc = Z[(I - m) % I];
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

// ------------------------------------------------------------- kernels
// Several truncation groups in one launch: CTA blockIdx.x belongs to the
// group whose block range contains it; the group's length selects the
// register FFT (cases up to RMAX are compiled in).
constexpr int FFT_MAXG = 8;
struct FftGroup {
  int N, J, batch, BB, R, blk0;
  const void *in;
  void *out;
  const void *tw;
};
struct FftLaunch {
  FftGroup g[FFT_MAXG];
  int ngroups;
};

template <typename T, int R, int RMAX, bool FWD>
__device__ __forceinline__ void dispatch_case(const FftGroup &G, int jj, int by, unsigned char *sm) {
  if constexpr (R <= RMAX) {
    using C = typename Cx<T>::t;
    if (FWD)
      fft_fwd_block<T, R>(G.N, G.J, G.batch, G.BB, (const double *)G.in, (T *)G.out, (const C *)G.tw, jj, by, sm);
    else
      fft_inv_block<T, R>(G.N, G.J, G.batch, G.BB, (const T *)G.in, (double *)G.out, (const C *)G.tw, jj, by, sm);
  }
}

template <typename T, int RMAX, bool FWD>
__global__ void __launch_bounds__(256) fft_multi_kernel(const __grid_constant__ FftLaunch L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int gi = 0;
  while (gi + 1 < L.ngroups && (int)blockIdx.x >= L.g[gi + 1].blk0) ++gi;
  const FftGroup &G = L.g[gi];
  const int lb = blockIdx.x - G.blk0;
  const int Jh = G.J / 2;
  const int jj = lb % Jh, by = lb / Jh;
  switch (G.R) {
    case 2: dispatch_case<T, 2, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 3: dispatch_case<T, 3, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 4: dispatch_case<T, 4, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 6: dispatch_case<T, 6, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 8: dispatch_case<T, 8, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 12: dispatch_case<T, 12, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 16: dispatch_case<T, 16, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 24: dispatch_case<T, 24, RMAX, FWD>(G, jj, by, smem_raw); break;
    case 32: dispatch_case<T, 32, RMAX, FWD>(G, jj, by, smem_raw); break;
    default: break;
  }
}

// Field-levels per CTA (one warp each) that fit a shared-memory budget.
static size_t fft_smem(int N, int I, int bb, bool fwd) {
  size_t s = (size_t)I * sizeof(float2) + (size_t)(N + 1) * 2 * bb * 2 * sizeof(float);
  if (fwd) s += (size_t)bb * I * sizeof(float2);
  return s;
}

// One launch over ngroups plans (FP32).  in/out per group as in the single case.
int fft_multi(Plan *const *plans, const int *batch, const void *const *in, void *const *out, int ngroups, bool fwd,
              cudaStream_t s) {
  if (ngroups < 1 || ngroups > FFT_MAXG) return DCCM_ERR_UNSUPPORTED;
  const size_t budget = 96 * 1024;
  int BB = tunables().fft_bb > 0 && tunables().fft_bb <= 8 ? tunables().fft_bb : 8, rmax = 2;
  for (int g = 0; g < ngroups; ++g) {
    if (!fft_length_supported(plans[g]->I)) return DCCM_ERR_UNSUPPORTED;
    rmax = plans[g]->I / 32 > rmax ? plans[g]->I / 32 : rmax;
    while (BB > 1 && fft_smem(plans[g]->N, plans[g]->I, BB, fwd) > budget) BB /= 2;
  }
  FftLaunch L;
  memset(&L, 0, sizeof L);
  int nblk = 0, ng = 0;
  size_t smem = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (batch[g] <= 0) continue;
    const Plan &P = *plans[g];
    FftGroup &G = L.g[ng++];
    G.N = P.N;
    G.J = P.J;
    G.batch = batch[g];
    G.BB = BB;
    G.R = P.I / 32;
    G.blk0 = nblk;
    G.in = in[g];
    G.out = out[g];
    G.tw = P.d_tw32;
    nblk += P.Jh * ((batch[g] + BB - 1) / BB);
    const size_t sm = fft_smem(P.N, P.I, BB, fwd);
    smem = sm > smem ? sm : smem;
  }
  L.ngroups = ng;
  if (nblk == 0) return DCCM_OK;
  auto go = [&](auto kernel) -> int {
    DCCM_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<nblk, 32 * BB, smem, s>>>(L);
    DCCM_LAUNCH_CHECK();
    return DCCM_OK;
  };
  if (rmax <= 8) return fwd ? go(fft_multi_kernel<float, 8, true>) : go(fft_multi_kernel<float, 8, false>);
  return fwd ? go(fft_multi_kernel<float, 32, true>) : go(fft_multi_kernel<float, 32, false>);
}

bool fft_length_supported(int I) {
  if (I % 32 != 0) return false;
  switch (I / 32) {
    case 2: case 3: case 4: case 6: case 8: case 12: case 16: case 24: case 32: return true;
    default: return false;
  }
}

// The FP64 path uses the shared-memory Stockham transform (fft_f64.cu),
// which needs fewer FP64 operations than the register/shuffle one.
int fft_inverse(const Plan &P, int batch, bool fp32, const void *F, double *grid, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  if (!fp32) return fft_inverse_f64(P, batch, (const double *)F, grid, s);
  Plan *pp = const_cast<Plan *>(&P);
  void *out = grid;
  return fft_multi(&pp, &batch, &F, &out, 1, false, s);
}

int fft_forward(const Plan &P, int batch, bool fp32, const double *grid, void *G, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  if (!fp32) return fft_forward_f64(P, batch, grid, (double *)G, s);
  Plan *pp = const_cast<Plan *>(&P);
  const void *in = grid;
  return fft_multi(&pp, &batch, &in, &G, 1, true, s);
}

}  // namespace sht
}  // namespace dccm
