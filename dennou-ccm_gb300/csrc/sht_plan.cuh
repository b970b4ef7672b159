// Spherical-harmonic transform plan (internal header).
//
// Convention (the reference's SPML library is external and not vendored;
// this is the library's own, fixed and documented in the public header):
// latitudes ascending south to north, mu_j = sin(lat_j) the Gauss-Legendre
// nodes; longitudes 2 pi i / I; Pbar_n^m with integral Pbar^2 dmu = 2 and no
// Condon-Shortley phase; spectral coefficients complex, m-major,
// idx(m,n) = m(N+1) - m(m-1)/2 + (n-m); grid[b][j][i] (i fastest).
//
// Hemisphere pairing: jj = 0..J/2-1 indexes latitude pairs from the equator
// outwards, jn = J/2 + jj (north, mu > 0) and js = J/2 - 1 - jj (its mirror).
//
// Intermediate Fourier buffers (c = 2 b + {0: re, 1: im}, c fastest):
//   inverse: F[m][j][c]       Legendre synthesis output, FFT input;
//   forward: G[m][p][jj][c]   FFT output folded into parity p: p = 0 holds
//                             E = G(jn) + G(js), p = 1 holds O = G(jn) - G(js),
//                             already divided by I.
// Mixed precision: F is FP32; G is stored split as three BF16 planes (two
// FP16 planes, scaled per field-level, for DCCM_SHT_MIXED_FP16)
// G3[s][(2m + p) Jh + jj][c] (row length C2Bp = 2 max_batch rounded up to 8),
// the MN-major A operand of the tensor-core analysis; the spectra enter the
// tensor-core synthesis through Apack[s][c][x], BF16 planes of the split
// spectra with x = xoff(m, p) + k for n = m + p + 2k (K-major, each (m, p)
// segment rounded up to 16 with zeros).
#pragma once
#include <cuda.h>

#include <vector>

#include "common.cuh"

namespace dccm {
namespace sht {

// Layout of one Legendre operand table of bf16 split tiles (tensor path):
// rows of 64 bf16 (128 bytes) in a 2-D tensor [rows][64]; for (m, p) the
// tile of chunk q (64 wide along K) and split s starts at row
// base[m*2+p] + (q*3 + s) * nr[m*2+p], with nr rows (N-dimension extent
// rounded up to 16).  Entries past the valid K or N range are zero.
struct TileTable {
  std::vector<int64_t> base;  // per (m,p)
  std::vector<int> nr, nq, kval, nval;
  int64_t rows = 0;
  uint16_t *d = nullptr;      // device bf16 bits
  CUtensorMap map;            // TMA descriptor of the tiles, box {64, 128}
  CUtensorMap amap;           // TMA descriptor of the A operand (Apack or G3)
  bool map_ok = false;
  void *d_mi = nullptr;       // per-m tile metadata (device)
  int4 *d_items = nullptr;    // work items (m, ct, nt, -) for every 128-column block
  int items_per_ct = 0;       // work items per 128-column block of the batch
  int ntmax = 64;             // TMEM columns per accumulator (N tile bound)
};

struct Plan {
  int N = 0, I = 0, J = 0, Jh = 0;
  int precision = 0;
  int max_batch = 0;
  int64_t ncoef = 0;
  // host copies of the axes
  std::vector<double> mu, w;
  // device
  double *d_mu = nullptr, *d_w = nullptr;
  double *d_pnm = nullptr;     // FP64 Pbar(m, n, jj): [idx(m,n)][Jh]
  double2 *d_tw64 = nullptr;   // FFT twiddles e^{-2 pi i t / I}
  float2 *d_tw32 = nullptr;
  float2 *d_twl32 = nullptr;   // per-lane twiddles e^{-2 pi i l k / I} at [k][l], l < 32, k < I/32
  TileTable tinv, tfwd;        // bf16x3 tiles for the tensor path
  void *d_work = nullptr;      // Fourier buffer (F, G or G3), sized for max_batch
  size_t work_bytes = 0;
  int C2Bp = 0;                // row length of G3 and Apack (2 max_batch rounded up to 8)
  int64_t KX = 0;              // row length of Apack
  std::vector<int> xoff;       // Apack segment offset of (m, p) at [2m + p]
  uint16_t *d_apack = nullptr; // Apack[3][C2Bp][KX] (bf16 bits)
  int4 *d_punits = nullptr;    // pack units (m, q, x of parity 0, x of parity 1): 16 coefficients each
  int npunits = 0;
  int *d_err = nullptr;        // device error flag of bounded waits
  int nsplit = 3;              // tensor-path operand splits: 3 (BF16 x 3) or 2 (FP16 hi + lo)
  int *d_cexp = nullptr;       // FP16: per field-level scale exponents, [inverse | forward][max_batch]
  DevBuf stage;                // host entry point staging
  cudaStream_t stream = nullptr;
  // SPML real layout (spml.cu), set up by the first call that uses it:
  int2 *d_wa_pos = nullptr;    // per spectral index k: wa positions of Re and Im (-1: none)
  int *d_wa_src = nullptr;     // per wa position l: 2 k + (0: Re, 1: Im)
  DevBuf wa_spec;              // [max_batch][ncoef] complex spectra between layout and transform
};

__host__ __device__ inline int64_t idx_mn(int N, int m, int n) {
  return (int64_t)m * (N + 1) - (int64_t)m * (m - 1) / 2 + (n - m);
}

// Number of n in parity p (n - m = p mod 2) for zonal wavenumber m.
__host__ __device__ inline int count_np(int N, int m, int p) {
  const int first = m + p;
  return first > N ? 0 : (N - first) / 2 + 1;
}

// Kernel launchers (defined in the .cu files).
bool fft_length_supported(int I);
int fft_inverse_f64(const Plan &P, int batch, const double *F, double *grid, cudaStream_t s);
int fft_forward_f64(const Plan &P, int batch, const double *grid, double *G, cudaStream_t s);
int fft_inverse(const Plan &P, int batch, bool fp32, const void *F, double *grid, cudaStream_t s);
int fft_forward(const Plan &P, int batch, bool fp32, const double *grid, void *G, cudaStream_t s);
int legendre_inv_f64(const Plan &P, int batch, const double *spec, double *F, cudaStream_t s);
int legendre_fwd_f64(const Plan &P, int batch, const double *G, double *spec, cudaStream_t s);
int legendre_inv_tc(Plan &P, int batch, const double *spec, float *F, cudaStream_t s);
int legendre_fwd_tc(Plan &P, int batch, const void *G3, double *spec, cudaStream_t s);
int legendre_tc_multi(Plan *const *plans, const int *batch, const void *const *in, void *const *out,
                      int ngroups, int dir, cudaStream_t s);
int pack_spectra(Plan *const *plans, const int *batch, const double *const *spec, int ngroups, cudaStream_t s);
int field_exponents(const double *src, long long count, int batch, int *cexp, cudaStream_t s);
int fft_multi(Plan *const *plans, const int *batch, const void *const *in, void *const *out, int ngroups, bool fwd,
              cudaStream_t s);
int inverse(Plan &P, const double *spec, double *grid, int batch, cudaStream_t s);
int forward(Plan &P, const double *grid, double *spec, int batch, cudaStream_t s);
int build_tiles(Plan &P);

}  // namespace sht
}  // namespace dccm
