// Longitude FFT of the spherical-harmonic transform, FP32 (mixed path), one
// warp per pair of latitude rows.  The plain FP64 path has its own
// transform in fft_f64.cu.
//
// Two real latitude rows that mirror each other about the equator (jn, js)
// travel through one complex FFT of length I = 32 R: z = g(jn) + i g(js).
// Lane l holds R samples in registers and the transform is the four-step
// factorisation I = R x 32:
//   forward  (1) length-R DFT over r of z[32 r + l] in registers,
//            (2) twiddle e^{-2 pi i l k1 / I} (per-lane table [k1][l]),
//            (3) length-32 radix-2 decimation in frequency across the lanes
//                with __shfl_xor; lane l ends with Z[k1 + R brev5(l)];
//   inverse  the same steps mirrored (decimation in time across lanes from
//            bit-reversed input, conjugate twiddles, register DFT last), so
//            lane l ends with z[32 r + l] and the row stores are coalesced.
// Lane butterflies cost 8 instructions per complex value: the lane that
// owns the twiddled operand multiplies before the exchange (inverse) or
// after it (forward), the other lane multiplies by 1, and the sum or
// difference is one FMA with a per-lane sign.  Lane twiddles are loaded
// once per warp.
//
// Shared memory stages, per CTA (latitude pair jj, BB field-levels), the
// spectra of the CTA's row pairs: the inverse in the order its lanes read
// them (stage_z), the forward's results in planes of 17 R + 1 (re, im)
// pairs, one plane per (parity, field-level), coefficient m at slot
// (m mod R) * 17 + m / R.  A lane writes the m = k1 + R k2 it owns at
// k1 * 17 + k2 (consecutive across lanes, free of bank conflicts), and the
// copy to global memory takes up to four field-levels of one (m, parity)
// a thread, one 16-byte store per BF16 plane.
// Supported lengths: R in {2, 3, 4, 6, 8, 12, 16, 24, 32}, I = 64 ... 1024.
//
// Inverse: Z_m = A_m + i B_m and Z_{I-m} = conj(A_m) + i conj(B_m) from the
// Fourier coefficients A (row jn) and B (row js) in F[m][j][c]; Re z and
// Im z are the rows, written as FP64.
// Forward: Z_{I-m} comes from another lane by one shuffle (lane 31 - l,
// register R - k1; for k1 = 0 lane brev5(32 - k2)); A_m = (Z_m + conj
// Z_{I-m})/2, B_m = (Z_m - conj Z_{I-m})/(2i), folded into E = (A + B)/I and
// O = (A - B)/I and written split into three BF16 planes
// G3[s][(2m + p) Jh + jj][c] (p = 0: E, 1: O), the operand layout of the
// tensor-core analysis.
#include <string.h>

#include "fp_conv.cuh"
#include "sht_plan.cuh"

namespace dccm {
namespace sht {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// twiddle tw[t] = e^{-2 pi i t / I}; sign +1 uses its conjugate
__device__ __forceinline__ float2 twid(const float2 *tw, int t, int sign) {
  float2 w = __ldg(tw + t);
  if (sign > 0) w.y = -w.y;
  return w;
}
__device__ __forceinline__ float2 shfl_xor_c(float2 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
__device__ __forceinline__ float2 shfl_c(float2 v, int src) {
  v.x = __shfl_sync(0xffffffffu, v.x, src);
  v.y = __shfl_sync(0xffffffffu, v.y, src);
  return v;
}
__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

// Barrier of the nw warps of one row-pair group (named barrier 1 + g; 0 is
// __syncthreads): the groups' exchange buffers are their own, so one group's
// loads and arithmetic can overlap another's.  Every warp of the group
// executes it; warps outside every group execute none.
__device__ __forceinline__ void group_sync(int g, int nw) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(32 * nw) : "memory");
}

// e^{-2 pi i a / 24} (a multiple of 15 degrees) as literal constants: the
// in-register DFT lengths (2, 3, 4, 6, 8, 12) all divide 24, so their
// twiddles fold into the instructions instead of being loaded.  The values
// are the correctly rounded cos / sin of those angles, the same floats as
// the twiddle table built on the host.
__device__ __forceinline__ float2 unit24(int a) {
  constexpr float C15 = 0.96592582628906829f, S15 = 0.25881904510252076f;
  constexpr float C30 = 0.86602540378443865f, C45 = 0.70710678118654752f;
  float c, sn;  // cos and sin of 15 a degrees
  switch (((a % 24) + 24) % 24) {
    case 0: c = 1.f; sn = 0.f; break;
    case 1: c = C15; sn = S15; break;
    case 2: c = C30; sn = 0.5f; break;
    case 3: c = C45; sn = C45; break;
    case 4: c = 0.5f; sn = C30; break;
    case 5: c = S15; sn = C15; break;
    case 6: c = 0.f; sn = 1.f; break;
    case 7: c = -S15; sn = C15; break;
    case 8: c = -0.5f; sn = C30; break;
    case 9: c = -C45; sn = C45; break;
    case 10: c = -C30; sn = 0.5f; break;
    case 11: c = -C15; sn = S15; break;
    case 12: c = -1.f; sn = 0.f; break;
    case 13: c = -C15; sn = -S15; break;
    case 14: c = -C30; sn = -0.5f; break;
    case 15: c = -C45; sn = -C45; break;
    case 16: c = -0.5f; sn = -C30; break;
    case 17: c = -S15; sn = -C15; break;
    case 18: c = 0.f; sn = -1.f; break;
    case 19: c = S15; sn = -C15; break;
    case 20: c = 0.5f; sn = -C30; break;
    case 21: c = C45; sn = -C45; break;
    case 22: c = C30; sn = -0.5f; break;
    default: c = C15; sn = -S15; break;
  }
  return make_float2(c, -sn);
}

// o e^{sign 2 pi i a / 24}: the quarter turns (1, -i, -1, i) as swaps and
// negations, which the compiler cannot make of a multiply by 0 and -1 (x * 0
// is not 0 for infinities, NaN and -0).
__device__ __forceinline__ float2 mul_unit24(float2 o, int a, int sign) {
  const int b = (((sign > 0 ? -a : a) % 24) + 24) % 24;
  if (b == 0) return o;
  if (b == 6) return make_float2(o.y, -o.x);  // -i
  if (b == 12) return make_float2(-o.x, -o.y);
  if (b == 18) return make_float2(-o.y, o.x);  // +i
  return cmul(o, unit24(b));
}

// In-register DFT of length R: v[k] <- sum_r v[r] e^{sign 2 pi i r k / R}.
// Even lengths split into two halves (decimation in time), 3 is direct.
template <int R> struct RegDft {
  __device__ __forceinline__ static void run(float2 *v, const float2 *tw, int I, int sign) {
    if constexpr (R == 1) {
      return;
    } else if constexpr (R == 2) {
      const float2 a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else if constexpr (R == 3) {
      const float2 t1 = cadd(v[1], v[2]);
      const float2 d = csub(v[1], v[2]);
      const float h = 0.86602540378443864676f * (float)sign;  // sign * sqrt(3)/2
      float2 mm, q;
      mm.x = v[0].x - 0.5f * t1.x;
      mm.y = v[0].y - 0.5f * t1.y;
      q.x = -d.y * h;  // i * sign * sqrt(3)/2 * d
      q.y = d.x * h;
      v[0] = cadd(v[0], t1);
      v[1] = cadd(mm, q);
      v[2] = csub(mm, q);
    } else {
      static_assert(R % 2 == 0 && 24 % R == 0, "length");
      constexpr int H = R / 2;
      float2 e[H], o[H];
#pragma unroll
      for (int i = 0; i < H; ++i) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
      }
      RegDft<H>::run(e, tw, I, sign);
      RegDft<H>::run(o, tw, I, sign);
#pragma unroll
      for (int k = 0; k < H; ++k) {
        const float2 t = mul_unit24(o[k], k * (24 / R), sign);
        v[k] = cadd(e[k], t);
        v[k + H] = csub(e[k], t);
      }
    }
  }
};

// Per-lane twiddles of the five lane stages: stage s exchanges with lane
// l ^ h (forward h = 16 >> s, inverse h = 1 << s); the upper lane (l & h)
// multiplies by e^{-+2 pi i (l & (h-1)) / (2h)}, the lower one by 1.
template <int R>
__device__ __forceinline__ void lane_twiddles(const float2 *tw, int lane, bool inv, float2 (&w)[5]) {
  constexpr int I = 32 * R;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = inv ? (1 << s) : (16 >> s);
    w[s] = make_float2(1.f, 0.f);
    if (lane & h) w[s] = twid(tw, (lane & (h - 1)) * (I / (2 * h)), inv ? 1 : -1);
  }
}

// 32-point DFT across the lanes of every register n < NV, decimation in
// frequency: lane l ends with the output brev5(l).
template <int NV>
__device__ __forceinline__ void lane_dif(float2 (&v)[NV], const float2 (&w)[5], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 16 >> s;
    const float sg = (lane & h) ? -1.f : 1.f;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      // lower: a + b; upper: (a - b) w  (the lower lane holds a)
      const float2 p = shfl_xor_c(v[k], h);
      const float2 t = make_float2(fmaf(sg, v[k].x, p.x), fmaf(sg, v[k].y, p.y));
      v[k] = s == 4 ? t : cmul(t, w[s]);  // the last stage's twiddles are all 1
    }
  }
}

// Its inverse (unnormalised), decimation in time from bit-reversed input.
template <int NV>
__device__ __forceinline__ void lane_dit(float2 (&v)[NV], const float2 (&w)[5], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 1 << s;
    const float sg = (lane & h) ? -1.f : 1.f;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      // lower: a + w b; upper: a - w b  (the upper lane holds b)
      const float2 x = s == 0 ? v[k] : cmul(v[k], w[s]);  // the first stage's twiddles are all 1
      const float2 p = shfl_xor_c(x, h);
      v[k] = make_float2(fmaf(sg, x.x, p.x), fmaf(sg, x.y, p.y));
    }
  }
}

// Forward complex FFT of one row held as v[r] = z[32 r + lane];
// on return v[k1] = Z[k1 + R brev5(lane)].
template <int R>
__device__ __forceinline__ void warp_fft_fwd(float2 (&v)[R], const float2 *tw, const float2 *twl,
                                             const float2 (&w)[5], int lane) {
  constexpr int I = 32 * R;
  RegDft<R>::run(v, tw, I, -1);
#pragma unroll
  for (int k = 1; k < R; ++k) v[k] = cmul(v[k], __ldg(twl + k * 32 + lane));
  lane_dif<R>(v, w, lane);
}

// Inverse (unnormalised) FFT of one row held as v[k1] = Z[k1 + R brev5(lane)];
// on return v[r] = z[32 r + lane].
template <int R>
__device__ __forceinline__ void warp_fft_inv(float2 (&v)[R], const float2 *tw, const float2 *twl,
                                             const float2 (&w)[5], int lane) {
  constexpr int I = 32 * R;
  lane_dit<R>(v, w, lane);
#pragma unroll
  for (int k = 1; k < R; ++k) {
    float2 t = __ldg(twl + k * 32 + lane);
    t.y = -t.y;
    v[k] = cmul(v[k], t);
  }
  RegDft<R>::run(v, tw, I, +1);
}

constexpr int FFT_MAXG = 8;
struct FftGroup {
  int N, J, batch, BB, lbb, R, W, blk0, C2Bp;  // BB row pairs per CTA, lbb = log2(BB), W warps per row pair
  const void *in;
  void *out;
  const float2 *tw, *twl;
  int nsplit;        // forward output planes: 3 BF16, or 2 FP16 scaled by 2^(13 - cexp[b])
  const int *cexp;   // FP16: exponent of each field-level's largest |grid value|
};
struct FftLaunch {
  FftGroup g[FFT_MAXG];
  int ngroups;
};

template <int R> __device__ __forceinline__ int slot_of(int m) { return (m % R) * 17 + m / R; }

// ------------------------------------------------------------- inverse
// One CTA: latitude pair jj, field-levels [by*BB, by*BB + BB); warp bl
// transforms field-level b0 + bl.  The CTA first assembles the spectrum of
// every packed row pair z = g(jn) + i g(js) in shared memory, in the order
// the lanes read it: Zs[bl][k mod R][brev5(k / R)] (float2, rows of 33,
// field-level stride 33 R + 1, so that the field-levels and the consecutive
// m that a warp writes at once fall in different banks).  Z_m = A_m + i B_m and Z_{I-m} = conj(A_m) +
// i conj(B_m) from the Fourier coefficients A (row jn) and B (row js) in
// F[m][j][c] (imaginary parts of m = 0 taken as 0), zero for N < k < I - N.
// One thread per (m, field-level), field-levels fastest: a warp's float2
// loads cover whole 64-byte runs of F per (m, row).  Each lane then reads
// its R inputs with one conflict-free 64-bit load apiece.
// Residue rows of 33 float2 (32 lanes and one pad): consecutive m, which a
// warp's staging threads write at once, fall in different banks.
constexpr int ZQ = 33;
template <int R> __device__ __forceinline__ constexpr int zs_stride() { return ZQ * R + 1; }

template <int R>
__device__ __forceinline__ void stage_z(const FftGroup &G, int jn, int js, int b0, int nb, float2 *zs) {
  constexpr int I = 32 * R, ZB = zs_stride<R>();
  const int N = G.N, lbb = G.lbb, bmask = G.BB - 1;
  const long long C2B = 2LL * G.batch;
  const float *F = static_cast<const float *>(G.in);
  const int tot = (N + 1) << lbb;  // (m, bl), bl fastest
  constexpr int U = 2;             // both rows of two units in flight before the stores
#pragma unroll 1
  for (int t0 = threadIdx.x; t0 < tot; t0 += U * blockDim.x) {
    float2 a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = t0 + u * blockDim.x;
      const int bl = t & bmask, m = t >> lbb;
      a[u] = b[u] = make_float2(0.f, 0.f);
      if (t < tot && bl < nb) {
        const long long c = 2LL * (b0 + bl);
        a[u] = *reinterpret_cast<const float2 *>(F + ((long long)m * G.J + jn) * C2B + c);
        b[u] = *reinterpret_cast<const float2 *>(F + ((long long)m * G.J + js) * C2B + c);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int t = t0 + u * blockDim.x;
      if (t >= tot) break;
      const int bl = t & bmask, m = t >> lbb;
      float2 *z = zs + bl * ZB;
      const float ai = m ? a[u].y : 0.f, bi = m ? b[u].y : 0.f;
      z[(m % R) * ZQ + brev5(m / R)] = make_float2(a[u].x - bi, ai + b[u].x);
      if (m) {
        const int k = I - m;
        z[(k % R) * ZQ + brev5(k / R)] = make_float2(a[u].x + bi, b[u].x - ai);
      }
    }
  }
  const int gap = I - 2 * N - 1;  // k = N+1 .. I-N-1
#pragma unroll 1
  for (int t = threadIdx.x; t < (gap << lbb); t += blockDim.x) {
    const int k = N + 1 + (t >> lbb);
    zs[(t & bmask) * ZB + (k % R) * ZQ + brev5(k / R)] = make_float2(0.f, 0.f);
  }
}

template <int R>
__device__ __forceinline__ void fft_inv_block(const FftGroup &G, int jj, int by, float *st) {
  constexpr int I = 32 * R, ZB = zs_stride<R>();
  const int J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  float2 *zs = reinterpret_cast<float2 *>(st);
  stage_z<R>(G, jn, js, b0, nb, zs);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, true, w);
  for (int bl = warp; bl < nb; bl += nw) {
    float2 v[R];
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) v[k1] = zs[bl * ZB + k1 * ZQ + lane];
    warp_fft_inv<R>(v, G.tw, G.twl, w, lane);
    double *gn = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + jn) * I;
    double *gs = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + js) * I;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      gn[32 * r + lane] = f32_to_f64(v[r].x);
      gs[32 * r + lane] = f32_to_f64(v[r].y);
    }
  }
}

// ------------------------------------------------------------- forward
// The forward stages E and O of every row pair in shared memory as (re, im)
// pairs: plane (parity p, field-level bl) of 17 R + 1 float2, m at slot
// (m mod R) * 17 + m / R.
template <int R> __device__ __forceinline__ float2 *eo_plane(float *st, int BB, int p, int bl) {
  return reinterpret_cast<float2 *>(st) + (size_t)(p * BB + bl) * (R * 17 + 1);
}

// Split the staged E/O values into G3[s][(2m + p) Jh + jj][2 b0 + c], c =
// 2 bl + re/im.  A thread item is (m, p, FL consecutive field-levels): FL
// float2 reads and one store of 2 FL bf16 per plane (16, 8 or 4 bytes: the
// run starts at 2 b0 + 2 FL q in a row of C2Bp, a multiple of 8).  Values
// are split two at a time (packed conversions round each half as the
// scalar ones do).
template <int R, int FL>
__device__ __forceinline__ void write_g3_fl(const FftGroup &G, int jj, int b0, int nb, float *st) {
  const int N = G.N, Jh = G.J / 2, BB = G.BB, nq = BB / FL;
  unsigned short *G3 = static_cast<unsigned short *>(G.out);
  const size_t plane = (size_t)(N + 1) * 2 * Jh * G.C2Bp;
  const int tot = (N + 1) * 2 * nq;  // (m, p, q), q fastest
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int q = t % nq, p = (t / nq) & 1, m = t / (2 * nq);
    const int f0 = FL * q;
    if (f0 >= nb) continue;
    const int sl = slot_of<R>(m);
    float2 v[FL];
#pragma unroll
    for (int i = 0; i < FL; ++i) v[i] = eo_plane<R>(st, BB, p, f0 + i)[sl];
    unsigned short *o = G3 + ((size_t)(2 * m + p) * Jh + jj) * G.C2Bp + 2 * (b0 + f0);
    const bool full = f0 + FL <= nb;
    unsigned w[3][FL];
    if (G.nsplit == 2) {
#pragma unroll
      for (int i = 0; i < FL; ++i) {  // no scale past the batch
        const float sc = f0 + i < nb ? pow2f(13 - G.cexp[b0 + f0 + i]) : 0.f;
        split2h_x2(make_float2(v[i].x * sc, v[i].y * sc), w[0][i], w[1][i]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < FL; ++i) split3f_x2(v[i], w[0][i], w[1][i], w[2][i]);
    }
    const int ns = G.nsplit;
    if (full) {
#pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        if (s3 >= ns) break;
        unsigned short *os = o + s3 * plane;
        if constexpr (FL == 4) *reinterpret_cast<uint4 *>(os) = make_uint4(w[s3][0], w[s3][1], w[s3][2], w[s3][3]);
        else if constexpr (FL == 2) *reinterpret_cast<uint2 *>(os) = make_uint2(w[s3][0], w[s3][1]);
        else *reinterpret_cast<unsigned *>(os) = w[s3][0];
      }
    } else {
#pragma unroll
      for (int i = 0; i < FL; ++i)
#pragma unroll
        for (int s3 = 0; s3 < 3; ++s3)
          if (f0 + i < nb && s3 < ns) {
            o[s3 * plane + 2 * i] = (unsigned short)w[s3][i];
            o[s3 * plane + 2 * i + 1] = (unsigned short)(w[s3][i] >> 16);
          }
    }
  }
}

template <int R>
__device__ __forceinline__ void write_g3(const FftGroup &G, int jj, int b0, int nb, float *st) {
  if (G.BB >= 4) write_g3_fl<R, 4>(G, jj, b0, nb, st);
  else if (G.BB == 2) write_g3_fl<R, 2>(G, jj, b0, nb, st);
  else write_g3_fl<R, 1>(G, jj, b0, nb, st);
}

// E_m = (A + B)/I and O_m = (A - B)/I of field-level bl from Z_m and
// Z_{I-m}, into the staging planes at slot sl (m = 0: imaginary parts 0).
template <int R>
__device__ __forceinline__ void store_eo(float *st, int BB, int bl, int m, int sl, float2 zm, float2 zc,
                                         float invI) {
  const float ar = 0.5f * (zm.x + zc.x), ai = 0.5f * (zm.y - zc.y);
  const float br = 0.5f * (zm.y + zc.y), bi = -0.5f * (zm.x - zc.x);
  eo_plane<R>(st, BB, 0, bl)[sl] = make_float2((ar + br) * invI, m ? (ai + bi) * invI : 0.f);
  eo_plane<R>(st, BB, 1, bl)[sl] = make_float2((ar - br) * invI, m ? (ai - bi) * invI : 0.f);
}

template <int R>
__device__ __forceinline__ void fft_fwd_block(const FftGroup &G, int jj, int by, float *st) {
  constexpr int I = 32 * R;
  const int N = G.N, J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int k2 = brev5(lane);
  const int src0 = brev5((32 - k2) & 31);
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, false, w);
  const float invI = 1.f / (float)I;
  for (int bl = warp; bl < nb; bl += nw) {
    const double *gn = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + jn) * I;
    const double *gs = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + js) * I;
    // all 2R loads of the row pair first, then the conversions
    double xn[R], xs[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      xn[r] = gn[32 * r + lane];
      xs[r] = gs[32 * r + lane];
    }
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = make_float2(f64_to_f32_rn(xn[r]), f64_to_f32_rn(xs[r]));
    warp_fft_fwd<R>(v, G.tw, G.twl, w, lane);
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
      const float2 zc = k1 ? shfl_c(v[(R - k1) % R], 31 - lane) : shfl_c(v[0], src0);  // Z[I - m]
      const int m = k1 + R * k2;
      if (m <= N) store_eo<R>(st, G.BB, bl, m, k1 * 17 + k2, v[k1], zc, invI);
    }
  }
  __syncthreads();
  write_g3<R>(G, jj, b0, nb, st);
}

// ---------------------------------------------- rows over several warps
// Long rows, R = 8 W with W = 2, 3, 4 (I = 512, 768, 1024): W warps share a
// row pair, 8 samples a lane, I = 8 L with L = 32 W and t = 32 wq + l:
//   forward  thread (wq, l) holds z[L r + t], r < 8; an 8-point DFT in
//            registers, twiddle e^{-2 pi i t k1 / I}, then the L-point DFT
//            over t: a W-point DFT across the warps through shared memory
//            (warp wq keeps output k_w = wq), twiddle e^{-2 pi i l k_w / L},
//            and the 32-point lane DFT; thread (wq, l) ends with
//            Z[k1 + 8 (wq + W brev5(l))], i.e. m mod R = k1 + 8 wq and
//            m / R = brev5(l), as in the one-warp path;
//   inverse  the mirror image.
// The partner Z_{I-m} of the forward separation comes through the same
// exchange buffer, float2 [8][W][32] per row pair.  8 samples a lane keep
// the register count of the R = 8 rows (the one-warp R = 32 row needs 175).
constexpr int MW_R0 = 8;

template <int W>
__device__ __forceinline__ void fft_inv_block_mw(const FftGroup &G, int jj, int by, float *st) {
  constexpr int R = MW_R0 * W, I = 32 * R, L = 32 * W;
  constexpr int ZB = zs_stride<R>();
  const int J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  float2 *zs = reinterpret_cast<float2 *>(st);
  stage_z<R>(G, jn, js, b0, nb, zs);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bl = warp / W, wq = warp % W;
  const bool own = bl < G.BB;  // this warp has a staged spectrum and an exchange slot
  float2 *xb = zs + (size_t)G.BB * ZB + (size_t)(own ? bl : 0) * MW_R0 * W * 32;
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, true, w);
  float2 v[MW_R0];
#pragma unroll
  for (int k1 = 0; k1 < MW_R0; ++k1)
    v[k1] = own ? zs[bl * ZB + (k1 + MW_R0 * wq) * ZQ + lane] : make_float2(0.f, 0.f);
  lane_dit<MW_R0>(v, w, lane);
  const float2 tq = twid(G.tw, lane * wq * (I / L), +1);
#pragma unroll
  for (int k1 = 0; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], tq);
  if (own) {
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) xb[(k1 * W + wq) * 32 + lane] = v[k1];
    group_sync(bl, W);
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) {
      float2 acc = xb[(k1 * W) * 32 + lane];
#pragma unroll
      for (int kw = 1; kw < W; ++kw)
        acc = cadd(acc, cmul(xb[(k1 * W + kw) * 32 + lane], twid(G.tw, ((wq * kw) % W) * (I / W), +1)));
      v[k1] = acc;
    }
  }
  const int t = 32 * wq + lane;
#pragma unroll
  for (int k1 = 1; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], twid(G.tw, t * k1, +1));
  RegDft<MW_R0>::run(v, G.tw, I, +1);
  if (bl < nb) {
    double *gn = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + jn) * I;
    double *gs = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + js) * I;
#pragma unroll
    for (int r = 0; r < MW_R0; ++r) {
      gn[L * r + t] = f32_to_f64(v[r].x);
      gs[L * r + t] = f32_to_f64(v[r].y);
    }
  }
}

template <int W>
__device__ __forceinline__ void fft_fwd_block_mw(const FftGroup &G, int jj, int by, float *st) {
  constexpr int R = MW_R0 * W, I = 32 * R, L = 32 * W, PS = R * 17 + 1;
  const int N = G.N, J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bl = warp / W, wq = warp % W;
  const bool own = bl < G.BB;
  const int kl = brev5(lane);
  const int t = 32 * wq + lane;
  float2 *xb = reinterpret_cast<float2 *>(st + 4 * G.BB * PS) + (size_t)(own ? bl : 0) * MW_R0 * W * 32;
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, false, w);
  float2 v[MW_R0];
  if (bl < nb) {
    const double *gn = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + jn) * I;
    const double *gs = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + js) * I;
    double xn[MW_R0], xs[MW_R0];  // all loads first, then the conversions
#pragma unroll
    for (int r = 0; r < MW_R0; ++r) {
      xn[r] = gn[L * r + t];
      xs[r] = gs[L * r + t];
    }
#pragma unroll
    for (int r = 0; r < MW_R0; ++r) v[r] = make_float2(f64_to_f32_rn(xn[r]), f64_to_f32_rn(xs[r]));
  } else {
#pragma unroll
    for (int r = 0; r < MW_R0; ++r) v[r] = make_float2(0.f, 0.f);
  }
  RegDft<MW_R0>::run(v, G.tw, I, -1);
#pragma unroll
  for (int k1 = 1; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], twid(G.tw, t * k1, -1));
  if (own) {
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) xb[(k1 * W + wq) * 32 + lane] = v[k1];
    group_sync(bl, W);
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) {
      float2 acc = xb[(k1 * W) * 32 + lane];
#pragma unroll
      for (int kw = 1; kw < W; ++kw)
        acc = cadd(acc, cmul(xb[(k1 * W + kw) * 32 + lane], twid(G.tw, ((wq * kw) % W) * (I / W), -1)));
      v[k1] = acc;
    }
  }
  const float2 tq = twid(G.tw, lane * wq * (I / L), -1);
#pragma unroll
  for (int k1 = 0; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], tq);
  lane_dif<MW_R0>(v, w, lane);
  if (own) {
    group_sync(bl, W);  // every warp of the group is done reading the exchange buffer
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) xb[(k1 * W + wq) * 32 + lane] = v[k1];
    group_sync(bl, W);
  }
  if (bl < nb) {
    const float invI = 1.f / (float)I;
#pragma unroll
    for (int k1 = 0; k1 < MW_R0; ++k1) {
      const int q = k1 + MW_R0 * wq;
      const int m = q + R * kl;
      if (m <= N) {
        // Z[I - m]: residue R - q (register (8 - k1) mod 8 of warp W-1-wq, or
        // W-wq when k1 = 0) in lane 31 - l; for m = 0 mod R lane brev5(32 - kl)
        int src;
        if (q) src = ((((MW_R0 - k1) % MW_R0) * W) + (k1 ? W - 1 - wq : W - wq)) * 32 + (31 - lane);
        else src = brev5((32 - kl) & 31);
        store_eo<R>(st, G.BB, bl, m, q * 17 + kl, v[k1], xb[src], invI);
      }
    }
  }
  __syncthreads();
  write_g3<R>(G, jj, b0, nb, st);
}

// ------------------------------- rows over two or four warps, one exchange
// For W = 2 and 4 the W-point step runs where its inputs meet instead: warp
// wq owns 8 / W of the residues k1 and all W indices of the cross-warp
// step, so each value crosses the exchange buffer once, read once (the
// variant above reads every entry W times, once per output warp).  The
// residues are paired (k1, 8 - k1) within a warp: {0, 4} and {2, 6} (W = 2)
// in warp 0, {1, 7} and {3, 5} in warp 1; for W = 4 {0, 4}, {1, 7}, {2, 6},
// {3, 5}.  So the forward's partner Z_{I-m} is in the same warp, one
// shuffle away.
//   forward  thread (wq, l): z[L r + t] (t = 32 wq + l) -> 8-point DFT and
//            twiddle e^{-2 pi i t k1 / I} as above -> exchange -> for each
//            owned k1 the W-point DFT over t_w, twiddle e^{-2 pi i l k_w / L},
//            32-point lane DFT: register (j, k_w) of lane l holds
//            Z[k1_j + 8 k_w + R brev5(l)];
//   inverse  the mirror: thread (wq, l) reads Z[k1_j + 8 k_w + R brev5(l)]
//            from the staged spectrum, lane DFT, twiddle, W-point DFT to t_w,
//            exchange, and continues as above with all k1 of t_w = wq.
template <int W> __device__ __forceinline__ int mw_base(int wq, int j) { return wq + W * (j >> 1); }
template <int W> __device__ __forceinline__ int mw_k1(int wq, int j) {
  const int b = mw_base<W>(wq, j);
  return (j & 1) ? (b ? MW_R0 - b : 4) : b;
}

// A CTA's warps form groups of W, one row pair per group at a time; with
// more row pairs than groups (the fft_rpw knob) a group takes them in
// turns (passes), every pass ending at the group's own barrier before its
// exchange buffer is written again.  More field-levels a CTA make the
// forward's G3 runs longer (a whole 32-byte sector per BF16 plane from 8
// field-levels).
template <int W>
__device__ __forceinline__ void fft_inv_block_mwp(const FftGroup &G, int jj, int by, float *st) {
  constexpr int R = MW_R0 * W, I = 32 * R, L = 32 * W, NK = MW_R0 / W;
  constexpr int ZB = zs_stride<R>();
  const int J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  float2 *zs = reinterpret_cast<float2 *>(st);
  stage_z<R>(G, jn, js, b0, nb, zs);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ng = (int)(blockDim.x >> 5) / W, grp = warp / W, wq = warp % W;
  float2 *xb = zs + (size_t)G.BB * ZB + (size_t)grp * MW_R0 * W * 32;
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, true, w);
  const int t = 32 * wq + lane;
  const int passes = (G.BB + ng - 1) / ng;
  for (int rd = 0; rd < passes; ++rd) {
    const int bl = rd * ng + grp;
    const bool own = grp < ng && bl < G.BB;  // this group has a staged spectrum in this pass
    float2 v[MW_R0];  // v[j W + k_w]
#pragma unroll
    for (int j = 0; j < NK; ++j)
#pragma unroll
      for (int kw = 0; kw < W; ++kw)
        v[j * W + kw] = own ? zs[bl * ZB + (mw_k1<W>(wq, j) + MW_R0 * kw) * ZQ + lane] : make_float2(0.f, 0.f);
    lane_dit<MW_R0>(v, w, lane);
#pragma unroll
    for (int kw = 1; kw < W; ++kw) {
      const float2 tq = twid(G.tw, lane * kw * (I / L), +1);
#pragma unroll
      for (int j = 0; j < NK; ++j) v[j * W + kw] = cmul(v[j * W + kw], tq);
    }
#pragma unroll
    for (int j = 0; j < NK; ++j) RegDft<W>::run(v + j * W, G.tw, I, +1);
    if (own) {
#pragma unroll
      for (int j = 0; j < NK; ++j)
#pragma unroll
        for (int tx = 0; tx < W; ++tx) xb[(mw_k1<W>(wq, j) * W + tx) * 32 + lane] = v[j * W + tx];
    }
    if (grp < ng) group_sync(grp, W);
    if (own) {
#pragma unroll
      for (int k1 = 0; k1 < MW_R0; ++k1) v[k1] = xb[(k1 * W + wq) * 32 + lane];
    }
#pragma unroll
    for (int k1 = 1; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], twid(G.tw, t * k1, +1));
    RegDft<MW_R0>::run(v, G.tw, I, +1);
    if (own && bl < nb) {
      double *gn = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + jn) * I;
      double *gs = static_cast<double *>(G.out) + ((long long)(b0 + bl) * J + js) * I;
#pragma unroll
      for (int r = 0; r < MW_R0; ++r) {
        gn[L * r + t] = f32_to_f64(v[r].x);
        gs[L * r + t] = f32_to_f64(v[r].y);
      }
    }
    if (rd + 1 < passes && grp < ng) group_sync(grp, W);  // the exchange buffer is read before the next pass writes it
  }
}

template <int W>
__device__ __forceinline__ void fft_fwd_block_mwp(const FftGroup &G, int jj, int by, float *st) {
  constexpr int R = MW_R0 * W, I = 32 * R, L = 32 * W, PS = R * 17 + 1, NK = MW_R0 / W;
  const int N = G.N, J = G.J, Jh = J / 2;
  const int jn = Jh + jj, js = Jh - 1 - jj;
  const int b0 = by * G.BB;
  const int nb = min(G.BB, G.batch - b0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ng = (int)(blockDim.x >> 5) / W, grp = warp / W, wq = warp % W;
  const int kl = brev5(lane);
  const int t = 32 * wq + lane;
  float2 *xb = reinterpret_cast<float2 *>(st + 4 * G.BB * PS) + (size_t)grp * MW_R0 * W * 32;
  float2 w[5];
  lane_twiddles<R>(G.tw, lane, false, w);
  const int src0 = brev5((32 - kl) & 31);
  const float invI = 1.f / (float)I;
  const int passes = (G.BB + ng - 1) / ng;
  for (int rd = 0; rd < passes; ++rd) {
    const int bl = rd * ng + grp;
    const bool own = grp < ng && bl < G.BB;  // this group has an exchange slot and staging planes in this pass
    float2 v[MW_R0];
    if (own && bl < nb) {
      const double *gn = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + jn) * I;
      const double *gs = static_cast<const double *>(G.in) + ((long long)(b0 + bl) * J + js) * I;
      double xn[MW_R0], xs[MW_R0];  // all loads first, then the conversions
#pragma unroll
      for (int r = 0; r < MW_R0; ++r) {
        xn[r] = gn[L * r + t];
        xs[r] = gs[L * r + t];
      }
#pragma unroll
      for (int r = 0; r < MW_R0; ++r) v[r] = make_float2(f64_to_f32_rn(xn[r]), f64_to_f32_rn(xs[r]));
    } else {
#pragma unroll
      for (int r = 0; r < MW_R0; ++r) v[r] = make_float2(0.f, 0.f);
    }
    RegDft<MW_R0>::run(v, G.tw, I, -1);
#pragma unroll
    for (int k1 = 1; k1 < MW_R0; ++k1) v[k1] = cmul(v[k1], twid(G.tw, t * k1, -1));
    if (own) {
#pragma unroll
      for (int k1 = 0; k1 < MW_R0; ++k1) xb[(k1 * W + wq) * 32 + lane] = v[k1];
    }
    if (grp < ng) group_sync(grp, W);
    if (own) {
#pragma unroll
      for (int j = 0; j < NK; ++j)
#pragma unroll
        for (int tx = 0; tx < W; ++tx) v[j * W + tx] = xb[(mw_k1<W>(wq, j) * W + tx) * 32 + lane];
    }
#pragma unroll
    for (int j = 0; j < NK; ++j) RegDft<W>::run(v + j * W, G.tw, I, -1);
#pragma unroll
    for (int kw = 1; kw < W; ++kw) {
      const float2 tq = twid(G.tw, lane * kw * (I / L), -1);
#pragma unroll
      for (int j = 0; j < NK; ++j) v[j * W + kw] = cmul(v[j * W + kw], tq);
    }
    lane_dif<MW_R0>(v, w, lane);
    // Z[I - m] for m = k1 + 8 k_w + R kl, all within the warp:
    //   k1 in {1, 2, 3, 5, 6, 7}: register (partner j, W-1-k_w), lane 31 - l;
    //   k1 = 4: register (j, W-1-k_w), lane 31 - l;
    //   k1 = 0: register (j, W-k_w), lane 31 - l; for k_w = 0 register (j, 0),
    //   lane brev5(32 - kl).
#pragma unroll
    for (int j = 0; j < NK; ++j) {
      const bool paired = mw_base<W>(wq, j) != 0;  // warp-uniform
      const int k1 = mw_k1<W>(wq, j);
#pragma unroll
      for (int kw = 0; kw < W; ++kw) {
        float2 zc;
        if (paired) zc = shfl_c(v[(j ^ 1) * W + (W - 1 - kw)], 31 - lane);
        else if (j & 1) zc = shfl_c(v[j * W + (W - 1 - kw)], 31 - lane);
        else zc = kw ? shfl_c(v[j * W + (W - kw)], 31 - lane) : shfl_c(v[j * W], src0);
        const int q = k1 + MW_R0 * kw;
        const int m = q + R * kl;
        if (own && bl < nb && m <= N) store_eo<R>(st, G.BB, bl, m, q * 17 + kl, v[j * W + kw], zc, invI);
      }
    }
    if (rd + 1 < passes && grp < ng) group_sync(grp, W);  // the exchange buffer is read before the next pass writes it
  }
  __syncthreads();  // every group's planes are complete
  write_g3<R>(G, jj, b0, nb, st);
}

// ------------------------------------------------------------- kernels
// Several truncation groups in one launch: CTA blockIdx.x belongs to the
// group whose block range contains it; the group's length selects the
// register FFT (cases up to RMAX are compiled in).
template <int R, int RMAX, bool FWD>
__device__ __forceinline__ void dispatch_case(const FftGroup &G, int jj, int by, float *st) {
  if constexpr (R <= RMAX) {
    if constexpr (R == 24) {
      if (FWD) fft_fwd_block_mw<R / MW_R0>(G, jj, by, st);
      else fft_inv_block_mw<R / MW_R0>(G, jj, by, st);
    } else if constexpr (R >= 16) {
      if (FWD) fft_fwd_block_mwp<R / MW_R0>(G, jj, by, st);
      else fft_inv_block_mwp<R / MW_R0>(G, jj, by, st);
    } else {
      if (FWD) fft_fwd_block<R>(G, jj, by, st);
      else fft_inv_block<R>(G, jj, by, st);
    }
  }
}

// Up to 16 warps (512 threads) per CTA.  RFIX > 0: every group of the
// launch has R = RFIX and only that case is compiled in (one case keeps the
// register allocation of that case alone; a launch mixing lengths, e.g. an
// ensemble of truncations, takes the RFIX = 0 kernel with every case up to
// RMAX).
template <int RFIX, int RMAX, bool FWD>
__global__ void __launch_bounds__(512, 2) fft_multi_kernel(const __grid_constant__ FftLaunch L) {
  extern __shared__ __align__(16) float st[];
  pdl_wait();  // reads the previous kernel's output; the forward FFT overwrites the buffer it read
  pdl_trigger();
  int gi = 0;
  while (gi + 1 < L.ngroups && (int)blockIdx.x >= L.g[gi + 1].blk0) ++gi;
  const FftGroup &G = L.g[gi];
  // Forward: field-level blocks fastest, so the CTAs that share the G3 rows
  // of one latitude pair (each writes 2 BB columns of them) run together and
  // the 32-byte sectors they split are completed in L2, not written back
  // partly.  Inverse: latitude pairs fastest, so consecutive CTAs write
  // neighbouring grid rows of the same field-levels.
  const int lb = blockIdx.x - G.blk0;
  const int nby = (G.batch + G.BB - 1) / G.BB;
  const int Jh = G.J / 2;
  const int by = FWD ? lb % nby : lb / Jh, jj = FWD ? lb / nby : lb % Jh;
  if constexpr (RFIX > 0) {
    dispatch_case<RFIX, RMAX, FWD>(G, jj, by, st);
  } else {
    switch (G.R) {
      case 2: dispatch_case<2, RMAX, FWD>(G, jj, by, st); break;
      case 3: dispatch_case<3, RMAX, FWD>(G, jj, by, st); break;
      case 4: dispatch_case<4, RMAX, FWD>(G, jj, by, st); break;
      case 6: dispatch_case<6, RMAX, FWD>(G, jj, by, st); break;
      case 8: dispatch_case<8, RMAX, FWD>(G, jj, by, st); break;
      case 12: dispatch_case<12, RMAX, FWD>(G, jj, by, st); break;
      case 16: dispatch_case<16, RMAX, FWD>(G, jj, by, st); break;
      case 24: dispatch_case<24, RMAX, FWD>(G, jj, by, st); break;
      case 32: dispatch_case<32, RMAX, FWD>(G, jj, by, st); break;
      default: break;
    }
  }
}

// Warps per row pair and shared memory of one CTA: the staged spectra
// (inverse) or the E/O planes (forward) of its bb row pairs, and for rows
// over several warps the exchange buffers, 8 x W x 32 complex values for
// each of the CTA's nx warp groups (W = 3: one per row pair).
static int fft_warps_per_row(int R) { return R >= 16 ? R / MW_R0 : 1; }
static size_t fft_smem(int R, int bb, int nx) {
  const int W = fft_warps_per_row(R);
  const size_t planes = (size_t)4 * bb * (R * 17 + 1) * sizeof(float);  // forward: E/O planes
  const size_t zs = (size_t)bb * (33 * R + 1) * sizeof(float2);          // inverse: staged spectra
  size_t s = planes > zs ? planes : zs;
  if (W > 1) s += (size_t)(W == 3 ? bb : nx) * MW_R0 * W * 32 * sizeof(float2);
  return s;
}

// One launch over ngroups plans (FP32).  Inverse: in[g] = F, out[g] = grid;
// forward: in[g] = grid, out[g] = G3 (the plan's Fourier buffer).
int fft_multi(Plan *const *plans, const int *batch, const void *const *in, void *const *out, int ngroups, bool fwd,
              cudaStream_t s) {
  if (ngroups < 1 || ngroups > FFT_MAXG) return DCCM_ERR_UNSUPPORTED;
  // Warps per CTA (the fft_bb knob); each group fits as many row pairs as
  // its warps per row allow (a power of two), within the smem budget.  The
  // fft_rpw knob (2) gives each warp (group of W warps) two row pairs in
  // turn: half the warps for the same row pairs, twice the field-levels a
  // CTA (W = 3 rows keep one row pair a group).
  const size_t budget = 110 * 1024;  // two CTAs an SM
  const int tb = tunables().fft_bb;
  const int WPC = (tb == 4 || tb == 8 || tb == 16) ? tb : 8;
  const int rpw = tunables().fft_rpw == 2 ? 2 : 1;
  int rmax = 2, warps = 1;
  for (int g = 0; g < ngroups; ++g)
    if (!fft_length_supported(plans[g]->I)) return DCCM_ERR_UNSUPPORTED;
  FftLaunch L;
  memset(&L, 0, sizeof L);
  int nblk = 0, ng = 0;
  size_t smem = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (batch[g] <= 0) continue;
    const Plan &P = *plans[g];
    const int R = P.I / 32, W = fft_warps_per_row(R);
    const int rp = W == 3 ? 1 : rpw;
    int BB = 1;
    while (2 * BB * W <= WPC * rp && fft_smem(R, 2 * BB, WPC / W) <= budget) BB *= 2;
    int lbb = 0;
    while ((1 << lbb) < BB) ++lbb;
    rmax = R > rmax ? R : rmax;
    const int wg = (BB * W + rp - 1) / rp;
    warps = wg > warps ? wg : warps;
    FftGroup &G = L.g[ng++];
    G.N = P.N;
    G.J = P.J;
    G.batch = batch[g];
    G.BB = BB;
    G.lbb = lbb;
    G.W = W;
    G.R = R;
    G.blk0 = nblk;
    G.C2Bp = P.C2Bp;
    G.in = in[g];
    G.out = out[g];
    G.tw = P.d_tw32;
    G.twl = P.d_twl32;
    G.nsplit = P.nsplit;
    G.cexp = P.d_cexp ? P.d_cexp + P.max_batch : nullptr;
    if (fwd && P.nsplit == 2)
      DCCM_TRY(field_exponents(static_cast<const double *>(in[g]), (long long)P.J * P.I, batch[g], P.d_cexp + P.max_batch, s));
    nblk += P.Jh * ((batch[g] + BB - 1) / BB);
  }
  L.ngroups = ng;
  // the kernel forms warps / W groups of W warps whatever this group needed
  for (int g = 0; g < ng; ++g) {
    const size_t sm = fft_smem(L.g[g].R, L.g[g].BB, warps / L.g[g].W);
    smem = sm > smem ? sm : smem;
  }
  if (nblk == 0) return DCCM_OK;
  auto go = [&](auto kernel) -> int {
    DCCM_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DCCM_CUDA(launch_pdl(kernel, dim3(nblk), dim3(32 * warps), smem, s, L));
    return DCCM_OK;
  };
  bool one = true;  // every group of the same length
  for (int g = 1; g < ng; ++g) one = one && L.g[g].R == L.g[0].R;
  if (one) {
#define DCCM_FFT_FIX(RR) \
  case RR: return fwd ? go(fft_multi_kernel<RR, 32, true>) : go(fft_multi_kernel<RR, 32, false>);
    switch (L.g[0].R) {
      DCCM_FFT_FIX(2) DCCM_FFT_FIX(3) DCCM_FFT_FIX(4) DCCM_FFT_FIX(6) DCCM_FFT_FIX(8)
      DCCM_FFT_FIX(12) DCCM_FFT_FIX(16) DCCM_FFT_FIX(24) DCCM_FFT_FIX(32)
      default: return DCCM_ERR_UNSUPPORTED;
    }
#undef DCCM_FFT_FIX
  }
  if (rmax <= 8) return fwd ? go(fft_multi_kernel<0, 8, true>) : go(fft_multi_kernel<0, 8, false>);
  return fwd ? go(fft_multi_kernel<0, 32, true>) : go(fft_multi_kernel<0, 32, false>);
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
