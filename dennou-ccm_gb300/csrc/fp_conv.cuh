// FP32 <-> FP64 conversions on the integer pipes.
//
// On GB300 the FP64 pipe is a small fraction of the FP32 one, and the
// hardware conversion instructions between double and float run on it.
// The mixed-precision kernels convert every grid value and spectral
// coefficient once, so they use these bit-level IEEE-754 conversions
// instead (integer ALU and moves only).  Both are exact restatements of
// the IEEE rules: widening is exact; narrowing rounds to nearest, ties to
// even.  Operands outside the normal FP32 range (zero excepted), infinities
// and NaNs take the hardware instruction (the narrowing's in a call of its
// own).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace dccm {

__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned a = u & 0x7FFFFFFFu;
  if (a - 0x00800000u >= 0x7F000000u) {  // zero, subnormal, inf, nan
    if (a == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)f;
  }
  // exponent and mantissa move down 3 bits as one field; the bias grows by
  // 1023 - 127 = 896 (896 << 20 = 0x38000000)
  return __hiloint2double((int)(((a >> 3) + 0x38000000u) | (u & 0x80000000u)), (int)(u << 29));
}

// Operands outside FP32's normal range other than zero (subnormal results,
// overflow, inf, nan): the hardware instruction, in a call of its own so that
// the common path keeps a branch around it instead of issuing it predicated
// (it runs on the FP64 pipe).
static __device__ __noinline__ float f64_to_f32_special(double d) { return __double2float_rn(d); }

__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned hi = (unsigned)__double2hiint(d);
  // biased exponent e in [897, 1150]: the result is a normal FP32 number
  // (or rounds up to infinity at the top, as IEEE rounding does); zero
  // takes the hardware path with the other operands outside that range
  if ((hi & 0x7FF00000u) - 0x38100000u >= 0x0FE00000u) return f64_to_f32_special(d);
  // round to nearest, ties to even, at bit 29: adding 2^28 - 1 + lsb to
  // the 64-bit pattern carries out of the 29 dropped bits exactly when they
  // exceed half, or equal half with an odd lsb; a carry out of the mantissa
  // correctly increments the exponent
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned long long rb = b + (0x0FFFFFFFull + ((b >> 29) & 1ull));
  // (hi:lo) << 3 keeps e's low 9 bits above the top 23 mantissa bits;
  // subtracting 384 << 23 turns them into e - 896 (mod 512, which fits 8 bits)
  const unsigned r = __funnelshift_l((unsigned)rb, (unsigned)(rb >> 32), 3) - 0xC0000000u;
  return __uint_as_float(r | (hi & 0x80000000u));
}

// The same for inputs where zeros are common (padding, the imaginary parts
// of m = 0 coefficients): zero on the integer path, the rest as above.
__device__ __forceinline__ float f64_to_f32_rn_z(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  if (((hi << 1) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
  return f64_to_f32_rn(d);
}

// Exact split of an FP32 value into three BF16 numbers x = hi + mid + lo
// (FP32 arithmetic: each residual is exact because it has fewer
// significant bits than FP32), returned as raw bits.
__device__ __forceinline__ void split3f_bits(float x, unsigned short &h, unsigned short &m, unsigned short &l) {
  const __nv_bfloat16 bh = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(bh);
  const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
  const __nv_bfloat16 bl = __float2bfloat16_rn(r1 - __bfloat162float(bm));
  h = __bfloat16_as_ushort(bh);
  m = __bfloat16_as_ushort(bm);
  l = __bfloat16_as_ushort(bl);
}

// The same split for two values at once with the packed conversions (each
// half rounded as __float2bfloat16_rn rounds it, so the bits equal two
// split3f_bits calls); .x in the low 16 bits of each word.
__device__ __forceinline__ void split3f_x2(float2 x, unsigned &h, unsigned &m, unsigned &l) {
  const __nv_bfloat162 bh = __float22bfloat162_rn(x);
  const float2 fh = __bfloat1622float2(bh);
  const float2 r1 = make_float2(x.x - fh.x, x.y - fh.y);
  const __nv_bfloat162 bm = __float22bfloat162_rn(r1);
  const float2 fm = __bfloat1622float2(bm);
  const __nv_bfloat162 bl = __float22bfloat162_rn(make_float2(r1.x - fm.x, r1.y - fm.y));
  h = *reinterpret_cast<const unsigned *>(&bh);
  m = *reinterpret_cast<const unsigned *>(&bm);
  l = *reinterpret_cast<const unsigned *>(&bl);
}

// Split of an FP32 value into two FP16 numbers x ~ hi + lo (22 significant
// bits; the caller scales x by a power of two into FP16's range first),
// returned as raw bits.  The residual x - hi is exact in FP32.
__device__ __forceinline__ void split2h_bits(float x, unsigned short &h, unsigned short &l) {
  const __half hh = __float2half_rn(x);
  const __half hl = __float2half_rn(x - __half2float(hh));
  h = __half_as_ushort(hh);
  l = __half_as_ushort(hl);
}

// Two values at once (packed conversions; the same bits as split2h_bits).
__device__ __forceinline__ void split2h_x2(float2 x, unsigned &h, unsigned &l) {
  const __half2 hh = __float22half2_rn(x);
  const float2 fh = __half22float2(hh);
  const __half2 hl = __float22half2_rn(make_float2(x.x - fh.x, x.y - fh.y));
  h = *reinterpret_cast<const unsigned *>(&hh);
  l = *reinterpret_cast<const unsigned *>(&hl);
}

// 2^k as an FP32 number, for exponents of normal numbers (-126 <= k <= 127;
// clamped outside).
__device__ __forceinline__ float pow2f(int k) {
  k = k < -126 ? -126 : (k > 127 ? 127 : k);
  return __int_as_float((k + 127) << 23);
}

// x * 2^s for a normal double whose result stays normal, by exponent
// arithmetic on the integer pipes (exact); zero and subnormal x give 0.
__device__ __forceinline__ double scale_pow2(double x, int s) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0.0;
  int ne = e + s;
  ne = ne < 1 ? 1 : (ne > 2046 ? 2046 : ne);
  return __longlong_as_double((b & ~(0x7ffLL << 52)) | ((long long)ne << 52));
}

// Unbiased binary exponent of the largest |x| contributing to a power-of-two
// scale: floor(log2|x|) for normal doubles, -1023 for zero and subnormals.
__device__ __forceinline__ int f64_exponent(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}

}  // namespace dccm
