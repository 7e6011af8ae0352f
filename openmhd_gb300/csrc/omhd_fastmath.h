// omhd_fastmath.h -- FP64 reciprocal and reciprocal square root by
// Newton-Raphson from hardware approximations, and binary32 <-> binary64
// conversions on the integer pipe (device code).
#pragma once

namespace omhd {

// ---------------------------------------------------------------------------
// FP64 division and square root on a GPU whose FP64 pipe issues ~0.5 T
// instructions/s: an IEEE divide costs ~4.4 FP64-pipe instruction slots and a
// square root ~7 (measured on GB300).  The performance variants (FAST = true)
// replace them by one higher-order refinement of a hardware approximation
// from the special-function unit, which does not occupy the FP64 pipe:
//   rcp_nr   : y0 = rcp.approx.ftz.f64(x) (relative error <= 2^-19.9,
//              measured), e = 1 - x*y0 (one FMA, exact), then
//              1/x = y0/(1-e) = y0*(1 + e + e^2 + O(e^3)): 3 FP64 operations,
//              truncation ~e^3 ~ 2^-60 (the geometric series of 1/(1-e));
//   rsqrt_nr : r0 = rsqrt.approx.ftz.f64(x) (relative error <= 2^-20.0,
//              measured), e = 1 - x*r0^2, then
//              1/sqrt(x) = r0*(1-e)^(-1/2) = r0*(1 + e/2 + 3e^2/8 + O(e^3)):
//              5 FP64 operations, truncation ~(5/16)e^3 ~ 2^-62 (binomial
//              series);
//   sqrt_nr  : the same series applied to s0 = x*r0 ~ sqrt(x):
//              sqrt(x) = s0*(1-e)^(-1/2) with e = 1 - s0*r0, 5 FP64
//              operations.
// Each returns a double within 1 ulp of the correctly rounded value (two
// Newton-Raphson steps, the textbook alternative, cost 4 and 8 operations);
// tests/test_gpu_fastmath.py enforces the 1-ulp bound on the GPU over
// 2^-60..2^59 and over each function's whole domain.  The seeds flush
// subnormal arguments, so rsqrt_nr and sqrt_nr take the IEEE operation outside
// the positive normal range (a branch that the solver's positive normal
// arguments never take); rcp_nr has no such branch and is meant for
// |x| in [2^-1022, 2^1022] (x and 1/x normal); the solver's denominators
// (densities, wave-speed differences, star-state factors) lie far inside it.  The parity variant (FAST = false) keeps the reference's
// IEEE operations.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(fma(e, e, e), y, y);
}

// x positive, normal and finite (one integer compare on the bit pattern)
__device__ __forceinline__ bool pos_normal(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return b - 0x0010000000000000ULL < 0x7fe0000000000000ULL;
}

__device__ __forceinline__ double rsqrt_nr(double x) {
  if (!pos_normal(x)) return 1.0 / sqrt(x);
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-(x * r), r, 1.0);
  return fma(r * e, fma(0.375, e, 0.5), r);
}

__device__ __forceinline__ double sqrt_nr(double x) {
  if (!pos_normal(x)) return sqrt(x);
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double s = x * r;
  const double e = fma(-s, r, 1.0);
  return fma(s * e, fma(0.375, e, 0.5), s);
}

// ---------------------------------------------------------------------------
// binary32 <-> binary64 conversions on the integer pipe.  GB300 executes the
// F2F conversions on its FP64 pipe, one slot each like an FMA; the FP32-mixed
// kernels convert every loaded primitive to binary32 and every face flux back,
// which took a quarter of their FP64-pipe time.  These forms move the bits with
// 8-15 integer instructions instead (IEEE 754 formats: binary32 = 1/8/23 bits,
// bias 127; binary64 = 1/11/52 bits, bias 1023):
//   widen_f32  : exact for normal floats, +-0, +-inf and NaN (payload kept);
//                a subnormal float (|f| < 2^-126) becomes a signed zero.
//   narrow_f64 : round to nearest, ties to even, as cvt.rn.f32.f64, for every
//                argument of magnitude 2^-126 or more, with overflow to
//                +-inf; a smaller argument gives a signed zero (no subnormal
//                results); NaN stays NaN (quiet).
// tests/test_gpu_convert.py checks both against IEEE conversions on the host,
// bit for bit, over random bit patterns and every boundary of the formats;
// tests/test_convert_algorithm.py restates the bit manipulation in numpy and
// checks it the same way without a GPU.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned mag = u & 0x7fffffffu;
  // rebias the exponent: + (1023 - 127) in the high word's exponent field, and
  // twice that for inf/NaN so that exponent 255 lands on 2047
  unsigned hi = (mag >> 3) + (mag >= 0x7f800000u ? 0x70000000u : 0x38000000u);
  unsigned lo = u << 29;  // the three low mantissa bits
  if (mag < 0x00800000u) hi = lo = 0u;
  return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}

__device__ __forceinline__ float narrow_f64(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ahi = hi & 0x7fffffffu;
  // round the 64-bit magnitude at bit 29: add half an ulp of the result minus
  // one, plus the kept lowest bit (ties go to even), then drop 29 bits
  const unsigned long long a = ((unsigned long long)ahi << 32) | lo;
  const unsigned long long r = a + (0x0fffffffull + ((lo >> 29) & 1u));
  unsigned f = (unsigned)(r >> 29) - (896u << 23);  // rebias 1023 -> 127
  f = ahi >= 0x47f00000u ? 0x7f800000u : f;         // |x| >= 2^128: inf (also inf/NaN inputs)
  f = ahi < 0x38100000u ? 0u : f;                   // |x| < 2^-126: zero
  f = a > 0x7ff0000000000000ull ? 0x7fc00000u : f;  // NaN
  return __uint_as_float(f | (hi & 0x80000000u));
}
#endif

}  // namespace omhd
