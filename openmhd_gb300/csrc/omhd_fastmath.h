// omhd_fastmath.h -- FP64 reciprocal and reciprocal square root by
// Newton-Raphson from hardware approximations (device code).
#pragma once

namespace omhd {

// ---------------------------------------------------------------------------
// FP64 division and square root on a GPU whose FP64 pipe issues ~0.5 T
// instructions/s: an IEEE divide costs ~8.5 FP64-pipe instructions and a
// square root ~10.  The performance variants (FAST = true) replace them by
// one higher-order refinement of a hardware approximation:
//   rcp_nr   : y0 = rcp.approx.ftz.f64(x) (the special-function unit, ~20
//              bits), e = 1 - x*y0 (one FMA, exact), then
//              1/x = y0/(1-e) = y0*(1 + e + e^2 + O(e^3)): 3 FP64 operations,
//              truncation ~e^3 ~ 2^-60 (the geometric series of 1/(1-e));
//   rsqrt_nr : r0 = rsqrt.approx.ftz.f32 of the float-rounded argument (~22
//              bits), e = 1 - x*r0^2, then
//              1/sqrt(x) = r0*(1-e)^(-1/2) = r0*(1 + e/2 + 3e^2/8 + O(e^3)):
//              5 FP64 operations, truncation ~(5/16)e^3 ~ 2^-66 (binomial
//              series).
// Both return the double nearest the true value to within ~1 ulp (two
// Newton-Raphson steps, the textbook alternative, cost 4 and 8 operations).
// One reciprocal or one rsqrt is shared by every use of the same
// denominator.  The parity variant (FAST = false) keeps the reference's IEEE
// operations.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(fma(e, e, e), y, y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
  const float xf = (float)x;
  if (!(xf > 1.0e-37f && xf < 1.0e37f)) return 1.0 / sqrt(x);  // outside the float seed's range
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(xf));
  const double r = (double)y0;
  const double e = fma(-(x * r), r, 1.0);
  return fma(r * e, fma(0.375, e, 0.5), r);
}
#endif

}  // namespace omhd
