// omhd_fastmath.h -- FP64 reciprocal and reciprocal square root by
// Newton-Raphson from hardware approximations (device code).
#pragma once

namespace omhd {

// ---------------------------------------------------------------------------
// FP64 division and square root on a GPU whose FP64 pipe issues ~0.5 T
// instructions/s: an IEEE divide costs ~8.5 FP64-pipe instructions and a
// square root ~10.  The performance variants (FAST = true) replace them by
// Newton-Raphson iterations (Newton's method for f(y) = 1/y - x and
// f(y) = 1/y^2 - x, quadratic convergence) started from hardware
// approximations: rcp.approx.ftz.f64 (the special-function unit, ~20 bits)
// and rsqrt.approx.ftz.f32 on the float-rounded argument (~22 bits).  Two
// iterations give ~1 ulp; one reciprocal or one rsqrt is shared by every use
// of the same denominator.  The parity variant (FAST = false) keeps the
// reference's IEEE operations.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
  const float xf = (float)x;
  if (!(xf > 1.0e-37f && xf < 1.0e37f)) return 1.0 / sqrt(x);  // outside the float seed's range
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(xf));
  double y = (double)y0;
  double e = fma(-x * y, y, 1.0);
  y = fma(0.5 * y, e, y);
  e = fma(-x * y, y, 1.0);
  return fma(0.5 * y, e, y);
}
#endif

}  // namespace omhd
