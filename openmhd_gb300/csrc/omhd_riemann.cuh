// omhd_riemann.cuh -- face reconstruction (slope limiters) and numerical
// fluxes, as device templates over the arithmetic type T (double or float)
// and the face direction DIR (1,2,3).
//
// Face states use the reference's VL/VR slot order (main.f90:91-99):
//   w = (vx, vy, vz, p, rho, Bx, By, Bz, psi)
// and fluxes the conserved slot order (mx, my, mz, E, rho, Bx, By, Bz, psi).
// Every formula keeps the reference's operation order so that a translation
// unit built with --fmad=false reproduces the reference arithmetic exactly;
// the performance build of the same source lets the compiler contract
// multiply-adds.
#pragma once
#include "omhd_common.cuh"
#include "omhd_fastmath.h"
#include "omhd_tape.h"

namespace omhd {

// Comparisons of the FP64 performance variants on the integer pipe (the FP64
// pipe is the bottleneck; a floating-point compare or min/max occupies it like
// an FMA).  Each returns the IEEE comparison's truth value (signed zeros
// compare equal; NaN does not occur on the path), so results are bit-identical.
__device__ __forceinline__ long long okey(double x) {  // order-preserving integer key
  long long b = __double_as_longlong(x);
  b = (b == (long long)0x8000000000000000ULL) ? 0 : b;  // -0 == +0
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
template <class T, bool FAST>
__device__ __forceinline__ bool ge0_(T x) {  // x >= 0
  if constexpr (FAST && sizeof(T) == 8) {
    const long long b = __double_as_longlong(double(x));
    return b >= 0 || b == (long long)0x8000000000000000ULL;
  }
  return x >= T(0);
}
template <class T, bool FAST>
__device__ __forceinline__ bool le0_(T x) {  // x <= 0
  if constexpr (FAST && sizeof(T) == 8) return __double_as_longlong(double(x)) <= 0;
  return x <= T(0);
}
template <class T, bool FAST>
__device__ __forceinline__ bool lt0_(T x) {  // x < 0
  if constexpr (FAST && sizeof(T) == 8) {
    const long long b = __double_as_longlong(double(x));
    return b < 0 && b != (long long)0x8000000000000000ULL;
  }
  return x < T(0);
}
template <bool FAST>
__device__ __forceinline__ bool gt0_(double x) {  // x > 0 (false for NaN, as the IEEE compare)
  if constexpr (FAST) {
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
  }
  return x > 0.0;
}
template <class T, bool FAST>
__device__ __forceinline__ bool lt_(T a, T b) {  // a < b
  if constexpr (FAST && sizeof(T) == 8) return okey(double(a)) < okey(double(b));
  return a < b;
}

// a / b and 1 / b under the variant's policy
template <class T, bool FAST>
__device__ __forceinline__ T rcp_(T b) {
  if constexpr (FAST && sizeof(T) == 8) return rcp_nr(b);
  return T(1) / b;
}
template <class T, bool FAST>
__device__ __forceinline__ T div_(T a, T b) {
  if constexpr (FAST && sizeof(T) == 8) return a * rcp_nr(b);
  return a / b;
}
// square root under the variant's policy: sqrt_nr for FAST FP64 (5 FP64-pipe
// operations instead of ~7 for the IEEE sqrt; within ~1 ulp; IEEE outside the
// positive normal range, so sqrt(+-0) = +-0)
template <class T, bool FAST>
__device__ __forceinline__ T sqrt_(T x) {
  if constexpr (FAST && sizeof(T) == 8) return sqrt_nr(x);
  return sqrt(x);
}
// sqrt(a / b) for a, b > 0: a * (1/sqrt(a*b)) for FAST FP64 (one product and
// one rsqrt refinement replace a division and a square root), IEEE otherwise
template <class T, bool FAST>
__device__ __forceinline__ T sqrt_ratio_(T a, T b) {
  if constexpr (FAST && sizeof(T) == 8) {
    const double ab = a * b;
    return pos_normal(ab) ? a * rsqrt_nr(ab) : sqrt(a / b);
  }
  return sqrt(a / b);
}
// a / b given rb = rcp_<T,FAST>(b) computed once for several numerators
template <class T, bool FAST>
__device__ __forceinline__ T divr_(T a, T b, T rb) {
  if constexpr (FAST && sizeof(T) == 8) return a * rb;
  return a / b;
}

// primitive (FP64) -> the face arithmetic's type T, and face flux -> FP64: the
// FP32-mixed kernels convert on the integer pipe (omhd_fastmath.h), the FP64
// kernels pass the value through
template <class T>
__device__ __forceinline__ T to_face(double x) {
  if constexpr (sizeof(T) == 4)
    return narrow_f64(x);
  else
    return x;
}
template <class T>
__device__ __forceinline__ double to_f64(T x) {
  if constexpr (sizeof(T) == 4)
    return widen_f32(x);
  else
    return x;
}

enum { LM_FLAT = 0, LM_MINMOD = 1, LM_MC = 2, LM_VANLEER = 3, LM_KOREN = 4 };
enum { FX_LLF = 0, FX_HLL = 1, FX_HLLC = 2, FX_HLLD = 3, FX_LHLLD = 4 };

// Slope-limited reconstruction of one cell (2D_basic/limiter.f90):
//   right = state at the cell's lower face   (wR(i-1) in the reference)
//   left  = state at the cell's upper face   (wL(i)   in the reference)
// minmod :98, MC :141-158, van Leer :201-210, Koren :256-272, flat :54-71.
template <class T>
__device__ __forceinline__ void reconstruct(int type, T wm, T w0, T wp, T& left, T& right) {
  const T gA = (w0 - wm);
  const T gB = (wp - w0);
  T grad;
  switch (type) {
    case LM_MINMOD:
      grad = (fsign(T(0.25), gA) + fsign(T(0.25), gB)) * fmin2(fabs(gA), fabs(gB));
      right = w0 - grad;
      left = w0 + grad;
      break;
    case LM_MC: {
      const T gC = T(0.25) * (wp - wm);
      grad = (fsign(T(0.5), gA) + fsign(T(0.5), gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      right = w0 - grad;
      left = w0 + grad;
      break;
    }
    case LM_VANLEER:
      if (gA * gB <= T(0))
        grad = T(0);
      else
        grad = gA * gB / (gA + gB);
      right = w0 - grad;
      left = w0 + grad;
      break;
    case LM_KOREN: {
      const T f6 = T(1) / T(6);
      T gC = f6 * (2 * gA + gB);
      right = w0 - (fsign(T(0.5), gA) + fsign(T(0.5), gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      gC = f6 * (gA + 2 * gB);
      left = w0 + (fsign(T(0.5), gA) + fsign(T(0.5), gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      break;
    }
    default:  // flat: the state itself on both faces
      right = w0;
      left = w0;
  }
}

// Minimum of two non-negative doubles on the integer pipe: for x, y >= 0 the
// order of the IEEE bit patterns is the numeric order.
__device__ __forceinline__ double min_nonneg(double a, double b) {
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  return (ib < ia) ? b : a;  // same operand choice as fmin2(a, b)
}

// The FAST minmod / MC reconstruction of reconstruct_fp64 from the slopes
// gA = w0 - wm and gB = wp - w0 (computed once for two neighbouring cells,
// whose gB and gA are the same difference); records the selection under
// TAPE = tape::kRecord
template <int TAPE = tape::kNone>
__device__ __forceinline__ void reconstruct_fp64_g(int type, double gA, double gB, double wm, double w0, double wp,
                                                   double& left, double& right, unsigned char* code = nullptr) {
  const long long sa = __double_as_longlong(gA), sb = __double_as_longlong(gB);
  const long long ia = __double_as_longlong(fabs(gA)), ib = __double_as_longlong(fabs(gB));
  double m = min_nonneg(fabs(gA), fabs(gB));
  double c = 0.5;  // minmod: (0.25 + 0.25)
  bool pickC = false;
  double gC = 0.0;
  if (type == LM_MC) {
    gC = 0.25 * (wp - wm);
    const long long ic = __double_as_longlong(fabs(gC));
    pickC = ic < __double_as_longlong(m);
    m = min_nonneg(m, fabs(gC));
    c = 1.0;  // MC: (0.5 + 0.5)
  }
  const bool zero = (sa ^ sb) < 0;
  const double s = zero ? 0.0 : copysign(c, gA);
  left = fma(s, m, w0);
  right = fma(-s, m, w0);
  if constexpr (TAPE == tape::kRecord) {
    unsigned char k;
    if (zero)
      k = tape::kLimZero;
    else if (pickC)
      k = (unsigned char)(tape::kLimC | (((sa ^ __double_as_longlong(gC)) < 0) ? tape::kLimCNeg : 0));
    else
      k = (ib < ia) ? tape::kLimB : tape::kLimA;
    *code = k;
  }
}

// minmod and MC reconstruction for FP64 with the sign logic and the minimum
// on the integer pipe.  (sign(c,gA)+sign(c,gB)) is 0 when the signs differ and
// +-2c otherwise, and 2c*min(...) is an exact power-of-two scaling, so the face
// states equal the reference's bit for bit: w0 +- (+-2c)*m is one fused
// multiply-add with an exactly representable product.
//
// Under a decision tape (TAPE = tape::kRecord / kReplay, minmod and MC only)
// the selection is recorded in *code, or taken from it: a replayed selection
// is applied as the linear map it stands for (c*gA, c*gB or +-gC), which
// equals the recorded arithmetic bit for bit while no slope changes sign.
template <bool FAST, int TAPE = tape::kNone>
__device__ __forceinline__ void reconstruct_fp64(int type, double wm, double w0, double wp, double& left,
                                                 double& right, unsigned char* code = nullptr) {
  if constexpr (TAPE == tape::kReplay) {
    const double c = (type == LM_MC) ? 1.0 : 0.5;
    const unsigned char k = *code;
    double sel = 0.0, cc = c;
    switch (k & 3) {
      case tape::kLimA: sel = w0 - wm; break;
      case tape::kLimB: sel = wp - w0; break;
      case tape::kLimC:
        sel = 0.25 * (wp - wm);
        if (k & tape::kLimCNeg) cc = -c;
        break;
      default: cc = 0.0;
    }
    left = fma(cc, sel, w0);
    right = fma(-cc, sel, w0);
    return;
  }
  if constexpr (FAST) {
    if (type == LM_MINMOD || type == LM_MC) {
      reconstruct_fp64_g<TAPE>(type, w0 - wm, wp - w0, wm, w0, wp, left, right, code);
      return;
    }
  }
  reconstruct<double>(type, wm, w0, wp, left, right);
}

template <class T, bool FAST>
__device__ __forceinline__ void reconstruct_t(int type, T wm, T w0, T wp, T& left, T& right) {
  if constexpr (sizeof(T) == 8)
    reconstruct_fp64<FAST>(type, wm, w0, wp, left, right);
  else
    reconstruct<T>(type, wm, w0, wp, left, right);
}

// HLLD intermediate (star) state of one side (flux_solver.f90:482-493 for L,
// :496-507 for R, the same expressions with the side's values): side state
// rho, normal / tangential velocities, tangential fields, wave speed a, total
// energy E, total pressure pts, v.B, star density ros = rho*(a - un)/(a - aM)
// and ie = 1/(a - aM); returns the star state's conserved variables in S and
// its tangential velocities in v1, v2.
template <class T, bool FAST, int vn, int vt1, int vt2, int bt1, int bt2, int mn, int mt1, int mt2>
__device__ __forceinline__ void star_state(T ro, T un, T ut1, T ut2, T b1, T b2, T a, T E, T pts, T vB, T ros, T ie,
                                           T aM, T pt, T Bn, T (&S)[NV], T& v1, T& v2) {
  const T t = a - un;
  const T f = rcp_<T, FAST>(ro * t * (a - aM) - Bn * Bn);
  const T fb = f * (ro * (t * t) - Bn * Bn);  // B_t* = B_t fb, v_t* = v_t - B_t fv
  const T fv = f * Bn * (aM - un);
  S[bt1] = b1 * fb;
  S[bt2] = b2 * fb;
  v1 = ut1 - fv * b1;
  v2 = ut2 - fv * b2;
  S[RO] = ros;
  S[EN] = divr_<T, FAST>((t * E - pts * un + pt * aM + Bn * (vB - aM * Bn - v1 * S[bt1] - v2 * S[bt2])), (a - aM), ie);
  S[mn] = ros * aM;
  S[mt1] = ros * v1;
  S[mt2] = ros * v2;
}

// Per-side quantities of the FP64 HLLD solver (flux_solver.f90:359-401)
// that both sides need: conserved normal momentum, normal momentum flux,
// total pressure and the numerator of the fast speed squared,
// cf^2 = num / (2 rho); the conserved energy and v.B (UE, vB) are filled in
// by hlld_side_e for the sides whose star state or flux is built.
struct HSide {
  double B2, vB, Umn, UE, Fmn, pt, num;
};

template <int DIR, int TAPE>
__device__ __forceinline__ HSide hlld_side(const double (&S)[NV], double gamma, double r1, unsigned* code,
                                           unsigned clamp_bit) {
  constexpr int vn = VX + (DIR - 1) % 3, bn = BX + (DIR - 1) % 3;
  HSide o;
  o.B2 = S[BX] * S[BX] + S[BY] * S[BY] + S[BZ] * S[BZ];
  o.vB = 0.0;
  o.UE = 0.0;
  o.Umn = S[RO] * S[vn];
  o.pt = S[PR] + 0.5 * o.B2;
  o.Fmn = o.Umn * S[vn] + o.pt - S[bn] * S[bn];  // rho vn^2 + pt - bn^2
  const double f1 = gamma * S[PR], f2 = 4 * (S[bn] * S[bn]);
  const double D = (f1 + o.B2) * (f1 + o.B2) - f1 * f2;
  const bool cl = tape::decide<TAPE>(lt0_<double, true>(D), code, clamp_bit);  // fmax2(D, 0)
  o.num = (f1 + o.B2) + sqrt_nr(cl ? 0.0 : D);
  return o;
}

// conserved energy and v.B of one side (flux_solver.f90:360-362)
__device__ __forceinline__ void hlld_side_e(const double (&S)[NV], double r1, HSide& o) {
  const double v2 = S[VX] * S[VX] + S[VY] * S[VY] + S[VZ] * S[VZ];
  o.vB = S[VX] * S[BX] + S[VY] * S[BY] + S[VZ] * S[BZ];
  o.UE = 0.5 * (S[RO] * v2 + o.B2) + r1 * S[PR];
}

// the physical flux of one side from its primitive state and HSide values
template <int DIR>
__device__ __forceinline__ void hlld_phys_flux(const double (&S)[NV], const HSide& h, double (&F)[NV]) {
  constexpr int vn = VX + (DIR - 1) % 3, vt1 = VX + DIR % 3, vt2 = VX + (DIR + 1) % 3;
  constexpr int bn = BX + (DIR - 1) % 3, bt1 = BX + DIR % 3, bt2 = BX + (DIR + 1) % 3;
  constexpr int mn = MX + (DIR - 1) % 3, mt1 = MX + DIR % 3, mt2 = MX + (DIR + 1) % 3;
  F[RO] = h.Umn;
  F[mn] = h.Fmn;
  F[mt1] = h.Umn * S[vt1] - S[bn] * S[bt1];
  F[mt2] = h.Umn * S[vt2] - S[bn] * S[bt2];
  F[EN] = (h.UE + h.pt) * S[vn] - h.vB * S[bn];  // (E + pt) vn - (v.B) bn
  F[bt1] = S[vn] * S[bt1] - S[bn] * S[vt1];
  F[bt2] = S[vn] * S[bt2] - S[bn] * S[vt2];
  F[bn] = 0.0;
  F[PS] = 0.0;
}

// HLLD flux of the FAST FP64 variant (flux_solver.f90:352-585, HLLC-G
// fallback :447-476, GLM fluxes :580-581).  Same mathematics and decisions as
// riemann_flux<double, DIR, FX_HLLD>; its work is cut to what the face's
// region uses: per side only the quantities both sides need (the conserved
// normal momentum and energy, the normal momentum flux, total pressure and
// the fast-speed numerator); the HLL average only for rho, the normal momentum
// and Bn (the tangential components serve the HLLC-G fallback alone); the
// physical flux and the star state of the side s the region uses, from
// side-selected inputs (the central region adds the other side's star state).
template <int DIR, int TAPE>
__device__ __forceinline__ void hlld_f64(const double (&L)[NV], const double (&R)[NV], double ch, double gamma,
                                         double r1, double r2, double (&Fo)[NV], unsigned* code_io) {
  using tape::decide;
  unsigned code_reg = (TAPE == tape::kReplay) ? *code_io : 0u;
  unsigned* const code = &code_reg;
  constexpr int vn = VX + (DIR - 1) % 3, vt1 = VX + DIR % 3, vt2 = VX + (DIR + 1) % 3;
  constexpr int bn = BX + (DIR - 1) % 3, bt1 = BX + DIR % 3, bt2 = BX + (DIR + 1) % 3;
  constexpr int mn = MX + (DIR - 1) % 3, mt1 = MX + DIR % 3, mt2 = MX + (DIR + 1) % 3;
  (void)r2;
  HSide hL = hlld_side<DIR, TAPE>(L, gamma, r1, code, tape::kClampL);
  HSide hR = hlld_side<DIR, TAPE>(R, gamma, r1, code, tape::kClampR);
  // largest fast speed: cf^2 = num / (2 rho), numL/rhoL < numR/rhoR <=> numL*rhoR < numR*rhoL
  const bool sr = decide<TAPE>(lt_<double, true>(hL.num * R[RO], hR.num * L[RO]), code, tape::kArSel);
  const double cf = sqrt_ratio_<double, true>(sr ? hR.num : hL.num, 2 * (sr ? R[RO] : L[RO]));
  const double aL = (decide<TAPE>(lt_<double, true>(R[vn], L[vn]), code, tape::kMinR) ? R[vn] : L[vn]) - cf;
  const double aR = (decide<TAPE>(lt_<double, true>(L[vn], R[vn]), code, tape::kMaxR) ? R[vn] : L[vn]) + cf;
  if (decide<TAPE>(ge0_<double, true>(aL), code, tape::kFL)) {
    hlld_side_e(L, r1, hL);
    hlld_phys_flux<DIR>(L, hL, Fo);
  } else if (decide<TAPE>(le0_<double, true>(aR), code, tape::kFR)) {
    hlld_side_e(R, r1, hR);
    hlld_phys_flux<DIR>(R, hR, Fo);
  } else {
    // HLL average (:408-417) of rho, the normal momentum and Bn
    const double f1 = rcp_nr(aR - aL);
    const double tL = aL - L[vn], tR = aR - R[vn];
    const double rtL = L[RO] * tL, rtR = R[RO] * tR;  // rho (a - vn) = a*rho - F[rho]
    const double UhRO = f1 * (rtR - rtL);
    const double Uhmn = f1 * ((aR * hR.Umn - hR.Fmn) - (aL * hL.Umn - hL.Fmn));
    const double Ubn = f1 * (aR * R[bn] - aL * L[bn]);
    const double aM = Uhmn * rcp_nr(UhRO);
    const double pt = hL.pt + rtL * (aM - L[vn]);
    const double ieL = rcp_nr(aL - aM), ieR = rcp_nr(aR - aM);
    const double roL = rtL * ieL, roR = rtR * ieR;
    const bool bneg = decide<TAPE>(signbit(Ubn) != 0, code, tape::kBnNeg);
    const double aBn = (TAPE == tape::kNone) ? fabs(Ubn) : (bneg ? -Ubn : Ubn);
    // Alfven speeds aV = |Bn|/sqrt(rho*) enter the HLLC-G switch and the region
    // only through comparisons, which are made on squares (no square root
    // unless the central states need sqrt(rho*)):
    //   aL >= aM - h aV_L  <=>  aM - aL <= 0  or  h^2 Bn^2 >= (aM - aL)^2 rho*_L
    //   aM + h aV_R >= aR  <=>  aR - aM <= 0  or  h^2 Bn^2 >= (aR - aM)^2 rho*_R
    const double hllg = 1.001;
    const double Bn2 = Ubn * Ubn, hB2 = (hllg * hllg) * Bn2;
    const double cL = aM - aL, cR = aR - aM;
    if (decide<TAPE>(le0_<double, true>(cL) || !lt_<double, true>(hB2, (cL * cL) * roL) ||
                         le0_<double, true>(cR) || !lt_<double, true>(hB2, (cR * cR) * roR),
                     code, tape::kG)) {
      // HLLC-G fallback :450-476 (rare): the tangential HLL components and
      // both physical fluxes
      hlld_side_e(L, r1, hL);
      hlld_side_e(R, r1, hR);
      double FL[NV], FR[NV];
      hlld_phys_flux<DIR>(L, hL, FL);
      hlld_phys_flux<DIR>(R, hR, FR);
      const double ULt1 = L[RO] * L[vt1], ULt2 = L[RO] * L[vt2], URt1 = R[RO] * R[vt1], URt2 = R[RO] * R[vt2];
      const double Uhmt1 = f1 * (aR * URt1 - aL * ULt1 - FR[mt1] + FL[mt1]);
      const double Uhmt2 = f1 * (aR * URt2 - aL * ULt2 - FR[mt2] + FL[mt2]);
      const double Uhbt1 = f1 * (aR * R[bt1] - aL * L[bt1] - FR[bt1] + FL[bt1]);
      const double Uhbt2 = f1 * (aR * R[bt2] - aL * L[bt2] - FR[bt2] + FL[bt2]);
      const double f2 = aL * aR;
      Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
      Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
      const double iUr = rcp_nr(UhRO);
      const double at1 = Uhmt1 * iUr, at2 = Uhmt2 * iUr;
      const double enL = ((aL - L[vn]) * hL.UE - hL.pt * L[vn] + pt * aM +
                          Ubn * (hL.vB - aM * Ubn - at1 * Uhbt1 - at2 * Uhbt2)) * ieL;
      const double enR = ((aR - R[vn]) * hR.UE - hR.pt * R[vn] + pt * aM +
                          Ubn * (hR.vB - aM * Ubn - at1 * Uhbt1 - at2 * Uhbt2)) * ieR;
      const double g1 = (TAPE != tape::kNone) ? (decide<TAPE>(signbit(aM) == 0, code, tape::kGLeft) ? 1.0 : 0.0)
                                              : 0.5 + fsign(0.5, aM);  // 0.5 + sign(0.5, aM)
      const double g2 = 1.0 - g1;
      Fo[mn] = g1 * (aL * (roL * aM - hL.Umn) + FL[mn]) + g2 * (aR * (roR * aM - hR.Umn) + FR[mn]);
      Fo[mt1] = g1 * (aL * (roL * at1 - ULt1) + FL[mt1]) + g2 * (aR * (roR * at1 - URt1) + FR[mt1]);
      Fo[mt2] = g1 * (aL * (roL * at2 - ULt2) + FL[mt2]) + g2 * (aR * (roR * at2 - URt2) + FR[mt2]);
      Fo[EN] = g1 * (aL * (enL - hL.UE) + FL[EN]) + g2 * (aR * (enR - hR.UE) + FR[EN]);
      Fo[RO] = g1 * (aL * (roL - L[RO]) + FL[RO]) + g2 * (aR * (roR - R[RO]) + FR[RO]);
    } else {
      // region (:482-572), then the side s whose state the flux uses
      //   aL1 = aM - aV_L >= 0  <=>  aM >= 0 and aM^2 rho*_L >= Bn^2
      //   aR1 = aM + aV_R <= 0  <=>  aM <= 0 and aM^2 rho*_R >= Bn^2
      const double aM2 = aM * aM;
      const bool sLs = decide<TAPE>(ge0_<double, true>(aM) && !lt_<double, true>(aM2 * roL, Bn2), code, tape::kLS);
      const bool sRs =
          !sLs && decide<TAPE>(le0_<double, true>(aM) && !lt_<double, true>(aM2 * roR, Bn2), code, tape::kRS);
      const bool cen = !sLs && !sRs;
      const bool sR = sRs || (cen && !decide<TAPE>(ge0_<double, true>(aM), code, tape::kSSLeft));
      double Ss[NV];  // side primitive state
#pragma unroll
      for (int v = 0; v < NV; ++v) Ss[v] = sR ? R[v] : L[v];
      HSide hs;
      hs.B2 = sR ? hR.B2 : hL.B2;
      hs.Umn = sR ? hR.Umn : hL.Umn;
      hs.Fmn = sR ? hR.Fmn : hL.Fmn;
      hs.pt = sR ? hR.pt : hL.pt;
      hlld_side_e(Ss, r1, hs);
      const double as = sR ? aR : aL;
      double S1[NV] = {}, vs1, vs2;
      star_state<double, true, vn, vt1, vt2, bt1, bt2, mn, mt1, mt2>(
          Ss[RO], Ss[vn], Ss[vt1], Ss[vt2], Ss[bt1], Ss[bt2], as, hs.UE, hs.pt, hs.vB, sR ? roR : roL,
          sR ? ieR : ieL, aM, pt, Ubn, S1, vs1, vs2);
      double Fs[NV], Us[NV];  // the side's physical flux and state (conserved MX..EN, primitive rho and B)
      hlld_phys_flux<DIR>(Ss, hs, Fs);
      Us[mn] = hs.Umn;
      Us[mt1] = Ss[RO] * Ss[vt1];
      Us[mt2] = Ss[RO] * Ss[vt2];
      Us[EN] = hs.UE;
      Us[RO] = Ss[RO];
      Us[bt1] = Ss[bt1];
      Us[bt2] = Ss[bt2];
      if (!cen) {  // F(L*) :514-519 / F(R*) :522-527
#pragma unroll
        for (int v = MX; v <= EN; ++v) Fo[v] = as * (S1[v] - Us[v]) + Fs[v];
        Fo[RO] = as * (S1[RO] - Us[RO]) + Fs[RO];
        Fo[bt1] = as * (S1[bt1] - Us[bt1]) + Fs[bt1];
        Fo[bt2] = as * (S1[bt2] - Us[bt2]) + Fs[bt2];
      } else {  // central states :533-572, symmetric in (s, o); sigma = +1 for s = L, -1 for s = R
        double So[NV];  // the other side's primitive state
#pragma unroll
        for (int v = 0; v < NV; ++v) So[v] = sR ? L[v] : R[v];
        HSide ho;
        ho.B2 = sR ? hL.B2 : hR.B2;
        ho.pt = sR ? hL.pt : hR.pt;
        hlld_side_e(So, r1, ho);
        double O1[NV] = {}, vo1, vo2;
        star_state<double, true, vn, vt1, vt2, bt1, bt2, mn, mt1, mt2>(
            So[RO], So[vn], So[vt1], So[vt2], So[bt1], So[bt2], sR ? aL : aR, ho.UE, ho.pt, ho.vB,
            sR ? roL : roR, sR ? ieL : ieR, aM, pt, Ubn, O1, vo1, vo2);
        const double ros = sR ? roR : roL, roo = sR ? roL : roR;
        const double rsS = rsqrt_nr(ros), rsO = rsqrt_nr(roo);  // 1/sqrt(rho*) of s and o
        const double rss = ros * rsS, rso = roo * rsO;          // sqrt(rho*) of s and o
        const double fc = rcp_nr(rss + rso);
        const double f2 = (TAPE == tape::kNone) ? fsign(1.0, Ubn) : (bneg ? -1.0 : 1.0);
        const double f2s = sR ? -f2 : f2;
        double U2[NV];
        const double at1 = fc * (rss * vs1 + rso * vo1 + (O1[bt1] - S1[bt1]) * f2s);
        const double at2 = fc * (rss * vs2 + rso * vo2 + (O1[bt2] - S1[bt2]) * f2s);
        U2[bt1] = fc * (rss * O1[bt1] + rso * S1[bt1] + rss * rso * (vo1 - vs1) * f2s);
        U2[bt2] = fc * (rss * O1[bt2] + rso * S1[bt2] + rss * rso * (vo2 - vs2) * f2s);
        U2[RO] = ros;
        U2[EN] = S1[EN] - rss * (vs1 * S1[bt1] + vs2 * S1[bt2] - at1 * U2[bt1] - at2 * U2[bt2]) * f2s;
        U2[mn] = ros * aM;
        U2[mt1] = ros * at1;
        U2[mt2] = ros * at2;
        const double as1 = sR ? aM + aBn * rsS : aM - aBn * rsS;  // aR1 = aM + aV_R, aL1 = aM - aV_L
#pragma unroll
        for (int v = MX; v <= EN; ++v) Fo[v] = as1 * U2[v] - (as1 - as) * S1[v] - as * Us[v] + Fs[v];
        Fo[RO] = as1 * U2[RO] - (as1 - as) * S1[RO] - as * Us[RO] + Fs[RO];
        Fo[bt1] = as1 * U2[bt1] - (as1 - as) * S1[bt1] - as * Us[bt1] + Fs[bt1];
        Fo[bt2] = as1 * U2[bt2] - (as1 - as) * S1[bt2] - as * Us[bt2] + Fs[bt2];
      }
    }
  }
  // GLM fluxes :580-581, the halving folded into the (exact) half speeds
  const double hch = 0.5 * ch, hch2 = 0.5 * (ch * ch);
  Fo[bn] = 0.5 * (L[PS] + R[PS]) - hch * (R[bn] - L[bn]);
  Fo[PS] = hch2 * (L[bn] + R[bn]) - hch * (R[PS] - L[PS]);
  if constexpr (TAPE == tape::kRecord) *code_io = code_reg;
}

// Numerical flux across one face (2D_basic/flux_solver.f90):
//   LLF :89-148, HLL :153-221, HLLC :226-347, HLLD :352-585 (HLLC-G fallback
//   :447-476), LHLLD :590-789; GLM fluxes for Bn and psi :580-581.
// r1 = 1/(gamma-1), r2 = gamma/(gamma-1) are passed in (flux_solver.f90:38-39).
//
// Under a decision tape (TAPE != tape::kNone; HLLD only) every comparison that
// selects a wave speed, a region or a sign is recorded in *code or replayed
// from it (tape::kArSel ... tape::kClampR); the arithmetic is unchanged.
template <class T, int DIR, int TYPE, bool FAST = false, int TAPE = tape::kNone>
__device__ __forceinline__ void riemann_flux(const T (&L)[NV], const T (&R)[NV], T ch, T gamma, T r1,
                                             T r2, T (&Fo)[NV], unsigned* code_io = nullptr) {
  using tape::decide;
  if constexpr (FAST && sizeof(T) == 8 && TYPE == FX_HLLD) {
    hlld_f64<DIR, TAPE>(L, R, ch, gamma, r1, r2, Fo, code_io);
    return;
  }
  // the face's decision word lives in a register here; read from / written to
  // *code_io once (replay / record)
  unsigned code_reg = (TAPE == tape::kReplay) ? *code_io : 0u;
  unsigned* const code = &code_reg;
  constexpr int vn = VX + (DIR - 1) % 3, vt1 = VX + DIR % 3, vt2 = VX + (DIR + 1) % 3;
  constexpr int bn = BX + (DIR - 1) % 3, bt1 = BX + DIR % 3, bt2 = BX + (DIR + 1) % 3;
  constexpr int mn = MX + (DIR - 1) % 3, mt1 = MX + DIR % 3, mt2 = MX + (DIR + 1) % 3;
  const T hllg_factor = T(1.001);
  const T ch2 = ch * ch;

  T UL[4], UR[4], FL[NV], FR[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    FL[v] = T(0);
    FR[v] = T(0);
    Fo[v] = T(0);
  }
  T v2, B2, vBL, vBR, f1, f2, aL, aR, ptL = T(0), ptR = T(0), aL1 = T(0), aR1 = T(0);

  // VL --> UL, FL  (:359-372)
  v2 = L[VX] * L[VX] + L[VY] * L[VY] + L[VZ] * L[VZ];
  B2 = L[BX] * L[BX] + L[BY] * L[BY] + L[BZ] * L[BZ];
  vBL = L[VX] * L[BX] + L[VY] * L[BY] + L[VZ] * L[BZ];
  UL[MX] = L[RO] * L[VX];
  UL[MY] = L[RO] * L[VY];
  UL[MZ] = L[RO] * L[VZ];
  UL[EN] = T(0.5) * (L[RO] * v2 + B2) + r1 * L[PR];
  FL[RO] = L[RO] * L[vn];
  FL[mn] = L[RO] * L[vn] * L[vn] - L[bn] * L[bn] + L[PR] + T(0.5) * B2;
  FL[EN] = (T(0.5) * L[RO] * v2 + r2 * L[PR] + B2) * L[vn] - vBL * L[bn];
  FL[mt1] = L[RO] * L[vn] * L[vt1] - L[bn] * L[bt1];
  FL[mt2] = L[RO] * L[vn] * L[vt2] - L[bn] * L[bt2];
  FL[bt1] = L[vn] * L[bt1] - L[bn] * L[vt1];
  FL[bt2] = L[vn] * L[bt2] - L[bn] * L[vt2];
  f1 = gamma * L[PR];
  f2 = 4 * (L[bn] * L[bn]);
  if (TYPE == FX_LLF) {
    aL = sqrt(div_<T, FAST>((f1 + B2) + sqrt((f1 + B2) * (f1 + B2) - f1 * f2), 2 * L[RO]));
  } else {
    {  // fmax2(D, 0)
      const T D = (f1 + B2) * (f1 + B2) - f1 * f2;
      const bool cl = decide<TAPE>(lt0_<T, FAST>(D), code, tape::kClampL);
      aL = div_<T, FAST>((f1 + B2) + sqrt_<T, FAST>(cl ? T(0) : D), 2 * L[RO]);
    }
    ptL = L[PR] + T(0.5) * B2;
    if (TYPE == FX_LHLLD) {
      const T g1 = L[RO] * v2;
      aL1 = div_<T, FAST>((g1 + B2) + sqrt(fmax2((g1 + B2) * (g1 + B2) - g1 * f2, T(0))), 2 * L[RO]);
    }
  }

  // VR --> UR, FR  (:381-401)
  v2 = R[VX] * R[VX] + R[VY] * R[VY] + R[VZ] * R[VZ];
  B2 = R[BX] * R[BX] + R[BY] * R[BY] + R[BZ] * R[BZ];
  vBR = R[VX] * R[BX] + R[VY] * R[BY] + R[VZ] * R[BZ];
  UR[MX] = R[RO] * R[VX];
  UR[MY] = R[RO] * R[VY];
  UR[MZ] = R[RO] * R[VZ];
  UR[EN] = T(0.5) * (R[RO] * v2 + B2) + r1 * R[PR];
  FR[RO] = R[RO] * R[vn];
  FR[mn] = R[RO] * R[vn] * R[vn] - R[bn] * R[bn] + R[PR] + T(0.5) * B2;
  FR[EN] = (T(0.5) * R[RO] * v2 + r2 * R[PR] + B2) * R[vn] - vBR * R[bn];
  FR[mt1] = R[RO] * R[vn] * R[vt1] - R[bn] * R[bt1];
  FR[mt2] = R[RO] * R[vn] * R[vt2] - R[bn] * R[bt2];
  FR[bt1] = R[vn] * R[bt1] - R[bn] * R[vt1];
  FR[bt2] = R[vn] * R[bt2] - R[bn] * R[vt2];
  f1 = gamma * R[PR];
  f2 = 4 * (R[bn] * R[bn]);
  if (TYPE == FX_LLF) {
    aR = sqrt(div_<T, FAST>((f1 + B2) + sqrt((f1 + B2) * (f1 + B2) - f1 * f2), 2 * R[RO]));
  } else {
    {  // fmax2(D, 0)
      const T D = (f1 + B2) * (f1 + B2) - f1 * f2;
      const bool cl = decide<TAPE>(lt0_<T, FAST>(D), code, tape::kClampR);
      aR = div_<T, FAST>((f1 + B2) + sqrt_<T, FAST>(cl ? T(0) : D), 2 * R[RO]);
    }
    ptR = R[PR] + T(0.5) * B2;
    if (TYPE == FX_LHLLD) {
      const T g1 = R[RO] * v2;
      aR1 = div_<T, FAST>((g1 + B2) + sqrt(fmax2((g1 + B2) * (g1 + B2) - g1 * f2, T(0))), 2 * R[RO]);
    }
  }

  if (TYPE == FX_LLF) {  // :138-142
    f1 = fmax2(fabs(L[vn]) + aL, fabs(R[vn]) + aR);
#pragma unroll
    for (int v = MX; v <= EN; ++v) Fo[v] = T(0.5) * (FL[v] + FR[v] - f1 * (UR[v] - UL[v]));
    Fo[RO] = T(0.5) * (FL[RO] + FR[RO] - f1 * (R[RO] - L[RO]));
    Fo[bt1] = T(0.5) * (FL[bt1] + FR[bt1] - f1 * (R[bt1] - L[bt1]));
    Fo[bt2] = T(0.5) * (FL[bt2] + FR[bt2] - f1 * (R[bt2] - L[bt2]));
  } else if (TYPE == FX_HLL) {  // :205-214
    f1 = sqrt(fmax2(aL, aR));
    aL = fmin2(fmin2(L[vn], R[vn]) - f1, T(0));
    aR = fmax2(fmax2(L[vn], R[vn]) + f1, T(0));
    f1 = rcp_<T, FAST>(aR - aL);
    f2 = aL * aR;
#pragma unroll
    for (int v = MX; v <= EN; ++v) Fo[v] = f1 * (aR * FL[v] - aL * FR[v] + f2 * (UR[v] - UL[v]));
    Fo[RO] = f1 * (aR * FL[RO] - aL * FR[RO] + f2 * (R[RO] - L[RO]));
    Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
    Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
  } else if (TYPE == FX_HLLC) {  // :281-340
    T Uh[NV];
    f1 = sqrt(fmax2(aL, aR));
    aL = fmin2(fmin2(L[vn], R[vn]) - f1, T(0));
    aR = fmax2(fmax2(L[vn], R[vn]) + f1, T(0));
    f1 = rcp_<T, FAST>(aR - aL);
    f2 = aL * aR;
#pragma unroll
    for (int v = MX; v <= MZ; ++v) Uh[v] = f1 * (aR * UR[v] - aL * UL[v] - FR[v] + FL[v]);
#pragma unroll
    for (int v = RO; v <= BZ; ++v) Uh[v] = f1 * (aR * R[v] - aL * L[v] - FR[v] + FL[v]);
    Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
    Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
    f2 = rcp_<T, FAST>(Uh[RO]);
    const T aM = Uh[mn] * f2;
    const T at1 = Uh[mt1] * f2;
    const T at2 = Uh[mt2] * f2;
    const T pt = ptL + L[RO] * (aL - L[vn]) * (aM - L[vn]);
    const T roL = div_<T, FAST>(L[RO] * (aL - L[vn]), aL - aM);
    const T enL = div_<T, FAST>(((aL - L[vn]) * UL[EN] - ptL * L[vn] + pt * aM +
                   Uh[bn] * (vBL - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])), (aL - aM));
    const T roR = div_<T, FAST>(R[RO] * (aR - R[vn]), aR - aM);
    const T enR = div_<T, FAST>(((aR - R[vn]) * UR[EN] - ptR * R[vn] + pt * aM +
                   Uh[bn] * (vBR - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])), (aR - aM));
    f1 = T(0.5) + fsign(T(0.5), aM);
    f2 = T(1) - f1;
    Fo[mn] = f1 * (aL * (roL * aM - UL[mn]) + FL[mn]) + f2 * (aR * (roR * aM - UR[mn]) + FR[mn]);
    Fo[mt1] = f1 * (aL * (roL * at1 - UL[mt1]) + FL[mt1]) + f2 * (aR * (roR * at1 - UR[mt1]) + FR[mt1]);
    Fo[mt2] = f1 * (aL * (roL * at2 - UL[mt2]) + FL[mt2]) + f2 * (aR * (roR * at2 - UR[mt2]) + FR[mt2]);
    Fo[EN] = f1 * (aL * (enL - UL[EN]) + FL[EN]) + f2 * (aR * (enR - UR[EN]) + FR[EN]);
    Fo[RO] = f1 * (aL * (roL - L[RO]) + FL[RO]) + f2 * (aR * (roR - R[RO]) + FR[RO]);
  } else {  // HLLD :408-576 / LHLLD :648-780
    T psi = T(0);
    if (TYPE == FX_LHLLD) {
      f1 = fmin2(T(1), div_<T, FAST>(fmax2(aL1, aR1), fmax2(aL, aR)));
      psi = 2 * sqrt(f1) - f1;
    }
    f1 = sqrt_<T, FAST>(decide<TAPE>(lt_<T, FAST>(aL, aR), code, tape::kArSel) ? aR : aL);  // fmax2(aL, aR)
    aL = (decide<TAPE>(lt_<T, FAST>(R[vn], L[vn]), code, tape::kMinR) ? R[vn] : L[vn]) - f1;  // fmin2
    aR = (decide<TAPE>(lt_<T, FAST>(L[vn], R[vn]), code, tape::kMaxR) ? R[vn] : L[vn]) + f1;  // fmax2
    if (decide<TAPE>(ge0_<T, FAST>(aL), code, tape::kFL)) {
#pragma unroll
      for (int v = 0; v < NV; ++v) Fo[v] = FL[v];
    } else if (decide<TAPE>(le0_<T, FAST>(aR), code, tape::kFR)) {
#pragma unroll
      for (int v = 0; v < NV; ++v) Fo[v] = FR[v];
    } else {
      T Uh[NV];
      f1 = rcp_<T, FAST>(aR - aL);
#pragma unroll
      for (int v = MX; v <= MZ; ++v) Uh[v] = f1 * (aR * UR[v] - aL * UL[v] - FR[v] + FL[v]);
#pragma unroll
      for (int v = RO; v <= BZ; ++v) Uh[v] = f1 * (aR * R[v] - aL * L[v] - FR[v] + FL[v]);
      const T aM = div_<T, FAST>(Uh[mn], Uh[RO]);
      T pt;
      if (TYPE == FX_LHLLD) {
        pt = div_<T, FAST>(R[RO] * ptL * (aR - R[vn]) - L[RO] * ptR * (aL - L[vn]) +
                               psi * L[RO] * R[RO] * (aR - R[vn]) * (aL - L[vn]) * (R[vn] - L[vn]),
                           R[RO] * (aR - R[vn]) - L[RO] * (aL - L[vn]));
      } else {
        pt = ptL + L[RO] * (aL - L[vn]) * (aM - L[vn]);
      }
      // one reciprocal of (aL - aM) and of (aR - aM) serves rho*, E* (FAST)
      const T ieL = (FAST && sizeof(T) == 8) ? rcp_<T, FAST>(aL - aM) : T(0);
      const T ieR = (FAST && sizeof(T) == 8) ? rcp_<T, FAST>(aR - aM) : T(0);
      const T roL = divr_<T, FAST>(L[RO] * (aL - L[vn]), aL - aM, ieL);
      const T roR = divr_<T, FAST>(R[RO] * (aR - R[vn]), aR - aM, ieR);
      // Alfven speeds; the FAST variant keeps 1/sqrt(rho*) for the central states
      T rsL = T(0), rsR = T(0);
      if constexpr (FAST && sizeof(T) == 8) {
        rsL = rsqrt_nr(roL);
        rsR = rsqrt_nr(roR);
      }
      // |Bn| and sign(1, Bn) from one recorded sign bit under a tape
      const bool bneg = decide<TAPE>(signbit(Uh[bn]) != 0, code, tape::kBnNeg);
      const T aBn = (TAPE == tape::kNone) ? fabs(Uh[bn]) : (bneg ? -Uh[bn] : Uh[bn]);
      const T aVL = (FAST && sizeof(T) == 8) ? aBn * rsL : aBn / sqrt(roL);
      const T aVR = (FAST && sizeof(T) == 8) ? aBn * rsR : aBn / sqrt(roR);
      if (TYPE == FX_HLLD && decide<TAPE>(!lt_<T, FAST>(aL, aM - hllg_factor * aVL) ||
                                              !lt_<T, FAST>(aM + hllg_factor * aVR, aR),
                                          code, tape::kG)) {
        // HLLC-G fallback :450-476
        f2 = aL * aR;
        Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
        Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
        const T at1 = div_<T, FAST>(Uh[mt1], Uh[RO]);
        const T at2 = div_<T, FAST>(Uh[mt2], Uh[RO]);
        const T enL = divr_<T, FAST>(((aL - L[vn]) * UL[EN] - ptL * L[vn] + pt * aM +
                       Uh[bn] * (vBL - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])), (aL - aM), ieL);
        const T enR = divr_<T, FAST>(((aR - R[vn]) * UR[EN] - ptR * R[vn] + pt * aM +
                       Uh[bn] * (vBR - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])), (aR - aM), ieR);
        if constexpr (TAPE != tape::kNone)
          f1 = decide<TAPE>(signbit(aM) == 0, code, tape::kGLeft) ? T(1) : T(0);  // 0.5 + sign(0.5, aM)
        else
          f1 = T(0.5) + fsign(T(0.5), aM);
        f2 = T(1) - f1;
        Fo[mn] = f1 * (aL * (roL * aM - UL[mn]) + FL[mn]) + f2 * (aR * (roR * aM - UR[mn]) + FR[mn]);
        Fo[mt1] = f1 * (aL * (roL * at1 - UL[mt1]) + FL[mt1]) + f2 * (aR * (roR * at1 - UR[mt1]) + FR[mt1]);
        Fo[mt2] = f1 * (aL * (roL * at2 - UL[mt2]) + FL[mt2]) + f2 * (aR * (roR * at2 - UR[mt2]) + FR[mt2]);
        Fo[EN] = f1 * (aL * (enL - UL[EN]) + FL[EN]) + f2 * (aR * (enR - UR[EN]) + FR[EN]);
        Fo[RO] = f1 * (aL * (roL - L[RO]) + FL[RO]) + f2 * (aR * (roR - R[RO]) + FR[RO]);
      } else {
        // Region first (aL1, aR1 need only aM and the Alfven speeds), then the
        // intermediate states that region uses: F(L*) needs L* only, F(R*)
        // R* only, the central states both.  Same expressions as :482-507.
        aL1 = aM - aVL;
        aR1 = aM + aVR;
        const bool sLs = decide<TAPE>(ge0_<T, FAST>(aL1), code, tape::kLS);
        const bool sRs = !sLs && decide<TAPE>(le0_<T, FAST>(aR1), code, tape::kRS);
        // (the FP32 arithmetic of the mixed variant computes both states
        // unconditionally: there the branch costs more than the work)
        constexpr bool kEager = !(FAST && sizeof(T) == 8);
        T UL1[NV] = {}, UR1[NV] = {};
        T vt1L = T(0), vt2L = T(0), vt1R = T(0), vt2R = T(0);
        if (kEager || !sRs) {  // L* (:482-493)
          const T tL = aL - L[vn];
          f1 = rcp_<T, FAST>(L[RO] * tL * (aL - aM) - Uh[bn] * Uh[bn]);
          UL1[bt1] = L[bt1] * f1 * (L[RO] * (tL * tL) - Uh[bn] * Uh[bn]);
          UL1[bt2] = L[bt2] * f1 * (L[RO] * (tL * tL) - Uh[bn] * Uh[bn]);
          vt1L = L[vt1] - f1 * Uh[bn] * L[bt1] * (aM - L[vn]);
          vt2L = L[vt2] - f1 * Uh[bn] * L[bt2] * (aM - L[vn]);
          UL1[RO] = roL;
          UL1[EN] = divr_<T, FAST>(((aL - L[vn]) * UL[EN] - ptL * L[vn] + pt * aM +
                     Uh[bn] * (vBL - aM * Uh[bn] - vt1L * UL1[bt1] - vt2L * UL1[bt2])), (aL - aM), ieL);
          UL1[mn] = roL * aM;
          UL1[mt1] = roL * vt1L;
          UL1[mt2] = roL * vt2L;
        }
        if (kEager || !sLs) {  // R* (:496-507)
          const T tR = aR - R[vn];
          f1 = rcp_<T, FAST>(R[RO] * tR * (aR - aM) - Uh[bn] * Uh[bn]);
          UR1[bt1] = R[bt1] * f1 * (R[RO] * (tR * tR) - Uh[bn] * Uh[bn]);
          UR1[bt2] = R[bt2] * f1 * (R[RO] * (tR * tR) - Uh[bn] * Uh[bn]);
          vt1R = R[vt1] - f1 * Uh[bn] * R[bt1] * (aM - R[vn]);
          vt2R = R[vt2] - f1 * Uh[bn] * R[bt2] * (aM - R[vn]);
          UR1[RO] = roR;
          UR1[EN] = divr_<T, FAST>(((aR - R[vn]) * UR[EN] - ptR * R[vn] + pt * aM +
                     Uh[bn] * (vBR - aM * Uh[bn] - vt1R * UR1[bt1] - vt2R * UR1[bt2])), (aR - aM), ieR);
          UR1[mn] = roR * aM;
          UR1[mt1] = roR * vt1R;
          UR1[mt2] = roR * vt2R;
        }
        if (sLs) {  // F(L*) :514-519
#pragma unroll
          for (int v = MX; v <= EN; ++v) Fo[v] = aL * (UL1[v] - UL[v]) + FL[v];
          Fo[RO] = aL * (UL1[RO] - L[RO]) + FL[RO];
          Fo[bt1] = aL * (UL1[bt1] - L[bt1]) + FL[bt1];
          Fo[bt2] = aL * (UL1[bt2] - L[bt2]) + FL[bt2];
                } else if (sRs) {  // F(R*) :522-527
#pragma unroll
          for (int v = MX; v <= EN; ++v) Fo[v] = aR * (UR1[v] - UR[v]) + FR[v];
          Fo[RO] = aR * (UR1[RO] - R[RO]) + FR[RO];
          Fo[bt1] = aR * (UR1[bt1] - R[bt1]) + FR[bt1];
          Fo[bt2] = aR * (UR1[bt2] - R[bt2]) + FR[bt2];
                } else {  // central states :533-572
          T U2[NV];
          const T roLs = (FAST && sizeof(T) == 8) ? roL * rsL : sqrt(roL);
          const T roRs = (FAST && sizeof(T) == 8) ? roR * rsR : sqrt(roR);
          f1 = rcp_<T, FAST>(roLs + roRs);
          f2 = (TAPE == tape::kNone) ? fsign(T(1), Uh[bn]) : (bneg ? T(-1) : T(1));
          const T at1 = f1 * (roLs * vt1L + roRs * vt1R + (UR1[bt1] - UL1[bt1]) * f2);
          const T at2 = f1 * (roLs * vt2L + roRs * vt2R + (UR1[bt2] - UL1[bt2]) * f2);
          U2[bt1] = f1 * (roLs * UR1[bt1] + roRs * UL1[bt1] + roLs * roRs * (vt1R - vt1L) * f2);
          U2[bt2] = f1 * (roLs * UR1[bt2] + roRs * UL1[bt2] + roLs * roRs * (vt2R - vt2L) * f2);
          if (decide<TAPE>(ge0_<T, FAST>(aM), code, tape::kSSLeft)) {  // F(L**)
            U2[RO] = roL;
            U2[EN] = UL1[EN] - roLs * (vt1L * UL1[bt1] + vt2L * UL1[bt2] - at1 * U2[bt1] - at2 * U2[bt2]) * f2;
            U2[mn] = roL * aM;
            U2[mt1] = roL * at1;
            U2[mt2] = roL * at2;
#pragma unroll
            for (int v = MX; v <= EN; ++v) Fo[v] = aL1 * U2[v] - (aL1 - aL) * UL1[v] - aL * UL[v] + FL[v];
            Fo[RO] = aL1 * U2[RO] - (aL1 - aL) * UL1[RO] - aL * L[RO] + FL[RO];
            Fo[bt1] = aL1 * U2[bt1] - (aL1 - aL) * UL1[bt1] - aL * L[bt1] + FL[bt1];
            Fo[bt2] = aL1 * U2[bt2] - (aL1 - aL) * UL1[bt2] - aL * L[bt2] + FL[bt2];
                    } else {  // F(R**)
            U2[RO] = roR;
            U2[EN] = UR1[EN] + roRs * (vt1R * UR1[bt1] + vt2R * UR1[bt2] - at1 * U2[bt1] - at2 * U2[bt2]) * f2;
            U2[mn] = roR * aM;
            U2[mt1] = roR * at1;
            U2[mt2] = roR * at2;
#pragma unroll
            for (int v = MX; v <= EN; ++v) Fo[v] = aR1 * U2[v] - (aR1 - aR) * UR1[v] - aR * UR[v] + FR[v];
            Fo[RO] = aR1 * U2[RO] - (aR1 - aR) * UR1[RO] - aR * R[RO] + FR[RO];
            Fo[bt1] = aR1 * U2[bt1] - (aR1 - aR) * UR1[bt1] - aR * R[bt1] + FR[bt1];
            Fo[bt2] = aR1 * U2[bt2] - (aR1 - aR) * UR1[bt2] - aR * R[bt2] + FR[bt2];
                    }
        }
      }
    }
  }
  // GLM fluxes :580-581
  Fo[bn] = T(0.5) * ((L[PS] + R[PS]) - ch * (R[bn] - L[bn]));
  Fo[PS] = T(0.5) * (ch2 * (L[bn] + R[bn]) - ch * (R[PS] - L[PS]));
  if constexpr (TAPE == tape::kRecord) *code_io = code_reg;
}

// u2v.f90:11-27 for one cell, into the face arithmetic's type: w = (vx, vy,
// vz, p, rho, Bx, By, Bz, psi) with the given (GLM-scaled) psi; pr and ro
// return p and rho for the positivity check (u2v.f90:36-45), in FP64 as the
// recovery computed them (binary32 values widened exactly).
// FP64 kernels: the reference's FP64 recovery.  FP32-mixed kernels: binary32
// recovery where E >= rho v^2 + B^2, i.e. where the internal energy is at
// least the kinetic plus the magnetic energy, so that the pressure -- a
// difference of energies -- amplifies the rounding of its inputs at most
// ~4-fold; FP64 recovery, then rounding, everywhere else (low beta, high
// Mach, and every unphysical state, whose check then sees FP64 values).
template <class T, bool FAST>
__device__ __forceinline__ void u2v_cell(const double (&u)[NV], double f1g, float f1g32, double psi, T (&w)[NV],
                                         double& pr, double& ro) {
  if constexpr (sizeof(T) == 4) {
    const float r = narrow_f64(u[RO]), mx = narrow_f64(u[MX]), my = narrow_f64(u[MY]), mz = narrow_f64(u[MZ]);
    const float bx = narrow_f64(u[BX]), by = narrow_f64(u[BY]), bz = narrow_f64(u[BZ]), en = narrow_f64(u[EN]);
    const float ir = __frcp_rn(r);
    const float vx = mx * ir, vy = my * ir, vz = mz * ir;
    const float rv2 = vx * mx + vy * my + vz * mz;
    const float B2 = bx * bx + by * by + bz * bz;
    if (en >= rv2 + B2) {
      w[VX] = vx;
      w[VY] = vy;
      w[VZ] = vz;
      w[PR] = f1g32 * (en - 0.5f * (rv2 + B2));
      w[RO] = r;
      w[BX] = bx;
      w[BY] = by;
      w[BZ] = bz;
      w[PS] = narrow_f64(psi);
      pr = widen_f32(w[PR]);
      ro = widen_f32(r);
      return;
    }
  }
  const double r = u[RO];
  const double mx = u[MX], my = u[MY], mz = u[MZ];
  const double ir = rcp_<double, FAST>(r);  // one reciprocal for the three velocities
  const double vx = divr_<double, FAST>(mx, r, ir), vy = divr_<double, FAST>(my, r, ir),
               vz = divr_<double, FAST>(mz, r, ir);  // u2v.f90:24
  const double rv2 = vx * mx + vy * my + vz * mz;
  const double bx = u[BX], by = u[BY], bz = u[BZ];
  const double B2 = bx * bx + by * by + bz * bz;
  const double p = f1g * (u[EN] - 0.5 * (rv2 + B2));  // u2v.f90:27
  w[VX] = to_face<T>(vx);
  w[VY] = to_face<T>(vy);
  w[VZ] = to_face<T>(vz);
  w[PR] = to_face<T>(p);
  w[RO] = to_face<T>(r);
  w[BX] = to_face<T>(bx);
  w[BY] = to_face<T>(by);
  w[BZ] = to_face<T>(bz);
  w[PS] = to_face<T>(psi);
  pr = p;
  ro = r;
}

// Fast magnetosonic speed used by set_dt (2D_basic/set_dt.f90:27-34).
template <class T, bool FAST = false>
__device__ __forceinline__ T fast_speed(T f1, T B2, T bd, T ro) {
  const T f2 = 4 * f1 * (bd * bd);
  const T D = (f1 + B2) * (f1 + B2) - f2;
  return sqrt_ratio_<T, FAST>((f1 + B2) + sqrt_<T, FAST>(lt0_<T, FAST>(D) ? T(0) : D), 2 * ro);
}

}  // namespace omhd
