// omhd_tape.h -- the decision tape of the FP64 2D step: the discrete choices
// a forward stage makes (slope-limiter selections and HLLD wave-speed / branch
// selections) recorded per cell and per face, so that
//   * the adjoint differentiates exactly the branch the forward took, and
//   * a forward can be replayed with every choice frozen: the smooth map
//     whose derivative the adjoint is (finite differences of it have no
//     kinks to straddle).
// Plain C++ (host and device).
#pragma once

namespace omhd {
namespace tape {

// modes of a taped kernel
constexpr int kNone = 0, kRecord = 1, kReplay = 2;

// limiter code of one (cell, variable, direction), one byte:
//   bits 0-1 : 0 slopes of opposite sign (grad = 0), 1 gA selected,
//              2 gB selected, 3 gC selected (MC);
//   bit 2    : the selected gC enters with a minus sign (sign(gA) != sign(gC))
constexpr unsigned char kLimZero = 0, kLimA = 1, kLimB = 2, kLimC = 3, kLimCNeg = 4;

// HLLD code of one face (flux_solver.f90:352-585), one 16-bit word
constexpr unsigned kArSel = 1u << 0;   // fmax2(aL, aR) took aR  (fast-speed proxy)
constexpr unsigned kMinR = 1u << 1;    // fmin2(vnL, vnR) took vnR
constexpr unsigned kMaxR = 1u << 2;    // fmax2(vnL, vnR) took vnR
constexpr unsigned kFL = 1u << 3;      // SL >= 0: F = F(L)
constexpr unsigned kFR = 1u << 4;      // SR <= 0: F = F(R)
constexpr unsigned kG = 1u << 5;       // HLLC-G fallback
constexpr unsigned kGLeft = 1u << 6;   // fallback: left state (aM >= +0)
constexpr unsigned kLS = 1u << 7;      // F(L*)
constexpr unsigned kRS = 1u << 8;      // F(R*)
constexpr unsigned kSSLeft = 1u << 9;  // central states: F(L**)
constexpr unsigned kBnNeg = 1u << 10;  // sign bit of the HLL-average normal field
constexpr unsigned kClampL = 1u << 11; // fast-speed discriminant clamped to 0, left
constexpr unsigned kClampR = 1u << 12; // ... right

// One decision under a tape mode: record sets the bit when the condition
// holds, replay returns the recorded bit, none passes the condition through.
template <int MODE, class C>
#ifdef __CUDACC__
__host__ __device__
#endif
inline bool decide(bool cond, C* code, C bit) {
  if constexpr (MODE == kReplay) return (*code & bit) != 0;
  if constexpr (MODE == kRecord) {
    if (cond) *code = (C)(*code | bit);
  }
  return cond;
}

}  // namespace tape
}  // namespace omhd
