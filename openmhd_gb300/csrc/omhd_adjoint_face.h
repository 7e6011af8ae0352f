// omhd_adjoint_face.h -- hand-written reverse-mode derivatives (vector-Jacobian
// products) of the per-face pieces of the step, in FP64:
//   hlld_vjp   : HLLD flux (2D_basic/flux_solver.f90:352-585) incl. the HLLC-G
//                fallback and the GLM fluxes of Bn and psi; the branch taken is
//                the forward's (recomputed from the same face states);
//   recon_vjp  : minmod / MC reconstruction (limiter.f90) with the selection
//                of the forward and a fixed subgradient at kinks (ties pick
//                the first operand, as fmin2 does; opposite signs -> zero);
//   u2v_vjp    : conserved -> primitive map (u2v.f90:24-27).
// Plain C++ (host and device): the CPU test harness compiles this header with
// g++ and checks every branch against central finite differences.
#pragma once
#include <cmath>

#include "omhd_fastmath.h"
#include "omhd_tape.h"

#ifdef __CUDACC__
#define OMHD_HD __host__ __device__ __forceinline__
#else
#define OMHD_HD inline
#endif

namespace omhd {
namespace adj {

// 1/x and 1/sqrt(x): Newton-Raphson from the hardware approximations on the
// device (omhd_fastmath.h, ~1 ulp), IEEE on the host.  Every denominator is
// inverted once and its uses multiply.
OMHD_HD double arcp(double x) {
#ifdef __CUDA_ARCH__
  return rcp_nr(x);
#else
  return 1.0 / x;
#endif
}
OMHD_HD double arsqrt(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt_nr(x);
#else
  return 1.0 / std::sqrt(x);
#endif
}

// slots: w = (vx vy vz p rho Bx By Bz psi); U/F = (mx my mz E rho Bx By Bz psi)
constexpr int kVX = 0, kPR = 3, kRO = 4, kBX = 5, kPS = 8, kEN = 3;

struct Side {
  double v2, B2, vB, Um[3], UE, F[9], f1, f2, Q, D, sq, a, pt, ir, isq;
};
using tape::decide;
struct SideG {
  double Um[3], UE, F[9], a, pt, vB;
};

OMHD_HD void zero(SideG& g) {
  for (int k = 0; k < 3; ++k) g.Um[k] = 0.0;
  for (int k = 0; k < 9; ++k) g.F[k] = 0.0;
  g.UE = g.a = g.pt = g.vB = 0.0;
}

// one side of the face: conserved state, physical flux, fast-speed^2 proxy,
// total pressure (flux_solver.f90:359-379)
template <int DIR, int MODE = tape::kNone>
OMHD_HD void side_fwd(const double* s, double gamma, double r1, double r2, Side& o, unsigned* code = nullptr,
                      unsigned clamp_bit = 0) {
  constexpr int vn = (DIR - 1) % 3, vt1 = DIR % 3, vt2 = (DIR + 1) % 3;
  constexpr int bn = kBX + (DIR - 1) % 3, bt1 = kBX + DIR % 3, bt2 = kBX + (DIR + 1) % 3;
  constexpr int mn = vn, mt1 = vt1, mt2 = vt2;
  o.v2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
  o.B2 = s[5] * s[5] + s[6] * s[6] + s[7] * s[7];
  o.vB = s[0] * s[5] + s[1] * s[6] + s[2] * s[7];
  for (int k = 0; k < 3; ++k) o.Um[k] = s[kRO] * s[k];
  o.UE = 0.5 * (s[kRO] * o.v2 + o.B2) + r1 * s[kPR];
  for (int k = 0; k < 9; ++k) o.F[k] = 0.0;
  o.F[kRO] = s[kRO] * s[vn];
  o.F[mn] = s[kRO] * s[vn] * s[vn] - s[bn] * s[bn] + s[kPR] + 0.5 * o.B2;
  o.f1 = gamma * s[kPR];
  o.f2 = 4 * (s[bn] * s[bn]);
  o.Q = o.f1 + o.B2;
  o.D = o.Q * o.Q - o.f1 * o.f2;
  const double Dc = decide<MODE>(0.0 > o.D, code, clamp_bit) ? 0.0 : o.D;  // fmax2(D, 0)
  o.isq = (Dc > 0.0) ? arsqrt(Dc) : 0.0;
  o.sq = Dc * o.isq;
  o.ir = 0.0;  // 1/rho and the fast speed squared a = (Q + sq)/(2 rho): set by
  o.a = 0.0;   // hlld_vjp for the side whose speed is the larger (side_cf)
  o.pt = s[kPR] + 0.5 * o.B2;
}

// the tangential momentum, energy and tangential field fluxes of one side
// (flux_solver.f90:368-372): only the HLLC-G fallback reads their values
template <int DIR>
OMHD_HD void side_fwd_tan(const double* s, double r2, Side& o) {
  constexpr int vn = (DIR - 1) % 3, vt1 = DIR % 3, vt2 = (DIR + 1) % 3;
  constexpr int bn = kBX + (DIR - 1) % 3, bt1 = kBX + DIR % 3, bt2 = kBX + (DIR + 1) % 3;
  constexpr int mt1 = vt1, mt2 = vt2;
  o.F[mt1] = s[kRO] * s[vn] * s[vt1] - s[bn] * s[bt1];
  o.F[mt2] = s[kRO] * s[vn] * s[vt2] - s[bn] * s[bt2];
  o.F[kEN] = (0.5 * s[kRO] * o.v2 + r2 * s[kPR] + o.B2) * s[vn] - o.vB * s[bn];
  o.F[bt1] = s[vn] * s[bt1] - s[bn] * s[vt1];
  o.F[bt2] = s[vn] * s[bt2] - s[bn] * s[vt2];
}

// 1/rho and the fast speed squared a = (Q + sq)/(2 rho) of one side
OMHD_HD void side_cf(const double* s, Side& o) {
  o.ir = arcp(s[kRO]);
  o.a = (o.Q + o.sq) * (0.5 * o.ir);
}

// flux = false: the side's tangential momentum, energy and tangential field
// fluxes carry no gradient (g.F is zero there), and their reverse is skipped;
// cf = false: the side's fast speed is not the face's (g.a is zero), and the
// reverse of its fast-speed chain is skipped
template <int DIR>
OMHD_HD void side_adj(const double* s, double gamma, double r1, double r2, const Side& o, const SideG& g,
                      double* gs, bool flux = true, bool cf = true) {
  constexpr int vn = (DIR - 1) % 3, vt1 = DIR % 3, vt2 = (DIR + 1) % 3;
  constexpr int bn = kBX + (DIR - 1) % 3, bt1 = kBX + DIR % 3, bt2 = kBX + (DIR + 1) % 3;
  constexpr int mn = vn, mt1 = vt1, mt2 = vt2;
  double gv[3] = {0.0, 0.0, 0.0}, gB[3] = {0.0, 0.0, 0.0};
  double gB2 = 0.0, gv2 = 0.0, gvB = g.vB, gp = 0.0, gro = 0.0;
  // pt = p + B2/2
  gp += g.pt;
  gB2 += 0.5 * g.pt;
  if (cf) {
    // a = (Q + sq) / (2 rho)
    const double gnum = g.a * (0.5 * o.ir);
    gro -= g.a * o.a * o.ir;
    double gQ = gnum;
    const double gsq = gnum;
    const double gD = (o.D > 0.0) ? gsq * 0.5 * o.isq : 0.0;
    gQ += 2 * o.Q * gD;
    double gf1 = -o.f2 * gD;
    const double gf2 = -o.f1 * gD;
    gf1 += gQ;
    gB2 += gQ;
    gB[bn - kBX] += 8 * s[bn] * gf2;
    gp += gamma * gf1;
  }
  if (flux) {
    // tangential field fluxes
    {
      const double q = g.F[bt2];
      gv[vn] += q * s[bt2];
      gB[bt2 - kBX] += q * s[vn];
      gB[bn - kBX] -= q * s[vt2];
      gv[vt2] -= q * s[bn];
    }
    {
      const double q = g.F[bt1];
      gv[vn] += q * s[bt1];
      gB[bt1 - kBX] += q * s[vn];
      gB[bn - kBX] -= q * s[vt1];
      gv[vt1] -= q * s[bn];
    }
    // energy flux (K vn - vB bn)
    {
      const double q = g.F[kEN];
      const double K = 0.5 * s[kRO] * o.v2 + r2 * s[kPR] + o.B2;
      const double gK = q * s[vn];
      gv[vn] += q * K;
      gvB -= q * s[bn];
      gB[bn - kBX] -= q * o.vB;
      gro += 0.5 * o.v2 * gK;
      gv2 += 0.5 * s[kRO] * gK;
      gp += r2 * gK;
      gB2 += gK;
    }
    // tangential momentum fluxes
    {
      const double q = g.F[mt2];
      gro += q * s[vn] * s[vt2];
      gv[vn] += q * s[kRO] * s[vt2];
      gv[vt2] += q * s[kRO] * s[vn];
      gB[bn - kBX] -= q * s[bt2];
      gB[bt2 - kBX] -= q * s[bn];
    }
    {
      const double q = g.F[mt1];
      gro += q * s[vn] * s[vt1];
      gv[vn] += q * s[kRO] * s[vt1];
      gv[vt1] += q * s[kRO] * s[vn];
      gB[bn - kBX] -= q * s[bt1];
      gB[bt1 - kBX] -= q * s[bn];
    }
  }
  // normal momentum flux
  {
    const double q = g.F[mn];
    gro += q * s[vn] * s[vn];
    gv[vn] += 2 * q * s[kRO] * s[vn];
    gB[bn - kBX] -= 2 * q * s[bn];
    gp += q;
    gB2 += 0.5 * q;
  }
  // mass flux
  gro += g.F[kRO] * s[vn];
  gv[vn] += g.F[kRO] * s[kRO];
  // conserved energy and momentum
  gro += 0.5 * o.v2 * g.UE;
  gv2 += 0.5 * s[kRO] * g.UE;
  gB2 += 0.5 * g.UE;
  gp += r1 * g.UE;
  for (int k = 0; k < 3; ++k) {
    gro += g.Um[k] * s[k];
    gv[k] += g.Um[k] * s[kRO];
  }
  for (int k = 0; k < 3; ++k) {
    gv[k] += gvB * s[kBX + k] + 2 * s[k] * gv2;
    gB[k] += gvB * s[k] + 2 * s[kBX + k] * gB2;
  }
  for (int k = 0; k < 3; ++k) {
    gs[k] += gv[k];
    gs[kBX + k] += gB[k];
  }
  gs[kPR] += gp;
  gs[kRO] += gro;
}

// gL, gR = (dF/dL)^T gF, (dF/dR)^T gF for the HLLD flux F(L, R) with ch fixed.
// MODE tape::kReplay takes every branch and selection from *code (the
// forward's decision tape, omhd_tape.h); otherwise they are recomputed from
// L and R (and recorded in *code under tape::kRecord).
template <int DIR, int MODE = tape::kNone>
OMHD_HD void hlld_vjp(const double* L, const double* R, double ch, double gamma, const double* gF, double* gL,
                      double* gR, unsigned* code = nullptr) {
  constexpr int vn = (DIR - 1) % 3, vt1 = DIR % 3, vt2 = (DIR + 1) % 3;
  constexpr int bn = kBX + (DIR - 1) % 3, bt1 = kBX + DIR % 3, bt2 = kBX + (DIR + 1) % 3;
  constexpr int mn = vn, mt1 = vt1, mt2 = vt2;
  const double r1 = arcp(gamma - 1.0), r2 = gamma * r1;
  const double hf = 1.001;
  for (int k = 0; k < 9; ++k) {
    gL[k] = 0.0;
    gR[k] = 0.0;
  }
  // GLM fluxes (flux_solver.f90:580-581), linear in the face states
  gL[kPS] += 0.5 * gF[bn] + 0.5 * ch * gF[kPS];
  gR[kPS] += 0.5 * gF[bn] - 0.5 * ch * gF[kPS];
  gL[bn] += 0.5 * ch * gF[bn] + 0.5 * (ch * ch) * gF[kPS];
  gR[bn] += -0.5 * ch * gF[bn] + 0.5 * (ch * ch) * gF[kPS];

  Side sL, sR;
  side_fwd<DIR, MODE>(L, gamma, r1, r2, sL, code, tape::kClampL);
  side_fwd<DIR, MODE>(R, gamma, r1, r2, sR, code, tape::kClampR);
  SideG gsL, gsR;
  zero(gsL);
  zero(gsR);
  const int fl[7] = {kRO, mn, mt1, mt2, kEN, bt1, bt2};  // slots set from the physical fluxes

  // fmax2(aL, aR) of a = (Q + sq)/(2 rho): aL < aR <=> (Q + sq)_L rho_R < (Q + sq)_R rho_L
  const bool aRsel = decide<MODE>((sL.Q + sL.sq) * R[kRO] < (sR.Q + sR.sq) * L[kRO], code, tape::kArSel);
  if (aRsel)
    side_cf(R, sR);
  else
    side_cf(L, sL);
  const double amax = aRsel ? sR.a : sL.a;
  const double icf = (amax > 0.0) ? arsqrt(amax) : 0.0;
  const double cf = amax * icf;
  const bool minR = decide<MODE>(R[vn] < L[vn], code, tape::kMinR);  // fmin2(vnL, vnR)
  const bool maxR = decide<MODE>(R[vn] > L[vn], code, tape::kMaxR);  // fmax2(vnL, vnR)
  const double SL = (minR ? R[vn] : L[vn]) - cf;
  const double SR = (maxR ? R[vn] : L[vn]) + cf;
  double gSL = 0.0, gSR = 0.0;

  bool fxL = false, fxR = false;  // the side's physical flux takes part in the face flux
  if (decide<MODE>(SL >= 0.0, code, tape::kFL)) {
    for (int q = 0; q < 7; ++q) gsL.F[fl[q]] += gF[fl[q]];
    fxL = true;
  } else if (decide<MODE>(SR <= 0.0, code, tape::kFR)) {
    for (int q = 0; q < 7; ++q) gsR.F[fl[q]] += gF[fl[q]];
    fxR = true;
  } else {
    const double ih = arcp(SR - SL);
    // HLL state: rho, the normal momentum and Bn here; the tangential
    // components only in the HLLC-G fallback, the one branch that uses them
    double NU[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Uh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    auto hll_m = [&](int k) {  // momentum components (conserved Um)
      NU[k] = SR * sR.Um[k] - SL * sL.Um[k] - sR.F[k] + sL.F[k];
      Uh[k] = ih * NU[k];
    };
    auto hll_p = [&](int k) {  // rho and B (primitive = conserved)
      NU[k] = SR * R[k] - SL * L[k] - sR.F[k] + sL.F[k];
      Uh[k] = ih * NU[k];
    };
    hll_m(mn);
    hll_p(kRO);
    hll_p(bn);
    const double iUr = arcp(Uh[kRO]);
    const double aM = Uh[mn] * iUr;
    const double tL = SL - L[vn], tR = SR - R[vn];
    const double pts = sL.pt + L[kRO] * tL * (aM - L[vn]);
    const double eL = SL - aM, eR = SR - aM;
    const double ieL = arcp(eL), ieR = arcp(eR);
    const double roL = L[kRO] * tL * ieL, roR = R[kRO] * tR * ieR;
    const double Ubn = Uh[bn];
    const bool bneg = decide<MODE>(std::signbit(Ubn), code, tape::kBnNeg);
    const double aUbn = (MODE == tape::kNone) ? std::fabs(Ubn) : (bneg ? -Ubn : Ubn);
    const double isqL = arsqrt(roL), isqR = arsqrt(roR);
    const double sqL = roL * isqL, sqR = roR * isqR;
    const double aVL = aUbn * isqL, aVR = aUbn * isqR;

    double gUh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double gih = 0.0, gaM = 0.0, gpts = 0.0, gtL = 0.0, gtR = 0.0, geL = 0.0, geR = 0.0;
    double groL = 0.0, groR = 0.0, gaVL = 0.0, gaVR = 0.0, gsqL = 0.0, gsqR = 0.0;

    const bool gbr = decide<MODE>((SL >= (aM - hf * aVL)) || ((aM + hf * aVR) >= SR), code, tape::kG);
    if (gbr) {
      // ---- HLLC-G fallback (flux_solver.f90:450-476) ----
      side_fwd_tan<DIR>(L, r2, sL);
      side_fwd_tan<DIR>(R, r2, sR);
      fxL = fxR = true;
      hll_m(mt1);
      hll_m(mt2);
      hll_p(bt1);
      hll_p(bt2);
      const double f2g = SL * SR;
      double gf2g = 0.0;
      const int bts[2] = {bt1, bt2};
      for (int q = 0; q < 2; ++q) {
        const int bt = bts[q];
        const double N1 = SR * sL.F[bt] - SL * sR.F[bt] + f2g * (R[bt] - L[bt]);
        gih += gF[bt] * N1;
        const double gN1 = ih * gF[bt];
        gSR += gN1 * sL.F[bt];
        gsL.F[bt] += gN1 * SR;
        gSL -= gN1 * sR.F[bt];
        gsR.F[bt] -= gN1 * SL;
        gf2g += gN1 * (R[bt] - L[bt]);
        gR[bt] += gN1 * f2g;
        gL[bt] -= gN1 * f2g;
      }
      gSL += gf2g * SR;
      gSR += gf2g * SL;
      const double at1 = Uh[mt1] * iUr, at2 = Uh[mt2] * iUr;
      double gat1 = 0.0, gat2 = 0.0;
      const bool left = decide<MODE>(!std::signbit(aM), code, tape::kGLeft);  // 0.5 + sign(0.5, aM) == 1
      const double* S = left ? L : R;
      const Side& sS = left ? sL : sR;
      SideG& gsS = left ? gsL : gsR;
      double* gS = left ? gL : gR;
      const double Sw = left ? SL : SR;
      const double tS = left ? tL : tR, ieS = left ? ieL : ieR, roS = left ? roL : roR;
      const double QS = sS.vB - aM * Ubn - at1 * Uh[bt1] - at2 * Uh[bt2];
      const double numS = tS * sS.UE - sS.pt * S[vn] + pts * aM + Ubn * QS;
      const double enS = numS * ieS;
      double gSw = gF[mn] * (roS * aM - sS.Um[mn]) + gF[mt1] * (roS * at1 - sS.Um[mt1]) +
                   gF[mt2] * (roS * at2 - sS.Um[mt2]) + gF[kEN] * (enS - sS.UE) + gF[kRO] * (roS - S[kRO]);
      const double groS = Sw * (gF[mn] * aM + gF[mt1] * at1 + gF[mt2] * at2 + gF[kRO]);
      gaM += Sw * roS * gF[mn];
      gat1 += Sw * roS * gF[mt1];
      gat2 += Sw * roS * gF[mt2];
      gsS.Um[mn] -= Sw * gF[mn];
      gsS.Um[mt1] -= Sw * gF[mt1];
      gsS.Um[mt2] -= Sw * gF[mt2];
      const double genS = Sw * gF[kEN];
      gsS.UE -= Sw * gF[kEN];
      gS[kRO] -= Sw * gF[kRO];
      gsS.F[mn] += gF[mn];
      gsS.F[mt1] += gF[mt1];
      gsS.F[mt2] += gF[mt2];
      gsS.F[kEN] += gF[kEN];
      gsS.F[kRO] += gF[kRO];
      // en = num / e
      const double gnum = genS * ieS;
      double geS = -genS * enS * ieS, gtS = 0.0;
      gtS += gnum * sS.UE;
      gsS.UE += gnum * tS;
      gsS.pt -= gnum * S[vn];
      gS[vn] -= gnum * sS.pt;
      gpts += gnum * aM;
      gaM += gnum * pts;
      gUh[bn] += gnum * QS;
      const double gQ = gnum * Ubn;
      gsS.vB += gQ;
      gaM -= gQ * Ubn;
      gUh[bn] -= gQ * aM;
      gat1 -= gQ * Uh[bt1];
      gUh[bt1] -= gQ * at1;
      gat2 -= gQ * Uh[bt2];
      gUh[bt2] -= gQ * at2;
      gUh[mt1] += gat1 * iUr;
      gUh[kRO] -= gat1 * at1 * iUr;
      gUh[mt2] += gat2 * iUr;
      gUh[kRO] -= gat2 * at2 * iUr;
      if (left) {
        gSL += gSw;
        groL += groS;
        geL += geS;
        gtL += gtS;
      } else {
        gSR += gSw;
        groR += groS;
        geR += geS;
        gtR += gtS;
      }
    } else {
      // ---- HLLD (flux_solver.f90:482-572) ----
      // Region first (it needs only aM and the Alfven speeds), then the
      // intermediate states it uses: F(L*) needs L* only, F(R*) R* only,
      // the central states both (the forward kernel does the same).
      const double aL1 = aM - aVL, aR1 = aM + aVR;
      const bool sLs = decide<MODE>(aL1 >= 0.0, code, tape::kLS);
      const bool sRs = !sLs && decide<MODE>(aR1 <= 0.0, code, tape::kRS);
      double dL = 0, iL = 0, kL = 0, UL1bt1 = 0, UL1bt2 = 0, dmL = 0, vt1L = 0, vt2L = 0, QL = 0, UL1E = 0;
      double UL1m[3] = {0, 0, 0};
      if (!sRs) {  // L* (flux_solver.f90:482-493)
        dL = L[kRO] * tL * eL - Ubn * Ubn;
        iL = arcp(dL);
        kL = L[kRO] * (tL * tL) - Ubn * Ubn;
        UL1bt1 = L[bt1] * iL * kL;
        UL1bt2 = L[bt2] * iL * kL;
        dmL = aM - L[vn];
        vt1L = L[vt1] - iL * Ubn * L[bt1] * dmL;
        vt2L = L[vt2] - iL * Ubn * L[bt2] * dmL;
        QL = sL.vB - aM * Ubn - vt1L * UL1bt1 - vt2L * UL1bt2;
        const double numL = tL * sL.UE - sL.pt * L[vn] + pts * aM + Ubn * QL;
        UL1E = numL * ieL;
        UL1m[mn] = roL * aM;
        UL1m[mt1] = roL * vt1L;
        UL1m[mt2] = roL * vt2L;
      }
      double dR = 0, iR = 0, kR = 0, UR1bt1 = 0, UR1bt2 = 0, dmR = 0, vt1R = 0, vt2R = 0, QR = 0, UR1E = 0;
      double UR1m[3] = {0, 0, 0};
      if (!sLs) {  // R* (flux_solver.f90:496-507)
        dR = R[kRO] * tR * eR - Ubn * Ubn;
        iR = arcp(dR);
        kR = R[kRO] * (tR * tR) - Ubn * Ubn;
        UR1bt1 = R[bt1] * iR * kR;
        UR1bt2 = R[bt2] * iR * kR;
        dmR = aM - R[vn];
        vt1R = R[vt1] - iR * Ubn * R[bt1] * dmR;
        vt2R = R[vt2] - iR * Ubn * R[bt2] * dmR;
        QR = sR.vB - aM * Ubn - vt1R * UR1bt1 - vt2R * UR1bt2;
        const double numR = tR * sR.UE - sR.pt * R[vn] + pts * aM + Ubn * QR;
        UR1E = numR * ieR;
        UR1m[mn] = roR * aM;
        UR1m[mt1] = roR * vt1R;
        UR1m[mt2] = roR * vt2R;
      }

      double gUL1m[3] = {0, 0, 0}, gUR1m[3] = {0, 0, 0};
      double gUL1E = 0, gUR1E = 0, gUL1bt1 = 0, gUL1bt2 = 0, gUR1bt1 = 0, gUR1bt2 = 0;
      double gvt1L = 0, gvt2L = 0, gvt1R = 0, gvt2R = 0;

      if (sLs) {  // F(L*)
        for (int k = 0; k < 3; ++k) {
          gSL += gF[k] * (UL1m[k] - sL.Um[k]);
          gUL1m[k] += SL * gF[k];
          gsL.Um[k] -= SL * gF[k];
        }
        gSL += gF[kEN] * (UL1E - sL.UE) + gF[kRO] * (roL - L[kRO]) + gF[bt1] * (UL1bt1 - L[bt1]) +
               gF[bt2] * (UL1bt2 - L[bt2]);
        gUL1E += SL * gF[kEN];
        gsL.UE -= SL * gF[kEN];
        groL += SL * gF[kRO];
        gL[kRO] -= SL * gF[kRO];
        gUL1bt1 += SL * gF[bt1];
        gL[bt1] -= SL * gF[bt1];
        gUL1bt2 += SL * gF[bt2];
        gL[bt2] -= SL * gF[bt2];
        for (int q = 0; q < 7; ++q) gsL.F[fl[q]] += gF[fl[q]];
        fxL = true;
      } else if (sRs) {  // F(R*)
        for (int k = 0; k < 3; ++k) {
          gSR += gF[k] * (UR1m[k] - sR.Um[k]);
          gUR1m[k] += SR * gF[k];
          gsR.Um[k] -= SR * gF[k];
        }
        gSR += gF[kEN] * (UR1E - sR.UE) + gF[kRO] * (roR - R[kRO]) + gF[bt1] * (UR1bt1 - R[bt1]) +
               gF[bt2] * (UR1bt2 - R[bt2]);
        gUR1E += SR * gF[kEN];
        gsR.UE -= SR * gF[kEN];
        groR += SR * gF[kRO];
        gR[kRO] -= SR * gF[kRO];
        gUR1bt1 += SR * gF[bt1];
        gR[bt1] -= SR * gF[bt1];
        gUR1bt2 += SR * gF[bt2];
        gR[bt2] -= SR * gF[bt2];
        for (int q = 0; q < 7; ++q) gsR.F[fl[q]] += gF[fl[q]];
        fxR = true;
      } else {  // central states
        const double rLs = sqL, rRs = sqR;
        const double ic = arcp(rLs + rRs);
        const double sg = (MODE == tape::kNone) ? std::copysign(1.0, Ubn) : (bneg ? -1.0 : 1.0);
        const double at1 = ic * (rLs * vt1L + rRs * vt1R + (UR1bt1 - UL1bt1) * sg);
        const double at2 = ic * (rLs * vt2L + rRs * vt2R + (UR1bt2 - UL1bt2) * sg);
        const double U2bt1 = ic * (rLs * UR1bt1 + rRs * UL1bt1 + rLs * rRs * (vt1R - vt1L) * sg);
        const double U2bt2 = ic * (rLs * UR1bt2 + rRs * UL1bt2 + rLs * rRs * (vt2R - vt2L) * sg);
        double gat1 = 0, gat2 = 0, gU2bt1 = 0, gU2bt2 = 0, grLs = 0, grRs = 0, gic = 0;
        const bool left = decide<MODE>(aM >= 0.0, code, tape::kSSLeft);
        fxL = left;
        fxR = !left;
        const double* S = left ? L : R;
        const Side& sS = left ? sL : sR;
        SideG& gsS = left ? gsL : gsR;
        double* gS = left ? gL : gR;
        const double Sw = left ? SL : SR;
        const double roS = left ? roL : roR;
        const double a1 = left ? aL1 : aR1;
        const double rSs = left ? rLs : rRs;
        const double* US1m = left ? UL1m : UR1m;
        const double US1E = left ? UL1E : UR1E;
        const double US1bt1 = left ? UL1bt1 : UR1bt1, US1bt2 = left ? UL1bt2 : UR1bt2;
        const double vt1S = left ? vt1L : vt1R, vt2S = left ? vt2L : vt2R;
        const double Pq = vt1S * US1bt1 + vt2S * US1bt2 - at1 * U2bt1 - at2 * U2bt2;
        const double sgS = left ? -1.0 : 1.0;  // U2E = US1E -/+ rSs*Pq*sg
        const double U2E = US1E + sgS * (rSs * Pq * sg);
        double U2m[3];
        U2m[mn] = roS * aM;
        U2m[mt1] = roS * at1;
        U2m[mt2] = roS * at2;
        // F = a1*U2 - (a1 - Sw)*US1 - Sw*US + FS
        const double c1 = a1 - Sw;
        double ga1 = 0.0, gSw = 0.0, gU2m[3] = {0, 0, 0}, gUS1m[3] = {0, 0, 0}, gU2E = 0, gUS1E = 0;
        double groS = 0.0, gUS1bt1 = 0, gUS1bt2 = 0, gvt1S = 0, gvt2S = 0;
        for (int k = 0; k < 3; ++k) {
          ga1 += gF[k] * (U2m[k] - US1m[k]);
          gSw += gF[k] * (US1m[k] - sS.Um[k]);
          gU2m[k] += a1 * gF[k];
          gUS1m[k] -= c1 * gF[k];
          gsS.Um[k] -= Sw * gF[k];
        }
        ga1 += gF[kEN] * (U2E - US1E) + gF[kRO] * (roS - roS) + gF[bt1] * (U2bt1 - US1bt1) + gF[bt2] * (U2bt2 - US1bt2);
        gSw += gF[kEN] * (US1E - sS.UE) + gF[kRO] * (roS - S[kRO]) + gF[bt1] * (US1bt1 - S[bt1]) +
               gF[bt2] * (US1bt2 - S[bt2]);
        gU2E += a1 * gF[kEN];
        gUS1E -= c1 * gF[kEN];
        gsS.UE -= Sw * gF[kEN];
        groS += a1 * gF[kRO] - c1 * gF[kRO];
        gS[kRO] -= Sw * gF[kRO];
        gU2bt1 += a1 * gF[bt1];
        gUS1bt1 -= c1 * gF[bt1];
        gS[bt1] -= Sw * gF[bt1];
        gU2bt2 += a1 * gF[bt2];
        gUS1bt2 -= c1 * gF[bt2];
        gS[bt2] -= Sw * gF[bt2];
        for (int q = 0; q < 7; ++q) gsS.F[fl[q]] += gF[fl[q]];
        // U2m
        groS += gU2m[mn] * aM + gU2m[mt1] * at1 + gU2m[mt2] * at2;
        gaM += gU2m[mn] * roS;
        gat1 += gU2m[mt1] * roS;
        gat2 += gU2m[mt2] * roS;
        // U2E = US1E + sgS*(rSs*Pq*sg)
        gUS1E += gU2E;
        const double grSs = gU2E * sgS * Pq * sg;
        const double gPq = gU2E * sgS * rSs * sg;
        gvt1S += gPq * US1bt1;
        gUS1bt1 += gPq * vt1S;
        gvt2S += gPq * US1bt2;
        gUS1bt2 += gPq * vt2S;
        gat1 -= gPq * U2bt1;
        gU2bt1 -= gPq * at1;
        gat2 -= gPq * U2bt2;
        gU2bt2 -= gPq * at2;
        // scatter the side-selected adjoints
        if (left) {
          gSL += gSw;
          groL += groS;
          grLs += grSs;
          for (int k = 0; k < 3; ++k) gUL1m[k] += gUS1m[k];
          gUL1E += gUS1E;
          gUL1bt1 += gUS1bt1;
          gUL1bt2 += gUS1bt2;
          gvt1L += gvt1S;
          gvt2L += gvt2S;
          gaM += ga1;  // aL1 = aM - aVL
          gaVL -= ga1;
        } else {
          gSR += gSw;
          groR += groS;
          grRs += grSs;
          for (int k = 0; k < 3; ++k) gUR1m[k] += gUS1m[k];
          gUR1E += gUS1E;
          gUR1bt1 += gUS1bt1;
          gUR1bt2 += gUS1bt2;
          gvt1R += gvt1S;
          gvt2R += gvt2S;
          gaM += ga1;  // aR1 = aM + aVR
          gaVR += ga1;
        }
        // U2bt = ic*(rLs*UR1bt + rRs*UL1bt + rLs*rRs*(vtR - vtL)*sg)
        {
          const double Nb = rLs * UR1bt1 + rRs * UL1bt1 + rLs * rRs * (vt1R - vt1L) * sg;
          gic += gU2bt1 * Nb;
          const double gN = ic * gU2bt1;
          grLs += gN * UR1bt1 + gN * rRs * (vt1R - vt1L) * sg;
          grRs += gN * UL1bt1 + gN * rLs * (vt1R - vt1L) * sg;
          gUR1bt1 += gN * rLs;
          gUL1bt1 += gN * rRs;
          gvt1R += gN * rLs * rRs * sg;
          gvt1L -= gN * rLs * rRs * sg;
        }
        {
          const double Nb = rLs * UR1bt2 + rRs * UL1bt2 + rLs * rRs * (vt2R - vt2L) * sg;
          gic += gU2bt2 * Nb;
          const double gN = ic * gU2bt2;
          grLs += gN * UR1bt2 + gN * rRs * (vt2R - vt2L) * sg;
          grRs += gN * UL1bt2 + gN * rLs * (vt2R - vt2L) * sg;
          gUR1bt2 += gN * rLs;
          gUL1bt2 += gN * rRs;
          gvt2R += gN * rLs * rRs * sg;
          gvt2L -= gN * rLs * rRs * sg;
        }
        // at = ic*(rLs*vtL + rRs*vtR + (UR1bt - UL1bt)*sg)
        {
          const double Na = rLs * vt1L + rRs * vt1R + (UR1bt1 - UL1bt1) * sg;
          gic += gat1 * Na;
          const double gN = ic * gat1;
          grLs += gN * vt1L;
          gvt1L += gN * rLs;
          grRs += gN * vt1R;
          gvt1R += gN * rRs;
          gUR1bt1 += gN * sg;
          gUL1bt1 -= gN * sg;
        }
        {
          const double Na = rLs * vt2L + rRs * vt2R + (UR1bt2 - UL1bt2) * sg;
          gic += gat2 * Na;
          const double gN = ic * gat2;
          grLs += gN * vt2L;
          gvt2L += gN * rLs;
          grRs += gN * vt2R;
          gvt2R += gN * rRs;
          gUR1bt2 += gN * sg;
          gUL1bt2 -= gN * sg;
        }
        const double gden = -gic * ic * ic;
        grLs += gden;
        grRs += gden;
        gsqL += grLs;
        gsqR += grRs;
      }
      // ---- back through the L* and R* states ----
      if (!sRs) {  // L
        groL += gUL1m[mn] * aM + gUL1m[mt1] * vt1L + gUL1m[mt2] * vt2L;
        gaM += gUL1m[mn] * roL;
        gvt1L += gUL1m[mt1] * roL;
        gvt2L += gUL1m[mt2] * roL;
        const double gnum = gUL1E * ieL;
        geL -= gUL1E * UL1E * ieL;
        gtL += gnum * sL.UE;
        gsL.UE += gnum * tL;
        gsL.pt -= gnum * L[vn];
        gL[vn] -= gnum * sL.pt;
        gpts += gnum * aM;
        gaM += gnum * pts;
        gUh[bn] += gnum * QL;
        const double gQ = gnum * Ubn;
        gsL.vB += gQ;
        gaM -= gQ * Ubn;
        gUh[bn] -= gQ * aM;
        gvt1L -= gQ * UL1bt1;
        gUL1bt1 -= gQ * vt1L;
        gvt2L -= gQ * UL1bt2;
        gUL1bt2 -= gQ * vt2L;
        double giL = 0.0, gdmL = 0.0, gkL = 0.0;
        {  // vt1L = L_vt1 - ((iL*Ubn)*L_bt1)*dmL
          gL[vt1] += gvt1L;
          const double gx = -gvt1L;
          giL += gx * Ubn * L[bt1] * dmL;
          gUh[bn] += gx * iL * L[bt1] * dmL;
          gL[bt1] += gx * iL * Ubn * dmL;
          gdmL += gx * iL * Ubn * L[bt1];
        }
        {
          gL[vt2] += gvt2L;
          const double gx = -gvt2L;
          giL += gx * Ubn * L[bt2] * dmL;
          gUh[bn] += gx * iL * L[bt2] * dmL;
          gL[bt2] += gx * iL * Ubn * dmL;
          gdmL += gx * iL * Ubn * L[bt2];
        }
        gaM += gdmL;
        gL[vn] -= gdmL;
        gL[bt1] += gUL1bt1 * iL * kL;
        giL += gUL1bt1 * L[bt1] * kL;
        gkL += gUL1bt1 * L[bt1] * iL;
        gL[bt2] += gUL1bt2 * iL * kL;
        giL += gUL1bt2 * L[bt2] * kL;
        gkL += gUL1bt2 * L[bt2] * iL;
        gL[kRO] += gkL * tL * tL;
        gtL += gkL * 2 * L[kRO] * tL;
        gUh[bn] -= 2 * gkL * Ubn;
        const double gdL = -giL * iL * iL;
        gL[kRO] += gdL * tL * eL;
        gtL += gdL * L[kRO] * eL;
        geL += gdL * L[kRO] * tL;
        gUh[bn] -= 2 * gdL * Ubn;
      }
      if (!sLs) {  // R
        groR += gUR1m[mn] * aM + gUR1m[mt1] * vt1R + gUR1m[mt2] * vt2R;
        gaM += gUR1m[mn] * roR;
        gvt1R += gUR1m[mt1] * roR;
        gvt2R += gUR1m[mt2] * roR;
        const double gnum = gUR1E * ieR;
        geR -= gUR1E * UR1E * ieR;
        gtR += gnum * sR.UE;
        gsR.UE += gnum * tR;
        gsR.pt -= gnum * R[vn];
        gR[vn] -= gnum * sR.pt;
        gpts += gnum * aM;
        gaM += gnum * pts;
        gUh[bn] += gnum * QR;
        const double gQ = gnum * Ubn;
        gsR.vB += gQ;
        gaM -= gQ * Ubn;
        gUh[bn] -= gQ * aM;
        gvt1R -= gQ * UR1bt1;
        gUR1bt1 -= gQ * vt1R;
        gvt2R -= gQ * UR1bt2;
        gUR1bt2 -= gQ * vt2R;
        double giR = 0.0, gdmR = 0.0, gkR = 0.0;
        {
          gR[vt1] += gvt1R;
          const double gx = -gvt1R;
          giR += gx * Ubn * R[bt1] * dmR;
          gUh[bn] += gx * iR * R[bt1] * dmR;
          gR[bt1] += gx * iR * Ubn * dmR;
          gdmR += gx * iR * Ubn * R[bt1];
        }
        {
          gR[vt2] += gvt2R;
          const double gx = -gvt2R;
          giR += gx * Ubn * R[bt2] * dmR;
          gUh[bn] += gx * iR * R[bt2] * dmR;
          gR[bt2] += gx * iR * Ubn * dmR;
          gdmR += gx * iR * Ubn * R[bt2];
        }
        gaM += gdmR;
        gR[vn] -= gdmR;
        gR[bt1] += gUR1bt1 * iR * kR;
        giR += gUR1bt1 * R[bt1] * kR;
        gkR += gUR1bt1 * R[bt1] * iR;
        gR[bt2] += gUR1bt2 * iR * kR;
        giR += gUR1bt2 * R[bt2] * kR;
        gkR += gUR1bt2 * R[bt2] * iR;
        gR[kRO] += gkR * tR * tR;
        gtR += gkR * 2 * R[kRO] * tR;
        gUh[bn] -= 2 * gkR * Ubn;
        const double gdR = -giR * iR * iR;
        gR[kRO] += gdR * tR * eR;
        gtR += gdR * R[kRO] * eR;
        geR += gdR * R[kRO] * tR;
        gUh[bn] -= 2 * gdR * Ubn;
      }
    }
    // ---- common tail: Alfven speeds, rho*, total pressure, aM, HLL state ----
    double gaUbn = gaVL * isqL + gaVR * isqR;
    gsqL -= gaVL * aVL * isqL;
    gsqR -= gaVR * aVR * isqR;
    groL += (sqL > 0.0) ? gsqL * 0.5 * isqL : 0.0;
    groR += (sqR > 0.0) ? gsqR * 0.5 * isqR : 0.0;
    // d|Bn|/dBn: the sign; at Bn == 0 it is 0 when recomputed (a central
    // difference there sees no slope) and the recorded sign under a tape
    if (MODE == tape::kNone)
      gUh[bn] += (Ubn > 0.0) ? gaUbn : ((Ubn < 0.0) ? -gaUbn : 0.0);
    else
      gUh[bn] += bneg ? -gaUbn : gaUbn;
    gL[kRO] += groL * tL * ieL;
    gtL += groL * L[kRO] * ieL;
    geL -= groL * roL * ieL;
    gR[kRO] += groR * tR * ieR;
    gtR += groR * R[kRO] * ieR;
    geR -= groR * roR * ieR;
    gSL += geL;
    gaM -= geL;
    gSR += geR;
    gaM -= geR;
    gsL.pt += gpts;
    gL[kRO] += gpts * tL * (aM - L[vn]);
    gtL += gpts * L[kRO] * (aM - L[vn]);
    gaM += gpts * L[kRO] * tL;
    gL[vn] -= gpts * L[kRO] * tL;
    gSL += gtL;
    gL[vn] -= gtL;
    gSR += gtR;
    gR[vn] -= gtR;
    gUh[mn] += gaM * iUr;
    gUh[kRO] -= gaM * aM * iUr;
    auto hll_m_adj = [&](int k) {
      gih += gUh[k] * NU[k];
      const double gN = ih * gUh[k];
      gSR += gN * sR.Um[k];
      gsR.Um[k] += gN * SR;
      gSL -= gN * sL.Um[k];
      gsL.Um[k] -= gN * SL;
      gsR.F[k] -= gN;
      gsL.F[k] += gN;
    };
    auto hll_p_adj = [&](int k) {
      gih += gUh[k] * NU[k];
      const double gN = ih * gUh[k];
      gSR += gN * R[k];
      gR[k] += gN * SR;
      gSL -= gN * L[k];
      gL[k] -= gN * SL;
      gsR.F[k] -= gN;
      gsL.F[k] += gN;
    };
    hll_m_adj(mn);
    hll_p_adj(kRO);
    hll_p_adj(bn);
    if (gbr) {  // the tangential components carry gradient only there
      hll_m_adj(mt1);
      hll_m_adj(mt2);
      hll_p_adj(bt1);
      hll_p_adj(bt2);
    }
    gSR -= gih * ih * ih;
    gSL += gih * ih * ih;
  }
  // ---- wave speeds ----
  const double gcf = -gSL + gSR;
  if (minR)
    gR[vn] += gSL;
  else
    gL[vn] += gSL;
  if (maxR)
    gR[vn] += gSR;
  else
    gL[vn] += gSR;
  const double gamax = gcf * 0.5 * icf;
  if (aRsel)
    gsR.a += gamax;
  else
    gsL.a += gamax;
  side_adj<DIR>(L, gamma, r1, r2, sL, gsL, gL, fxL, !aRsel);
  side_adj<DIR>(R, gamma, r1, r2, sR, gsR, gR, fxR, aRsel);
}

// Selection code (tape::kLim*) of the minmod (type 1) / MC (type 2)
// reconstruction of one cell, with the forward's tie rule (fmin2: the first
// operand wins ties; opposite signs -> zero slope).
OMHD_HD unsigned char recon_code(int type, double wm, double w0, double wp) {
  const double gA = w0 - wm, gB = wp - w0;
  if (std::signbit(gA) != std::signbit(gB)) return tape::kLimZero;
  const double aA = std::fabs(gA), aB = std::fabs(gB);
  if (type == 2) {
    const double gC = 0.25 * (wp - wm);
    const double m1 = (aB < aA) ? aB : aA;
    if (std::fabs(gC) < m1)
      return (unsigned char)(tape::kLimC | ((std::signbit(gA) != std::signbit(gC)) ? tape::kLimCNeg : 0));
  }
  return (aB < aA) ? tape::kLimB : tape::kLimA;
}

// Adjoint of one cell's reconstruction with a given selection code:
// left = w0 + grad (upper face), right = w0 - grad (lower face), grad the
// selected slope times 0.5 (minmod) or 1 (MC; gC = (wp - wm)/4 with its sign).
OMHD_HD void recon_vjp_code(int type, unsigned char code, double gleft, double gright, double& gwm, double& gw0,
                            double& gwp) {
  gw0 += gleft + gright;
  const double c = (type == 2) ? 1.0 : 0.5;
  const double gg = c * (gleft - gright);
  switch (code & 3) {
    case tape::kLimA:
      gw0 += gg;
      gwm -= gg;
      break;
    case tape::kLimB:
      gwp += gg;
      gw0 -= gg;
      break;
    case tape::kLimC: {
      const double k = (code & tape::kLimCNeg) ? -0.25 * gg : 0.25 * gg;
      gwp += k;
      gwm -= k;
      break;
    }
    default:
      break;
  }
}

// minmod (type 1) / MC (type 2) reconstruction of one cell and its adjoint,
// selection recomputed from the cell and its neighbours.
OMHD_HD void recon_vjp(int type, double wm, double w0, double wp, double gleft, double gright, double& gwm,
                       double& gw0, double& gwp) {
  recon_vjp_code(type, recon_code(type, wm, w0, wp), gleft, gright, gwm, gw0, gwp);
}

// u2v (u2v.f90:24-27) adjoint: gU += (dw/dU)^T gw for w = (v, p, rho, B, psi).
OMHD_HD void u2v_vjp(const double* U, double gamma, const double* gw, double* gU) {
  const double ro = U[kRO], ir = arcp(ro);
  const double v0 = U[0] * ir, v1 = U[1] * ir, v2 = U[2] * ir;
  const double f1 = gamma - 1;
  const double gp = gw[kPR];
  // v_k = m_k/rho
  gU[0] += gw[0] * ir;
  gU[1] += gw[1] * ir;
  gU[2] += gw[2] * ir;
  gU[kRO] -= (gw[0] * v0 + gw[1] * v1 + gw[2] * v2) * ir;
  // p = f1*(E - 0.5*(v.m + B.B)) with v.m = |m|^2/rho
  gU[kEN] += f1 * gp;
  gU[0] -= f1 * gp * v0;
  gU[1] -= f1 * gp * v1;
  gU[2] -= f1 * gp * v2;
  gU[kRO] += f1 * gp * 0.5 * (v0 * v0 + v1 * v1 + v2 * v2);
  gU[5] -= f1 * gp * U[5];
  gU[6] -= f1 * gp * U[6];
  gU[7] -= f1 * gp * U[7];
  // rho, B, psi pass through
  gU[kRO] += gw[kRO];
  gU[5] += gw[5];
  gU[6] += gw[6];
  gU[7] += gw[7];
  gU[kPS] += gw[kPS];
}

}  // namespace adj
}  // namespace omhd
