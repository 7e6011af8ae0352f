/*
 * omhd_oracle.c -- CPU restatement of OpenMHD's finite-volume MHD step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  The product never links or calls
 * this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs
 * do.  Parity status: PINNED to the reference's own source, executed through
 * its mechanical C translation (oracle/ref.py); see omhd_oracle.h.
 *
 * Every routine restates one reference routine in the reference's own
 * operation order.  Fortran semantics kept on purpose:
 *   - sign(a,b) == copysign(|a|,b), signed zero honoured;
 *   - x**2 == x*x; left-to-right evaluation of +,-,*,/ chains;
 *   - dot_product summed left to right;
 *   - literal constants computed in double at run time from gamma.
 * Build with -O2 -ffp-contract=off -fno-fast-math (oracle/Makefile).
 * Loops carry OpenMP pragmas where the reference carries !$omp; reductions are
 * min/max only, so the OpenMP build is bitwise identical to the serial one.
 */
#include "omhd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NV 9
#define IDX(i, j, k) ((size_t)(i) + (size_t)ix * ((size_t)(j) + (size_t)jx * (size_t)(k)))

static double g_gamma = 5.0 / 3.0; /* param.h:3 */

void omo_set_gamma(double gamma) { g_gamma = gamma; }
double omo_get_gamma(void) { return g_gamma; }

static inline double fsign(double a, double b) { return copysign(fabs(a), b); }
static inline double fmin2(double a, double b) { return (b < a) ? b : a; }
static inline double fmax2(double a, double b) { return (b > a) ? b : a; }

/* interior range along an axis of extent n, in 0-based indices:
 * reference min(2,n)..max(1,n-1) (1-based) */
static inline int lo_of(int n) { return (n < 2 ? n : 2) - 1; }
static inline int hi_of(int n) { return (n - 1 > 1 ? n - 1 : 1) - 1; }

/* ---------------------------------------------------------------------
 * u2v: 2D_basic/u2v.f90:1-46 ; 3D_basic/u2v.f90:1-48
 * ------------------------------------------------------------------- */
int omo_u2v(const double* U, double* V, int ix, int jx, int kx, omo_err* err) {
  const size_t n = (size_t)ix * jx * kx;
  const double f1 = g_gamma - 1; /* u2v.f90:11 */
  double prmin = U[OMO_EN * n + 0];
  double rhomin = U[OMO_RO * n + 0];
#pragma omp parallel for reduction(min : prmin, rhomin) schedule(static)
  for (long long c = 0; c < (long long)n; ++c) {
    const double ro = U[OMO_RO * n + c];
    const double mx = U[OMO_MX * n + c], my = U[OMO_MY * n + c], mz = U[OMO_MZ * n + c];
    const double vx = mx / ro, vy = my / ro, vz = mz / ro; /* u2v.f90:24 */
    const double rv2 = vx * mx + vy * my + vz * mz;
    const double bx = U[OMO_BX * n + c], by = U[OMO_BY * n + c], bz = U[OMO_BZ * n + c];
    const double B2 = bx * bx + by * by + bz * bz;
    const double pr = f1 * (U[OMO_EN * n + c] - 0.5 * (rv2 + B2)); /* u2v.f90:27 */
    V[OMO_VX * n + c] = vx;
    V[OMO_VY * n + c] = vy;
    V[OMO_VZ * n + c] = vz;
    V[OMO_PR * n + c] = pr;
    prmin = fmin2(pr, prmin);
    rhomin = fmin2(ro, rhomin);
  }
  if (prmin <= 0 || rhomin <= 0) { /* u2v.f90:36-45: minloc, then stop */
    const double* a = (prmin <= 0) ? (V + OMO_PR * n) : (U + OMO_RO * n);
    size_t best = 0;
    for (size_t c = 1; c < n; ++c)
      if (a[c] < a[best]) best = c;
    if (err) {
      err->code = (prmin <= 0) ? OMO_NEG_PRESSURE : OMO_NEG_DENSITY;
      err->i = (int)(best % ix);
      err->j = (int)((best / ix) % jx);
      err->k = (int)(best / ((size_t)ix * jx));
      err->value = a[best];
    }
    return (prmin <= 0) ? OMO_NEG_PRESSURE : OMO_NEG_DENSITY;
  }
  return OMO_OK;
}

/* ---------------------------------------------------------------------
 * limiter: 2D_basic/limiter.f90:1-318 ; 3D_basic/limiter.f90:1-419
 *   type 0 flat (:54-71), 1 minmod (:76-128), 2 MC (:133-188),
 *   3 van Leer (:193-243), 4 Koren (:248-307).
 * dir = 1,2,3.  Face m (0-based) lies between cells m and m+1 along dir.
 * ------------------------------------------------------------------- */
static inline void slopes(int type, double wm, double w0, double wp, double* left, double* right) {
  /* returns wR(m-1) (= *right: the left-going state at the lower face) and
   * wL(m) (= *left) for cell m with neighbours wm, wp */
  const double f6 = 1.0 / 6.0; /* limiter.f90:22 */
  double gA = (w0 - wm);
  double gB = (wp - w0);
  double grad, gC;
  switch (type) {
    case 1: /* limiter.f90:98 */
      grad = (fsign(0.25, gA) + fsign(0.25, gB)) * fmin2(fabs(gA), fabs(gB));
      *right = w0 - grad;
      *left = w0 + grad;
      break;
    case 2: /* limiter.f90:141-158 */
      gC = 0.25 * (wp - wm);
      grad = (fsign(0.5, gA) + fsign(0.5, gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      *right = w0 - grad;
      *left = w0 + grad;
      break;
    case 3: /* limiter.f90:201-210 */
      if (gA * gB <= 0)
        grad = 0.0;
      else
        grad = gA * gB / (gA + gB);
      *right = w0 - grad;
      *left = w0 + grad;
      break;
    case 4: /* limiter.f90:256-272 */
      gC = f6 * (2 * gA + gB);
      *right = w0 - (fsign(0.5, gA) + fsign(0.5, gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      gC = f6 * (gA + 2 * gB);
      *left = w0 + (fsign(0.5, gA) + fsign(0.5, gB)) * fmin2(fmin2(fabs(gA), fabs(gB)), fabs(gC));
      break;
    default:
      *right = w0;
      *left = w0;
  }
}

void omo_limiter(const double* wk, double* wL, double* wR, int ix, int jx, int kx, int dir, int type) {
  const int n[3] = {ix, jx, kx};
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  const int d = dir - 1;
  const int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
  const int lo1 = lo_of(n[a1]), hi1 = hi_of(n[a1]);
  const int lo2 = lo_of(n[a2]), hi2 = hi_of(n[a2]);
  const int nd = n[d];
  const size_t s = stride[d];
#pragma omp parallel for collapse(2) schedule(static)
  for (int q2 = lo2; q2 <= hi2; ++q2)
    for (int q1 = lo1; q1 <= hi1; ++q1) {
      const size_t base = (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
      if (type == 0) { /* limiter.f90:54-71: first order */
        for (int m = 0; m < nd - 1; ++m) {
          wL[base + m * s] = wk[base + m * s];
          wR[base + m * s] = wk[base + (m + 1) * s];
        }
        continue;
      }
      wL[base] = wk[base]; /* limiter.f90:82 */
      for (int m = 1; m < nd - 1; ++m) {
        double l, r;
        slopes(type, wk[base + (m - 1) * s], wk[base + m * s], wk[base + (m + 1) * s], &l, &r);
        wR[base + (m - 1) * s] = r;
        wL[base + m * s] = l;
      }
      wR[base + (nd - 2) * s] = wk[base + (nd - 1) * s]; /* limiter.f90:103 */
    }
}

/* HLLD branch histogram (test instrumentation): FL, FR, HLLC-G(L), HLLC-G(R),
 * L*, R*, L**, R**.  Counted only in the serial build. */
static long long g_branch[8];
#ifdef _OPENMP
#define BRANCH(b) ((void)0)
#else
#define BRANCH(b) (++g_branch[(b)])
#endif
void omo_branch_counts(long long out[8], int reset) {
  for (int b = 0; b < 8; ++b) {
    out[b] = g_branch[b];
    if (reset) g_branch[b] = 0;
  }
}

/* ---------------------------------------------------------------------
 * flux_solver: 2D_basic/flux_solver.f90:1-795 ; 3D_basic/flux_solver.f90
 *   LLF :89-148, HLL :153-221, HLLC :226-347, HLLD :352-585, LHLLD :590-789
 * ------------------------------------------------------------------- */
void omo_flux_solver(double* F, const double* VL, const double* VR, double ch, int ix, int jx,
                     int kx, int dir, int type) {
  const size_t n = (size_t)ix * jx * kx;
  const double gamma = g_gamma;
  const double r1 = 1.0 / (gamma - 1.0);   /* flux_solver.f90:38 */
  const double r2 = gamma / (gamma - 1.0); /* flux_solver.f90:39 */
  const double hllg_factor = 1.001;        /* flux_solver.f90:54 */
  const double ch2 = ch * ch;
  memset(F, 0, sizeof(double) * n * NV); /* flux_solver.f90:57 */

  /* direction rotation, flux_solver.f90:62-70 */
  const int vn = OMO_VX + (dir - 1) % 3, vt1 = OMO_VX + dir % 3, vt2 = OMO_VX + (dir + 1) % 3;
  const int bn = OMO_BX + (dir - 1) % 3, bt1 = OMO_BX + dir % 3, bt2 = OMO_BX + (dir + 1) % 3;
  const int mn = OMO_MX + (dir - 1) % 3, mt1 = OMO_MX + dir % 3, mt2 = OMO_MX + (dir + 1) % 3;

  /* loop bounds, flux_solver.f90:73-81 (0-based, inclusive) */
  int is, ie, js, je, ks, ke;
  is = lo_of(ix); ie = hi_of(ix);
  js = lo_of(jx); je = hi_of(jx);
  ks = lo_of(kx); ke = hi_of(kx);
  if (dir == 1) { is = 0; ie = ix - 2; }
  if (dir == 2) { js = 0; je = jx - 2; }
  if (dir == 3) { ks = 0; ke = kx - 2; }

#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        const size_t c = IDX(i, j, k);
        double L[NV], R[NV];
        for (int v = 0; v < NV; ++v) { L[v] = VL[v * n + c]; R[v] = VR[v * n + c]; }
        double UL[4], UR[4];
        double FL[NV], FR[NV];
        double Fo[NV];
        for (int v = 0; v < NV; ++v) { FL[v] = 0.0; FR[v] = 0.0; Fo[v] = 0.0; }
        double v2, B2, vBL, vBR, f1, f2, aL, aR, ptL = 0, ptR = 0, aL1 = 0, aR1 = 0;

        /* VL --> UL, FL (flux_solver.f90:359-372) */
        v2 = L[OMO_VX] * L[OMO_VX] + L[OMO_VY] * L[OMO_VY] + L[OMO_VZ] * L[OMO_VZ];
        B2 = L[OMO_BX] * L[OMO_BX] + L[OMO_BY] * L[OMO_BY] + L[OMO_BZ] * L[OMO_BZ];
        vBL = L[OMO_VX] * L[OMO_BX] + L[OMO_VY] * L[OMO_BY] + L[OMO_VZ] * L[OMO_BZ];
        UL[OMO_MX] = L[OMO_RO] * L[OMO_VX];
        UL[OMO_MY] = L[OMO_RO] * L[OMO_VY];
        UL[OMO_MZ] = L[OMO_RO] * L[OMO_VZ];
        UL[OMO_EN] = 0.5 * (L[OMO_RO] * v2 + B2) + r1 * L[OMO_PR];
        FL[OMO_RO] = L[OMO_RO] * L[vn];
        FL[mn] = L[OMO_RO] * L[vn] * L[vn] - L[bn] * L[bn] + L[OMO_PR] + 0.5 * B2;
        FL[mt1] = L[OMO_RO] * L[vn] * L[vt1] - L[bn] * L[bt1];
        FL[mt2] = L[OMO_RO] * L[vn] * L[vt2] - L[bn] * L[bt2];
        FL[OMO_EN] = (0.5 * L[OMO_RO] * v2 + r2 * L[OMO_PR] + B2) * L[vn] - vBL * L[bn];
        FL[bt1] = L[vn] * L[bt1] - L[bn] * L[vt1];
        FL[bt2] = L[vn] * L[bt2] - L[bn] * L[vt2];
        f1 = gamma * L[OMO_PR];
        f2 = 4 * (L[bn] * L[bn]);
        if (type == 0) {
          aL = sqrt(((f1 + B2) + sqrt((f1 + B2) * (f1 + B2) - f1 * f2)) / (2 * L[OMO_RO])); /* :114 */
        } else {
          aL = ((f1 + B2) + sqrt(fmax2((f1 + B2) * (f1 + B2) - f1 * f2, 0.0))) / (2 * L[OMO_RO]);
          ptL = L[OMO_PR] + 0.5 * B2;
          if (type == 4) { /* LHLLD :619-620 */
            double g1 = L[OMO_RO] * v2;
            aL1 = ((g1 + B2) + sqrt(fmax2((g1 + B2) * (g1 + B2) - g1 * f2, 0.0))) / (2 * L[OMO_RO]);
          }
        }

        /* VR --> UR, FR (flux_solver.f90:381-401) */
        v2 = R[OMO_VX] * R[OMO_VX] + R[OMO_VY] * R[OMO_VY] + R[OMO_VZ] * R[OMO_VZ];
        B2 = R[OMO_BX] * R[OMO_BX] + R[OMO_BY] * R[OMO_BY] + R[OMO_BZ] * R[OMO_BZ];
        vBR = R[OMO_VX] * R[OMO_BX] + R[OMO_VY] * R[OMO_BY] + R[OMO_VZ] * R[OMO_BZ];
        UR[OMO_MX] = R[OMO_RO] * R[OMO_VX];
        UR[OMO_MY] = R[OMO_RO] * R[OMO_VY];
        UR[OMO_MZ] = R[OMO_RO] * R[OMO_VZ];
        UR[OMO_EN] = 0.5 * (R[OMO_RO] * v2 + B2) + r1 * R[OMO_PR];
        FR[OMO_RO] = R[OMO_RO] * R[vn];
        FR[mn] = R[OMO_RO] * R[vn] * R[vn] - R[bn] * R[bn] + R[OMO_PR] + 0.5 * B2;
        FR[mt1] = R[OMO_RO] * R[vn] * R[vt1] - R[bn] * R[bt1];
        FR[mt2] = R[OMO_RO] * R[vn] * R[vt2] - R[bn] * R[bt2];
        FR[OMO_EN] = (0.5 * R[OMO_RO] * v2 + r2 * R[OMO_PR] + B2) * R[vn] - vBR * R[bn];
        FR[bt1] = R[vn] * R[bt1] - R[bn] * R[vt1];
        FR[bt2] = R[vn] * R[bt2] - R[bn] * R[vt2];
        f1 = gamma * R[OMO_PR];
        f2 = 4 * (R[bn] * R[bn]);
        if (type == 0) {
          aR = sqrt(((f1 + B2) + sqrt((f1 + B2) * (f1 + B2) - f1 * f2)) / (2 * R[OMO_RO])); /* :136 */
        } else {
          aR = ((f1 + B2) + sqrt(fmax2((f1 + B2) * (f1 + B2) - f1 * f2, 0.0))) / (2 * R[OMO_RO]);
          ptR = R[OMO_PR] + 0.5 * B2;
          if (type == 4) { /* LHLLD :644-645 */
            double g1 = R[OMO_RO] * v2;
            aR1 = ((g1 + B2) + sqrt(fmax2((g1 + B2) * (g1 + B2) - g1 * f2, 0.0))) / (2 * R[OMO_RO]);
          }
        }

        if (type == 0) {
          /* LLF, flux_solver.f90:138-142 */
          f1 = fmax2(fabs(L[vn]) + aL, fabs(R[vn]) + aR);
          for (int v = OMO_MX; v <= OMO_EN; ++v) Fo[v] = 0.5 * (FL[v] + FR[v] - f1 * (UR[v] - UL[v]));
          Fo[OMO_RO] = 0.5 * (FL[OMO_RO] + FR[OMO_RO] - f1 * (R[OMO_RO] - L[OMO_RO]));
          Fo[bt1] = 0.5 * (FL[bt1] + FR[bt1] - f1 * (R[bt1] - L[bt1]));
          Fo[bt2] = 0.5 * (FL[bt2] + FR[bt2] - f1 * (R[bt2] - L[bt2]));
        } else if (type == 1) {
          /* HLL, flux_solver.f90:205-214 */
          f1 = sqrt(fmax2(aL, aR));
          aL = fmin2(fmin2(L[vn], R[vn]) - f1, 0.0);
          aR = fmax2(fmax2(L[vn], R[vn]) + f1, 0.0);
          f1 = 1.0 / (aR - aL);
          f2 = aL * aR;
          for (int v = OMO_MX; v <= OMO_EN; ++v)
            Fo[v] = f1 * (aR * FL[v] - aL * FR[v] + f2 * (UR[v] - UL[v]));
          Fo[OMO_RO] = f1 * (aR * FL[OMO_RO] - aL * FR[OMO_RO] + f2 * (R[OMO_RO] - L[OMO_RO]));
          Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
          Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
        } else if (type == 2) {
          /* HLLC, flux_solver.f90:281-340 */
          double Uh[NV], aM, at1, at2, pt, roL, roR, enL, enR;
          f1 = sqrt(fmax2(aL, aR));
          aL = fmin2(fmin2(L[vn], R[vn]) - f1, 0.0);
          aR = fmax2(fmax2(L[vn], R[vn]) + f1, 0.0);
          f1 = 1.0 / (aR - aL);
          f2 = aL * aR;
          for (int v = OMO_MX; v <= OMO_MZ; ++v) Uh[v] = f1 * (aR * UR[v] - aL * UL[v] - FR[v] + FL[v]);
          for (int v = OMO_RO; v <= OMO_BZ; ++v) Uh[v] = f1 * (aR * R[v] - aL * L[v] - FR[v] + FL[v]);
          Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
          Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
          f2 = 1 / Uh[OMO_RO];
          aM = Uh[mn] * f2;
          at1 = Uh[mt1] * f2;
          at2 = Uh[mt2] * f2;
          pt = ptL + L[OMO_RO] * (aL - L[vn]) * (aM - L[vn]);
          roL = L[OMO_RO] * (aL - L[vn]) / (aL - aM);
          enL = ((aL - L[vn]) * UL[OMO_EN] - ptL * L[vn] + pt * aM +
                 Uh[bn] * (vBL - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) /
                (aL - aM);
          roR = R[OMO_RO] * (aR - R[vn]) / (aR - aM);
          enR = ((aR - R[vn]) * UR[OMO_EN] - ptR * R[vn] + pt * aM +
                 Uh[bn] * (vBR - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) /
                (aR - aM);
          f1 = 0.5 + fsign(0.5, aM);
          f2 = 1.0 - f1;
          Fo[mn] = f1 * (aL * (roL * aM - UL[mn]) + FL[mn]) + f2 * (aR * (roR * aM - UR[mn]) + FR[mn]);
          Fo[mt1] = f1 * (aL * (roL * at1 - UL[mt1]) + FL[mt1]) + f2 * (aR * (roR * at1 - UR[mt1]) + FR[mt1]);
          Fo[mt2] = f1 * (aL * (roL * at2 - UL[mt2]) + FL[mt2]) + f2 * (aR * (roR * at2 - UR[mt2]) + FR[mt2]);
          Fo[OMO_EN] = f1 * (aL * (enL - UL[OMO_EN]) + FL[OMO_EN]) + f2 * (aR * (enR - UR[OMO_EN]) + FR[OMO_EN]);
          Fo[OMO_RO] = f1 * (aL * (roL - L[OMO_RO]) + FL[OMO_RO]) + f2 * (aR * (roR - R[OMO_RO]) + FR[OMO_RO]);
        } else {
          /* HLLD (type 3) flux_solver.f90:408-576 ; LHLLD (type 4) :648-780 */
          double psi = 0.0;
          if (type == 4) {
            f1 = fmin2(1.0, fmax2(aL1, aR1) / fmax2(aL, aR));
            psi = 2 * sqrt(f1) - f1;
          }
          f1 = sqrt(fmax2(aL, aR));
          aL = fmin2(L[vn], R[vn]) - f1;
          aR = fmax2(L[vn], R[vn]) + f1;
          if (aL >= 0) {
            BRANCH(0);
            for (int v = 0; v < NV; ++v) Fo[v] = FL[v];
          } else if (aR <= 0) {
            BRANCH(1);
            for (int v = 0; v < NV; ++v) Fo[v] = FR[v];
          } else {
            double Uh[NV], UL1[NV], UR1[NV], U2[NV];
            double aM, at1, at2, pt, roL, roR, enL, enR, aVL, aVR, vt1L, vt2L, vt1R, vt2R, roLs, roRs;
            f1 = 1.0 / (aR - aL);
            for (int v = OMO_MX; v <= OMO_MZ; ++v) Uh[v] = f1 * (aR * UR[v] - aL * UL[v] - FR[v] + FL[v]);
            for (int v = OMO_RO; v <= OMO_BZ; ++v) Uh[v] = f1 * (aR * R[v] - aL * L[v] - FR[v] + FL[v]);
            aM = Uh[mn] / Uh[OMO_RO];
            if (type == 4) {
              pt = (R[OMO_RO] * ptL * (aR - R[vn]) - L[OMO_RO] * ptR * (aL - L[vn]) +
                    psi * L[OMO_RO] * R[OMO_RO] * (aR - R[vn]) * (aL - L[vn]) * (R[vn] - L[vn])) /
                   (R[OMO_RO] * (aR - R[vn]) - L[OMO_RO] * (aL - L[vn]));
            } else {
              pt = ptL + L[OMO_RO] * (aL - L[vn]) * (aM - L[vn]);
            }
            roL = L[OMO_RO] * (aL - L[vn]) / (aL - aM);
            roR = R[OMO_RO] * (aR - R[vn]) / (aR - aM);
            aVL = fabs(Uh[bn]) / sqrt(roL);
            aVR = fabs(Uh[bn]) / sqrt(roR);
            if (type == 3 && ((aL >= (aM - hllg_factor * aVL)) || ((aM + hllg_factor * aVR) >= aR))) {
              /* revert to HLLC-G, flux_solver.f90:447-476 */
              BRANCH(aM >= 0 ? 2 : 3);
              f2 = aL * aR;
              Fo[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2 * (R[bt1] - L[bt1]));
              Fo[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2 * (R[bt2] - L[bt2]));
              at1 = Uh[mt1] / Uh[OMO_RO];
              at2 = Uh[mt2] / Uh[OMO_RO];
              enL = ((aL - L[vn]) * UL[OMO_EN] - ptL * L[vn] + pt * aM +
                     Uh[bn] * (vBL - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) /
                    (aL - aM);
              enR = ((aR - R[vn]) * UR[OMO_EN] - ptR * R[vn] + pt * aM +
                     Uh[bn] * (vBR - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) /
                    (aR - aM);
              f1 = 0.5 + fsign(0.5, aM);
              f2 = 1.0 - f1;
              Fo[mn] = f1 * (aL * (roL * aM - UL[mn]) + FL[mn]) + f2 * (aR * (roR * aM - UR[mn]) + FR[mn]);
              Fo[mt1] = f1 * (aL * (roL * at1 - UL[mt1]) + FL[mt1]) + f2 * (aR * (roR * at1 - UR[mt1]) + FR[mt1]);
              Fo[mt2] = f1 * (aL * (roL * at2 - UL[mt2]) + FL[mt2]) + f2 * (aR * (roR * at2 - UR[mt2]) + FR[mt2]);
              Fo[OMO_EN] = f1 * (aL * (enL - UL[OMO_EN]) + FL[OMO_EN]) + f2 * (aR * (enR - UR[OMO_EN]) + FR[OMO_EN]);
              Fo[OMO_RO] = f1 * (aL * (roL - L[OMO_RO]) + FL[OMO_RO]) + f2 * (aR * (roR - R[OMO_RO]) + FR[OMO_RO]);
            } else {
              /* L* state, flux_solver.f90:482-493 */
              double tL = aL - L[vn];
              f1 = 1.0 / (L[OMO_RO] * tL * (aL - aM) - Uh[bn] * Uh[bn]);
              UL1[bt1] = L[bt1] * f1 * (L[OMO_RO] * (tL * tL) - Uh[bn] * Uh[bn]);
              UL1[bt2] = L[bt2] * f1 * (L[OMO_RO] * (tL * tL) - Uh[bn] * Uh[bn]);
              vt1L = L[vt1] - f1 * Uh[bn] * L[bt1] * (aM - L[vn]);
              vt2L = L[vt2] - f1 * Uh[bn] * L[bt2] * (aM - L[vn]);
              UL1[OMO_RO] = roL;
              UL1[OMO_EN] = ((aL - L[vn]) * UL[OMO_EN] - ptL * L[vn] + pt * aM +
                             Uh[bn] * (vBL - aM * Uh[bn] - vt1L * UL1[bt1] - vt2L * UL1[bt2])) /
                            (aL - aM);
              UL1[mn] = roL * aM;
              UL1[mt1] = roL * vt1L;
              UL1[mt2] = roL * vt2L;
              /* R* state, flux_solver.f90:496-507 */
              double tR = aR - R[vn];
              f1 = 1.0 / (R[OMO_RO] * tR * (aR - aM) - Uh[bn] * Uh[bn]);
              UR1[bt1] = R[bt1] * f1 * (R[OMO_RO] * (tR * tR) - Uh[bn] * Uh[bn]);
              UR1[bt2] = R[bt2] * f1 * (R[OMO_RO] * (tR * tR) - Uh[bn] * Uh[bn]);
              vt1R = R[vt1] - f1 * Uh[bn] * R[bt1] * (aM - R[vn]);
              vt2R = R[vt2] - f1 * Uh[bn] * R[bt2] * (aM - R[vn]);
              UR1[OMO_RO] = roR;
              UR1[OMO_EN] = ((aR - R[vn]) * UR[OMO_EN] - ptR * R[vn] + pt * aM +
                             Uh[bn] * (vBR - aM * Uh[bn] - vt1R * UR1[bt1] - vt2R * UR1[bt2])) /
                            (aR - aM);
              UR1[mn] = roR * aM;
              UR1[mt1] = roR * vt1R;
              UR1[mt2] = roR * vt2R;
              aL1 = aM - aVL;
              aR1 = aM + aVR;
              if (aL1 >= 0) { /* F(L*) :514-519 */
                BRANCH(4);
                for (int v = OMO_MX; v <= OMO_EN; ++v) Fo[v] = aL * (UL1[v] - UL[v]) + FL[v];
                Fo[OMO_RO] = aL * (UL1[OMO_RO] - L[OMO_RO]) + FL[OMO_RO];
                Fo[bt1] = aL * (UL1[bt1] - L[bt1]) + FL[bt1];
                Fo[bt2] = aL * (UL1[bt2] - L[bt2]) + FL[bt2];
              } else if (aR1 <= 0) { /* F(R*) :522-527 */
                BRANCH(5);
                for (int v = OMO_MX; v <= OMO_EN; ++v) Fo[v] = aR * (UR1[v] - UR[v]) + FR[v];
                Fo[OMO_RO] = aR * (UR1[OMO_RO] - R[OMO_RO]) + FR[OMO_RO];
                Fo[bt1] = aR * (UR1[bt1] - R[bt1]) + FR[bt1];
                Fo[bt2] = aR * (UR1[bt2] - R[bt2]) + FR[bt2];
              } else { /* central states :533-572 */
                roLs = sqrt(roL);
                roRs = sqrt(roR);
                f1 = 1.0 / (roLs + roRs);
                f2 = fsign(1.0, Uh[bn]);
                at1 = f1 * (roLs * vt1L + roRs * vt1R + (UR1[bt1] - UL1[bt1]) * f2);
                at2 = f1 * (roLs * vt2L + roRs * vt2R + (UR1[bt2] - UL1[bt2]) * f2);
                U2[bt1] = f1 * (roLs * UR1[bt1] + roRs * UL1[bt1] + roLs * roRs * (vt1R - vt1L) * f2);
                U2[bt2] = f1 * (roLs * UR1[bt2] + roRs * UL1[bt2] + roLs * roRs * (vt2R - vt2L) * f2);
                if (aM >= 0) { /* F(L**) */
                  BRANCH(6);
                  U2[OMO_RO] = roL;
                  U2[OMO_EN] = UL1[OMO_EN] - roLs * (vt1L * UL1[bt1] + vt2L * UL1[bt2] - at1 * U2[bt1] - at2 * U2[bt2]) * f2;
                  U2[mn] = roL * aM;
                  U2[mt1] = roL * at1;
                  U2[mt2] = roL * at2;
                  for (int v = OMO_MX; v <= OMO_EN; ++v)
                    Fo[v] = aL1 * U2[v] - (aL1 - aL) * UL1[v] - aL * UL[v] + FL[v];
                  Fo[OMO_RO] = aL1 * U2[OMO_RO] - (aL1 - aL) * UL1[OMO_RO] - aL * L[OMO_RO] + FL[OMO_RO];
                  Fo[bt1] = aL1 * U2[bt1] - (aL1 - aL) * UL1[bt1] - aL * L[bt1] + FL[bt1];
                  Fo[bt2] = aL1 * U2[bt2] - (aL1 - aL) * UL1[bt2] - aL * L[bt2] + FL[bt2];
                } else { /* F(R**) */
                  BRANCH(7);
                  U2[OMO_RO] = roR;
                  U2[OMO_EN] = UR1[OMO_EN] + roRs * (vt1R * UR1[bt1] + vt2R * UR1[bt2] - at1 * U2[bt1] - at2 * U2[bt2]) * f2;
                  U2[mn] = roR * aM;
                  U2[mt1] = roR * at1;
                  U2[mt2] = roR * at2;
                  for (int v = OMO_MX; v <= OMO_EN; ++v)
                    Fo[v] = aR1 * U2[v] - (aR1 - aR) * UR1[v] - aR * UR[v] + FR[v];
                  Fo[OMO_RO] = aR1 * U2[OMO_RO] - (aR1 - aR) * UR1[OMO_RO] - aR * R[OMO_RO] + FR[OMO_RO];
                  Fo[bt1] = aR1 * U2[bt1] - (aR1 - aR) * UR1[bt1] - aR * R[bt1] + FR[bt1];
                  Fo[bt2] = aR1 * U2[bt2] - (aR1 - aR) * UR1[bt2] - aR * R[bt2] + FR[bt2];
                }
              }
            }
            (void)enL; (void)enR;
          }
        }
        /* GLM fluxes, flux_solver.f90:580-581 (identical for every solver) */
        Fo[bn] = 0.5 * ((L[OMO_PS] + R[OMO_PS]) - ch * (R[bn] - L[bn]));
        Fo[OMO_PS] = 0.5 * (ch2 * (L[bn] + R[bn]) - ch * (R[OMO_PS] - L[OMO_PS]));
        for (int v = 0; v < NV; ++v) F[v * n + c] = Fo[v];
      }
}

/* ---------------------------------------------------------------------
 * rk: 2D_basic/rk.f90:9-131 ; 3D_basic/rk.f90:9-147.
 * The reference assumes dx == dy (== dz) (rk.f90:5).  With equal spacings
 * the reference expression is used verbatim; otherwise each direction gets
 * its own dt/d (declared extension).
 * ------------------------------------------------------------------- */
static inline int isotropic(double dx, double dy, double dz, int nd) {
  return dx == dy && (nd < 3 || dx == dz);
}

static inline double flux_div(const double* F, const double* G, const double* H, size_t q, size_t sx,
                              size_t sy, size_t sz, int nd, int iso, double dtx, double dty, double dtz) {
  if (iso) {
    if (nd == 3)
      return dtx * (F[q - sx] - F[q] + G[q - sy] - G[q] + H[q - sz] - H[q]);
    return dtx * (F[q - sx] - F[q] + G[q - sy] - G[q]);
  }
  if (nd == 3)
    return dtx * (F[q - sx] - F[q]) + dty * (G[q - sy] - G[q]) + dtz * (H[q - sz] - H[q]);
  return dtx * (F[q - sx] - F[q]) + dty * (G[q - sy] - G[q]);
}

static void rk_generic(int mode, double* U, double* U1, const double* F, const double* G,
                       const double* H, double dt, double dx, double dy, double dz, int ix, int jx,
                       int kx, int nd) {
  const size_t n = (size_t)ix * jx * kx;
  const int iso = isotropic(dx, dy, dz, nd);
  const double scale = (mode == 2) ? 0.5 * dt : dt; /* rk_std21: dtx = 0.5d0*dt/dx (rk.f90:76) */
  const double dtx = scale / dx, dty = scale / dy, dtz = scale / dz;
  const int k0 = (nd == 3) ? 1 : 0, k1 = (nd == 3) ? kx - 2 : 0;
  const size_t sx = 1, sy = ix, sz = (size_t)ix * jx;
#pragma omp parallel for collapse(2) schedule(static)
  for (int m = 0; m < NV; ++m)
    for (int k = k0; k <= k1; ++k)
      for (int j = 1; j <= jx - 2; ++j)
        for (int i = 1; i <= ix - 2; ++i) {
          const size_t q = m * n + IDX(i, j, k);
          const double d = flux_div(F, G, H, q, sx, sy, sz, nd, iso, dtx, dty, dtz);
          if (mode == 1) /* rk_tvd22 (rk.f90:56-66) */
            U[q] = 0.5 * (U[q] + U1[q] + d);
          else if (mode == 3) /* rk_std22 */
            U[q] = U[q] + d;
          else /* rk_tvd21, rk_std21 */
            U1[q] = U[q] + d;
        }
}

void omo_rk_tvd21(const double* U, double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd) {
  rk_generic(0, (double*)U, U1, F, G, H, dt, dx, dy, dz, ix, jx, kx, nd);
}
void omo_rk_tvd22(double* U, const double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd) {
  rk_generic(1, U, (double*)U1, F, G, H, dt, dx, dy, dz, ix, jx, kx, nd);
}
void omo_rk_std21(const double* U, double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd) {
  rk_generic(2, (double*)U, U1, F, G, H, dt, dx, dy, dz, ix, jx, kx, nd);
}
void omo_rk_std22(double* U, const double* F, const double* G, const double* H, double dt,
                  double dx, double dy, double dz, int ix, int jx, int kx, int nd) {
  rk_generic(3, U, NULL, F, G, H, dt, dx, dy, dz, ix, jx, kx, nd);
}

/* ---------------------------------------------------------------------
 * glm_ss2: 2D_basic/glm_ss2.f90:1-39 (whole array, ghosts included)
 * ------------------------------------------------------------------- */
void omo_glm_ss2(double* U, double ch, double dt, int ix, int jx, int kx) {
  const size_t n = (size_t)ix * jx * kx;
  const double cr = 0.2;
  const double f1 = exp(-(0.5 * dt * ch / cr));
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < (long long)n; ++c) U[OMO_PS * n + c] = f1 * U[OMO_PS * n + c];
}

/* ---------------------------------------------------------------------
 * set_dt: 2D_basic/set_dt.f90:1-68 ; 3D_basic/set_dt.f90:1-74.
 * Extension: dt = cfl*min(dx,dy[,dz])/vmax (== reference when isotropic).
 * ------------------------------------------------------------------- */
static inline double fast_speed(double f1, double B2, double bd, double ro) {
  const double f2 = 4 * f1 * (bd * bd);
  return sqrt(((f1 + B2) + sqrt(fmax2((f1 + B2) * (f1 + B2) - f2, 0.0))) / (2 * ro));
}

static inline double cell_speed(const double* U, const double* V, size_t n, size_t c, int nd, double gamma) {
  const double bx = U[OMO_BX * n + c], by = U[OMO_BY * n + c], bz = U[OMO_BZ * n + c];
  const double ro = U[OMO_RO * n + c];
  const double B2 = bx * bx + by * by + bz * bz;
  const double f1 = gamma * V[OMO_PR * n + c];
  const double vfx = fast_speed(f1, B2, bx, ro);
  const double vfy = fast_speed(f1, B2, by, ro);
  double s = fmax2(fabs(V[OMO_VX * n + c]) + vfx, fabs(V[OMO_VY * n + c]) + vfy);
  if (nd == 3) {
    const double vfz = fast_speed(f1, B2, bz, ro);
    s = fmax2(s, fabs(V[OMO_VZ * n + c]) + vfz);
  }
  return s;
}

int omo_set_dt(const double* U, const double* V, double* vmax_out, double* dt_out, double dx,
               double dy, double dz, double cfl, int ix, int jx, int kx, int nd, omo_err* err) {
  const size_t n = (size_t)ix * jx * kx;
  const int is = lo_of(ix), ie = hi_of(ix), js = lo_of(jx), je = hi_of(jx), ks = lo_of(kx),
            ke = hi_of(kx);
  const double gamma = g_gamma;
  double vmax = -1.0;
#pragma omp parallel for collapse(2) reduction(max : vmax) schedule(static)
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        const double s = cell_speed(U, V, n, IDX(i, j, k), nd, gamma);
        vmax = fmax2(s, vmax);
      }
  double dmin = dx;
  if (!isotropic(dx, dy, dz, nd)) {
    dmin = fmin2(dx, dy);
    if (nd == 3) dmin = fmin2(dmin, dz);
  }
  const double dt = cfl * dmin / vmax;
  *vmax_out = vmax;
  *dt_out = dt;
  if (dt < 1.0e-7) { /* set_dt.f90:55-65 */
    if (err) {
      /* maxloc over the interior (vtmp is undefined outside, set_dt.f90:52) */
      double best = -1.0;
      int bi = 0, bj = 0, bk = 0;
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie; ++i) {
            const double s = cell_speed(U, V, n, IDX(i, j, k), nd, gamma);
            if (s > best) { best = s; bi = i; bj = j; bk = k; }
          }
      err->code = OMO_DT_TOO_SMALL;
      err->i = bi; err->j = bj; err->k = bk;
      err->value = dt;
    }
    return OMO_DT_TOO_SMALL;
  }
  return OMO_OK;
}

/* 2D_reconnection/flux_resistive.f90:18-25 (Rm1 = 60); the Harris-xz kind
 * generalises it to dt <= 0.5*cfl*dx**2/eta_max. */
void omo_set_dt_resistive(double* dt, double dx, double cfl, int eta_kind) {
  if (eta_kind == OMO_ETA_RECON2D) {
    const double Rm1 = 60.0;
    *dt = fmin2(*dt, 0.5 * cfl * Rm1 * (dx * dx));
  } else if (eta_kind == OMO_ETA_HARRIS_XZ) {
    const double eta_max = 1.0e-3 + 1.0 / 60.0;
    *dt = fmin2(*dt, 0.5 * cfl / eta_max * (dx * dx));
  }
}

/* ---------------------------------------------------------------------
 * bc: 2D_basic/bc.f90:1-16 (periodic), 2D_KH/bc.f90:6-38 (walls),
 * 2D_reconnection/bc.f90:6-50, 3D_basic/bc.f90, 3D_reconnection_gpu/bc.cuf:7-98.
 * Order: x sides, then y, then z (as every reference bc routine).
 * ------------------------------------------------------------------- */
static void ghost_copy(double* U, int ix, int jx, int kx, int axis, int dst, int src, int flipmask) {
  const size_t n = (size_t)ix * jx * kx;
  const int ext[3] = {ix, jx, kx};
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  for (int v = 0; v < NV; ++v) {
    for (int q2 = 0; q2 < ext[a2]; ++q2)
      for (int q1 = 0; q1 < ext[a1]; ++q1) {
        const size_t b = (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
        const double s = U[v * n + b + (size_t)src * stride[axis]];
        U[v * n + b + (size_t)dst * stride[axis]] = ((flipmask >> v) & 1) ? -s : s;
      }
  }
}

void omo_bc(double* U, int ix, int jx, int kx, int nd, const omo_bcspec* bc) {
  const int ext[3] = {ix, jx, kx};
  for (int axis = 0; axis < nd; ++axis) {
    const int nx = ext[axis];
    const int lo = 2 * axis, hi = 2 * axis + 1;
    if (bc->kind[lo] == OMO_BC_PERIODIC) {
      ghost_copy(U, ix, jx, kx, axis, nx - 1, 1, 0); /* U(ix) = U(2) */
      ghost_copy(U, ix, jx, kx, axis, 0, nx - 2, 0); /* U(1) = U(ix-1) */
    } else {
      ghost_copy(U, ix, jx, kx, axis, 0, 1, bc->flip[lo]);
      ghost_copy(U, ix, jx, kx, axis, nx - 1, nx - 2, bc->flip[hi]);
    }
  }
}

/* face-state fix: main.f90:101-102,119-120 (periodic);
 * 2D_KH/bc.f90:42-83, 2D_reconnection/bc.f90:136-197 (mirror) */
void omo_facefix(double* VL, double* VR, int ix, int jx, int kx, int dir, const omo_bcspec* bc) {
  const size_t n = (size_t)ix * jx * kx;
  const int ext[3] = {ix, jx, kx};
  const int axis = dir - 1;
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  const int nx = ext[axis];
  const size_t f0 = 0, fl = (size_t)(nx - 2) * stride[axis];
  const int lo = 2 * axis, hi = 2 * axis + 1;
  for (int v = 0; v < NV; ++v)
    for (int q2 = 0; q2 < ext[a2]; ++q2)
      for (int q1 = 0; q1 < ext[a1]; ++q1) {
        const size_t b = v * n + (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
        if (bc->kind[lo] == OMO_BC_PERIODIC) {
          VR[b + fl] = VR[b + f0];
          VL[b + f0] = VL[b + fl];
        } else {
          const double s0 = VR[b + f0];
          VL[b + f0] = ((bc->flip[lo] >> v) & 1) ? -s0 : s0;
          const double s1 = VL[b + fl];
          VR[b + fl] = ((bc->flip[hi] >> v) & 1) ? -s1 : s1;
        }
      }
}

/* ---------------------------------------------------------------------
 * resistivity and resistive fluxes
 *   eta kind RECON2D: 2D_reconnection/flux_resistive.f90:1-16
 *   eta kind HARRIS_XZ: 1e-3 + (1/60) exp(-(x^2+z^2)/4)
 *   2D flux: 2D_reconnection/flux_resistive.f90:27-115
 *   3D flux: 3D_reconnection_gpu/flux_resistive.cuf:11-140
 * ------------------------------------------------------------------- */
double omo_eta(int eta_kind, double x, double y, double z) {
  if (eta_kind == OMO_ETA_RECON2D) {
    const double Rm1 = 60.0, Rm0 = 1000.0;
    const double eta0 = 1.0 / Rm0;
    const double eta01 = (Rm0 - Rm1) / (Rm0 * Rm1);
    const double c = cosh(fmin2(sqrt(x * x + y * y), 25.0));
    return eta0 + eta01 * (1.0 / (c * c));
  }
  if (eta_kind == OMO_ETA_HARRIS_XZ) {
    return 1.0e-3 + (1.0 / 60.0) * exp(-(x * x + z * z) / 4.0);
  }
  return 0.0;
}

void omo_flux_resistive(double* F, const double* U, const double* x, const double* y,
                        const double* z, double dx, int ix, int jx, int kx, int nd, int dir,
                        int eta_kind) {
  const size_t n = (size_t)ix * jx * kx;
  const double* Bx = U + OMO_BX * n;
  const double* By = U + OMO_BY * n;
  const double* Bz = U + OMO_BZ * n;
  double* Fen = F + OMO_EN * n;
  double* Fbx = F + OMO_BX * n;
  double* Fby = F + OMO_BY * n;
  double* Fbz = F + OMO_BZ * n;
  const size_t sx = 1, sy = ix, sz = (size_t)ix * jx;
  if (nd == 2) {
    const double odx = 1.0 / dx;
    const int is = (dir == 1) ? 0 : 1, ie = ix - 2, js = (dir == 2) ? 0 : 1, je = jx - 2;
#pragma omp parallel for schedule(static)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        const size_t c = IDX(i, j, 0);
        if (dir == 1) {
          const double eta_dx = omo_eta(eta_kind, x[i] + 0.5 * dx, y[j], 0.0) * odx;
          const double JyS = -eta_dx * (Bz[c + sx] - Bz[c]);
          const double JzS = eta_dx * ((By[c + sx] - By[c]) -
                                       0.25 * (Bx[c + sy] + Bx[c + sx + sy] - Bx[c - sy] - Bx[c + sx - sy]));
          Fen[c] = Fen[c] + 0.5 * (JyS * (Bz[c] + Bz[c + sx]) - JzS * (By[c] + By[c + sx]));
          Fby[c] = Fby[c] - JzS;
          Fbz[c] = Fbz[c] + JyS;
        } else {
          const double eta_dx = omo_eta(eta_kind, x[i], y[j] + 0.5 * dx, 0.0) * odx;
          const double JxS = eta_dx * (Bz[c + sy] - Bz[c]);
          const double JzS = eta_dx * (0.25 * (By[c + sx + sy] + By[c + sx] - By[c - sx + sy] - By[c - sx]) -
                                       (Bx[c + sy] - Bx[c]));
          Fen[c] = Fen[c] + 0.5 * (JzS * (Bx[c] + Bx[c + sy]) - JxS * (Bz[c] + Bz[c + sy]));
          Fbx[c] = Fbx[c] + JzS;
          Fbz[c] = Fbz[c] - JxS;
        }
      }
    return;
  }
  /* 3D */
  int is = 1, ie = ix - 2, js = 1, je = jx - 2, ks = 1, ke = kx - 2;
  if (dir == 1) is = 0;
  if (dir == 2) js = 0;
  if (dir == 3) ks = 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        const size_t c = IDX(i, j, k);
        double xx = x[i], yy = y[j], zz = z[k];
        if (dir == 1) xx = x[i] + 0.5 * dx;
        if (dir == 2) yy = y[j] + 0.5 * dx;
        if (dir == 3) zz = z[k] + 0.5 * dx;
        const double eta_dx = omo_eta(eta_kind, xx, yy, zz) / dx;
        if (dir == 1) {
          const double JyS = -(Bz[c + sx] - Bz[c]) +
                             0.25 * (Bx[c + sz] + Bx[c + sx + sz] - Bx[c - sz] - Bx[c + sx - sz]);
          const double JzS = (By[c + sx] - By[c]) -
                             0.25 * (Bx[c + sy] + Bx[c + sx + sy] - Bx[c - sy] - Bx[c + sx - sy]);
          Fen[c] = Fen[c] + 0.5 * eta_dx * (JyS * (Bz[c] + Bz[c + sx]) - JzS * (By[c] + By[c + sx]));
          Fby[c] = Fby[c] - eta_dx * JzS;
          Fbz[c] = Fbz[c] + eta_dx * JyS;
        } else if (dir == 2) {
          const double JxS = (Bz[c + sy] - Bz[c]) -
                             0.25 * (By[c + sz] + By[c + sy + sz] - By[c - sz] - By[c + sy - sz]);
          const double JzS = -(Bx[c + sy] - Bx[c]) +
                             0.25 * (By[c + sx] + By[c + sx + sy] - By[c - sx] - By[c - sx + sy]);
          Fen[c] = Fen[c] + 0.5 * eta_dx * (JzS * (Bx[c] + Bx[c + sy]) - JxS * (Bz[c] + Bz[c + sy]));
          Fbx[c] = Fbx[c] + eta_dx * JzS;
          Fbz[c] = Fbz[c] - eta_dx * JxS;
        } else {
          const double JyS = (Bx[c + sz] - Bx[c]) -
                             0.25 * (Bz[c + sx] + Bz[c + sx + sz] - Bz[c - sx] - Bz[c - sx + sz]);
          const double JxS = -(By[c + sz] - By[c]) +
                             0.25 * (Bz[c + sy] + Bz[c + sy + sz] - Bz[c - sy] - Bz[c - sy + sz]);
          Fen[c] = Fen[c] + 0.5 * eta_dx * (JxS * (By[c] + By[c + sz]) - JyS * (Bx[c] + Bx[c + sz]));
          Fbx[c] = Fbx[c] - eta_dx * JyS;
          Fby[c] = Fby[c] + eta_dx * JxS;
        }
      }
}

/* ---------------------------------------------------------------------
 * One step of the driver loop body: 2D_basic/main.f90:61-187 (u2v, set_dt,
 * glm, limiter x9 per direction, face fix, flux, [resistive], rk21, bc,
 * u2v, ..., rk22, bc, glm, t += dt).  The 3D driver is the same with a third
 * direction (3D_basic/main.f90, 3D_reconnection_gpu/main.cuf:115-299).
 * ------------------------------------------------------------------- */
size_t omo_workspace_doubles(const omo_cfg* cfg) {
  const size_t n = (size_t)cfg->ix * cfg->jx * cfg->kx;
  return (size_t)NV * n * 6 + 4 * n;
}

static void limit_all(const omo_cfg* c, const double* U, const double* V, double* VL, double* VR, int dir) {
  const size_t n = (size_t)c->ix * c->jx * c->kx;
  /* main.f90:91-99: vx,vy,vz,p from V ; ro,bx,by,bz,ps from U */
  for (int v = 0; v < 4; ++v)
    omo_limiter(V + v * n, VL + v * n, VR + v * n, c->ix, c->jx, c->kx, dir, c->lm_type);
  const int us[5] = {OMO_RO, OMO_BX, OMO_BY, OMO_BZ, OMO_PS};
  for (int q = 0; q < 5; ++q)
    omo_limiter(U + us[q] * n, VL + us[q] * n, VR + us[q] * n, c->ix, c->jx, c->kx, dir, c->lm_type);
}

/* The flop-counting build (oracle/flopcount.cpp) defines these to tally the
 * face reconstruction and flux work of a step, and its conserved-to-primitive
 * recoveries, apart from the rest. */
#ifndef OMO_FLUX_REGION
#define OMO_FLUX_REGION(on)
#endif
#ifndef OMO_U2V_REGION
#define OMO_U2V_REGION(on)
#endif

static int half_fluxes(const omo_cfg* c, const double* Ucur, double* V, double* VL, double* VR,
                       double* Fd[3], double ch, const double* x, const double* y, const double* z) {
  OMO_FLUX_REGION(1);
  for (int dir = 1; dir <= c->nd; ++dir) {
    limit_all(c, Ucur, V, VL, VR, dir);
    omo_facefix(VL, VR, c->ix, c->jx, c->kx, dir, &c->bc);
    omo_flux_solver(Fd[dir - 1], VL, VR, ch, c->ix, c->jx, c->kx, dir, c->flux_type);
    if (c->eta_kind != OMO_ETA_NONE)
      omo_flux_resistive(Fd[dir - 1], Ucur, x, y, z, c->dx, c->ix, c->jx, c->kx, c->nd, dir, c->eta_kind);
  }
  OMO_FLUX_REGION(0);
  return OMO_OK;
}

int omo_step(const omo_cfg* c, double* U, double* ws, const double* x, const double* y,
             const double* z, double* t, double* dt_out, double* ch_out, omo_err* err) {
  const size_t n = (size_t)c->ix * c->jx * c->kx;
  double* U1 = ws;
  double* VL = U1 + NV * n;
  double* VR = VL + NV * n;
  double* F = VR + NV * n;
  double* G = F + NV * n;
  double* H = G + NV * n;
  double* V = H + NV * n;
  double* Fd[3] = {F, G, H};
  double ch, dt;
  int st;
  omo_set_gamma(c->gamma);
  if (err) err->code = OMO_OK;

  OMO_U2V_REGION(1);
  st = omo_u2v(U, V, c->ix, c->jx, c->kx, err);
  OMO_U2V_REGION(0);
  if (st) return st;
  st = omo_set_dt(U, V, &ch, &dt, c->dx, c->dy, c->dz, c->cfl, c->ix, c->jx, c->kx, c->nd, err);
  if (c->eta_kind != OMO_ETA_NONE) omo_set_dt_resistive(&dt, c->dx, c->cfl, c->eta_kind);
  if (st) return st;
  omo_glm_ss2(U, ch, dt, c->ix, c->jx, c->kx);

  half_fluxes(c, U, V, VL, VR, Fd, ch, x, y, z);
  if (c->time_type == 0)
    omo_rk_tvd21(U, U1, F, G, H, dt, c->dx, c->dy, c->dz, c->ix, c->jx, c->kx, c->nd);
  else
    omo_rk_std21(U, U1, F, G, H, dt, c->dx, c->dy, c->dz, c->ix, c->jx, c->kx, c->nd);
  omo_bc(U1, c->ix, c->jx, c->kx, c->nd, &c->bc);
  OMO_U2V_REGION(1);
  st = omo_u2v(U1, V, c->ix, c->jx, c->kx, err);
  OMO_U2V_REGION(0);
  if (st) return st;

  half_fluxes(c, U1, V, VL, VR, Fd, ch, x, y, z);
  if (c->time_type == 0)
    omo_rk_tvd22(U, U1, F, G, H, dt, c->dx, c->dy, c->dz, c->ix, c->jx, c->kx, c->nd);
  else
    omo_rk_std22(U, F, G, H, dt, c->dx, c->dy, c->dz, c->ix, c->jx, c->kx, c->nd);
  omo_bc(U, c->ix, c->jx, c->kx, c->nd, &c->bc);
  omo_glm_ss2(U, ch, dt, c->ix, c->jx, c->kx);
  *t += dt;
  if (dt_out) *dt_out = dt;
  if (ch_out) *ch_out = ch;
  return OMO_OK;
}

/* ---------------------------------------------------------------------
 * seeded deviates and models
 * ------------------------------------------------------------------- */
static inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double omo_uniform_pm1(uint64_t seed, uint64_t n) {
  const uint64_t h = splitmix64(splitmix64(seed) ^ n);
  return (double)(h >> 11) * 0x1.0p-52 - 1.0;
}

/* grid recurrence of 2D_basic/model.f90:19-28: x(1) = x0 - d/2, x(i) = x(i-1) + d */
void omo_grid(double* x, int n, double x0, double d) {
  x[0] = x0 - d / 2;
  for (int i = 1; i < n; ++i) x[i] = x[i - 1] + d;
}

/* Harris-sheet vector potential A_y(x,y,z) built from a few seeded modes. */
static double harris_ay(const omo_model* m, double x, double y, double z, double Lx, double Ly) {
  const double two_pi = 8.0 * atan(1.0);
  double s = 0.0;
  for (int a = 1; a <= 4; ++a)
    for (int b = 0; b <= 1; ++b) {
      const uint64_t key = (uint64_t)(a * 8 + b);
      const double c = omo_uniform_pm1(m->seed, 2 * key);
      const double ph = (omo_uniform_pm1(m->seed, 2 * key + 1) + 1.0) * (two_pi / 2.0);
      s = s + c * cos(two_pi * a * x / Lx + two_pi * b * y / Ly + ph);
    }
  return m->amp * exp(-(z * z) / 4.0) * s;
}

/* vector-potential profile of the 3D field loop, 3D_basic/model.f90:1-6 (mya3) */
static double loop_a3(double xx, double yy, double zz) {
  const double myr = 0.3;
  const double a = 2 * xx + zz;
  const double m2 = fmin2(fmin2((a - 2) * (a - 2), a * a), (a + 2) * (a + 2));
  return fmax2(0.0, myr - sqrt(yy * yy + m2 / 5.0));
}

void omo_model_fill(const omo_model* m, double* U, const double* x, const double* y,
                    const double* z, int ix, int jx, int kx, double dx, double dy, double dz) {
  const size_t n = (size_t)ix * jx * kx;
  const double gamma = g_gamma;
  const double f1 = 1.0 / (gamma - 1);
  for (int k = 0; k < kx; ++k)
    for (int j = 0; j < jx; ++j)
      for (int i = 0; i < ix; ++i) {
        const size_t c = IDX(i, j, k);
        double ro, pr, vx, vy, vz, bx, by, bz;
        if (m->kind == 0) {
          /* Orszag-Tang, 2D_basic/model.f90:34-50 (amp, phases = 1, 0, 0 there) */
          ro = gamma * gamma;
          pr = gamma;
          vx = -sin(y[j] + m->phase_y);
          vy = sin(x[i] + m->phase_x);
          vz = 0.0;
          bx = m->amp * -sin(y[j] + m->phase_y);
          by = m->amp * sin(2 * (x[i] + m->phase_x));
          bz = 0.0;
        } else if (m->kind == 1) {
          /* KH shear layer: rho=1, p=0.5, vx=amp*tanh(y), Bx=bx0,
           * vy = pert*exp(-y^2)*r(x,y) with r seeded in [-1,1) */
          ro = 1.0;
          pr = 0.5;
          vx = m->amp * tanh(y[j]);
          vy = m->pert * exp(-(y[j] * y[j])) * omo_uniform_pm1(m->seed, (uint64_t)c);
          vz = 0.0;
          bx = m->bx0;
          by = 0.0;
          bz = 0.0;
        } else if (m->kind == 2) {
          /* Harris sheet in z: Bx=tanh(z), rho=1+cosh(z)^-2/beta, p=0.5*beta*rho, v=0,
           * plus curl(A_y yhat) by centred half-cell differences (3D_basic/model.f90:61-63) */
          const double Lx = dx * (ix - 2), Ly = dy * (jx - 2);
          const double ch = cosh(z[k]);
          ro = 1.0 + (1.0 / (ch * ch)) / m->beta;
          pr = 0.5 * m->beta * ro;
          vx = 0.0; vy = 0.0; vz = 0.0;
          const double dAz = (harris_ay(m, x[i], y[j], z[k] + dz / 2, Lx, Ly) -
                              harris_ay(m, x[i], y[j], z[k] - dz / 2, Lx, Ly)) / dz;
          const double dAx = (harris_ay(m, x[i] + dx / 2, y[j], z[k], Lx, Ly) -
                              harris_ay(m, x[i] - dx / 2, y[j], z[k], Lx, Ly)) / dx;
          bx = tanh(z[k]) - dAz;
          by = 0.0;
          bz = dAx;
        } else if (m->kind == 3) {
          /* 2D reconnection, 2D_reconnection/model.f90:37-58 (b1 = amp) */
          const double chy = cosh(fmin2(y[j], 25.0));
          ro = 1.0 + (1.0 / (chy * chy)) / m->beta;
          pr = 0.5 * m->beta * ro;
          vx = 0.0; vy = 0.0; vz = 0.0;
          const double r2 = x[i] * x[i] + y[j] * y[j];
          bx = tanh(y[j]) - m->amp * y[j] * exp(-r2 / 4.0);
          by = 0.0 + m->amp * x[i] * exp(-r2 / 4.0);
          bz = 0.0;
        } else if (m->kind == 4) {
          /* Brio-Wu shock tube, 1D_basic/model.f90:43-68 (the active states) */
          const int left = x[i] < 0.0;
          ro = left ? 1.0 : 0.125;
          pr = left ? 1.0 : 0.1;
          vx = 0.0; vy = 0.0; vz = 0.0;
          bx = 0.75;
          by = left ? 1.0 : -1.0;
          bz = 0.0;
        } else {
          /* 3D field loop, 3D_basic/model.f90:37-66 (A amplitude = amp) */
          ro = 1.0;
          pr = 1.0;
          vx = 1.0; vy = 1.0; vz = 2.0;
          const double fx = -(m->amp / dx) * (1.0 / sqrt(5.0));
          const double fz = +(m->amp / dx) * (2.0 / sqrt(5.0));
          const double h = dx / 2;
          const double xx = x[i], yy = y[j], zz = z[k];
          bx = fz * (loop_a3(xx, yy + h, zz) - loop_a3(xx, yy - h, zz));
          by = fx * (loop_a3(xx, yy, zz + h) - loop_a3(xx, yy, zz - h)) - fz * (loop_a3(xx + h, yy, zz) - loop_a3(xx - h, yy, zz));
          bz = -fx * (loop_a3(xx, yy + h, zz) - loop_a3(xx, yy - h, zz));
        }
        const double v2 = vx * vx + vy * vy + vz * vz;
        const double B2 = bx * bx + by * by + bz * bz;
        U[OMO_RO * n + c] = ro;
        U[OMO_MX * n + c] = ro * vx;
        U[OMO_MY * n + c] = ro * vy;
        U[OMO_MZ * n + c] = ro * vz;
        U[OMO_EN * n + c] = 0.5 * (ro * v2 + B2) + f1 * pr;
        U[OMO_BX * n + c] = bx;
        U[OMO_BY * n + c] = by;
        U[OMO_BZ * n + c] = bz;
        U[OMO_PS * n + c] = 0.0;
      }
}
