// omhd_fused2d.cuh -- one fused kernel per TVD-RK2 stage for 2D grids.
//
// A CTA owns a TX x TY tile of interior cells and stages the tile plus a
// two-cell halo of the state in shared memory.  Inside the CTA:
//   A  load + conserved->primitive recovery (u2v.f90) of the halo tile,
//      stage 1 applies the first GLM half (glm_ss2.f90) on the fly;
//   B  slope limiting (limiter.f90) in x and y -> face states of both
//      directions in one phase, then the wall face fixes (bc_for_F/G);
//   C  Riemann fluxes (flux_solver.f90) [+ resistive terms] of all x faces
//      and all y faces of the tile in one phase, warp-aligned so that no warp
//      mixes directions;
//   D  Runge-Kutta update (rk.f90) from the flux differences (FP64),
//      ghost-cell fill by the owner of each source cell (bc.f90); stage 2
//      applies the second GLM half and reduces the next step's CFL speed
//      (set_dt.f90); the last CTA plans the next step on the device.
// Per stage this reads the state once (plus halo) and writes it once: the
// face states and fluxes of the reference (VL, VR, F, G) never reach HBM.
// Three CTA-wide barriers per stage; the FP64 pipe is the bottleneck on
// GB300, so phases are arranged to keep every warp issuing FP64 work.
//
// Included by one translation unit per arithmetic variant; OMHD_VARIANT names
// the namespace so that instantiations built with different floating-point
// flags never collide at link time.
#pragma once
#include <cstring>

#include "omhd_fused.h"
#include "omhd_step.cuh"
#include "omhd_tma.h"

#ifndef OMHD_VARIANT
#error "define OMHD_VARIANT before including omhd_fused2d.cuh"
#endif

namespace omhd {
namespace OMHD_VARIANT {

constexpr int round32(int n) { return (n + 31) / 32 * 32; }
constexpr int imax(int a, int b) { return a > b ? a : b; }

// tile geometry: TX x TY interior cells
template <int TX_, int TY_>
struct Geo2 {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int RX = TX + 4, RY = TY + 4;  // halo tile
  static constexpr int NXS = TY * (TX + 2);       // cells reconstructed in x
  static constexpr int NYS = (TY + 2) * TX;       // cells reconstructed in y
  static constexpr int NXF = TY * (TX + 1);       // x faces
  static constexpr int NYF = (TY + 1) * TX;       // y faces
  static constexpr int NXFP = round32(NXF);       // x faces padded to whole warps
  // one thread per y face (or padded x face), at least one per cell
  static constexpr int NT = imax(imax(NXFP, round32(NYF)), round32(TX * TY));
  // face states in T, face fluxes in FP64 (the flux differences are FP64,
  // so each flux is widened once, when it is stored)
  template <class T>
  static constexpr size_t smem_bytes() {
    return sizeof(T) * (size_t)NV * (RY * RX + 2 * (NXS + NYS)) + sizeof(double) * (size_t)NV * (NXF + NYF);
  }
  static_assert((NV * (RY * RX + 2 * (NXS + NYS))) % 2 == 0, "flux block must start 8-byte aligned");
};
// tile of the single-grid stage kernel per arithmetic type.  FP64: 16x16, whose
// halo is the smallest of the shapes a 288-thread CTA serves (1.5 loaded cells
// per cell).  FP32-mixed: 16x8 tiles of 160 threads, four CTAs per SM (96
// registers): more CTAs interleave their barrier-separated phases; measured on
// KH 4096x2048, 16x8 at 4 / 3 CTAs per SM and 16x16 / 32x8 / 64x4 at 2 CTAs per
// SM gave 1.985e9 / 1.819e9 and 1.894e9 / 1.868e9 / 1.824e9 cell-updates/s
// (build-time constants, for tuning)
#ifndef OMHD_MIXED_TILE_X
#define OMHD_MIXED_TILE_X 16
#endif
#ifndef OMHD_MIXED_TILE_Y
#define OMHD_MIXED_TILE_Y 8
#endif
#ifndef OMHD_MIXED_MIN_CTAS  // resident CTAs per SM the FP32-mixed stage kernel is built for
#define OMHD_MIXED_MIN_CTAS 4
#endif
template <class T>
struct GeoFor {
  using type = Geo2<16, 16>;
};
template <>
struct GeoFor<float> {
  using type = Geo2<OMHD_MIXED_TILE_X, OMHD_MIXED_TILE_Y>;
};

__device__ __forceinline__ int map_index(int g, int n, bool periodic) {
  if (g >= 0 && g < n) return g;
  if (periodic) {
    const int P = n - 2;
    int r = (g - 1) % P;
    if (r < 0) r += P;
    return r + 1;
  }
  return g < 0 ? 0 : n - 1;
}

__device__ __forceinline__ double eta_at(int kind, double x, double y, double z) {
  if (kind == OMHD_ETA_RECON2D) {  // 2D_reconnection/flux_resistive.f90:1-16
    const double Rm1 = 60.0, Rm0 = 1000.0;
    const double eta0 = 1.0 / Rm0;
    const double eta01 = (Rm0 - Rm1) / (Rm0 * Rm1);
    const double c = cosh(fmin2(sqrt(x * x + y * y), 25.0));
    return eta0 + eta01 * (1.0 / (c * c));
  }
  if (kind == OMHD_ETA_HARRIS_XZ) return 1.0e-3 + (1.0 / 60.0) * exp(-(x * x + z * z) / 4.0);
  return 0.0;
}

// canonical interior cell of a (possibly ghost or out-of-grid) index along an
// axis of extent n, for decision-tape lookups: periodic ghosts wrap, other
// indices clamp (their states are unused)
__device__ __forceinline__ int tape_cell(int g, int n, bool periodic) {
  if (periodic) {
    const int P = n - 2;
    int r = (g - 1) % P;
    if (r < 0) r += P;
    return r + 1;
  }
  return g < 1 ? 1 : (g > n - 2 ? n - 2 : g);
}

// Shared-memory views of one tile: the primitive halo tile W, the face states
// of both directions, and where the face fluxes go.  Fluxes either have their
// own FP64 block (FX[v*fxv + cy*(TX+1) + fx], FY[v*fyv + fy*TX + cx]) or, in
// the FP64 pipelined kernel, overwrite the lower-cell face state that only
// their own face reads (FX = SLx with fxv = NXS and row stride TX+2).
template <class T>
struct TileMem {
  T* W;
  T *SLx, *SRx, *SLy, *SRy;
  double *FX, *FY;
  int fxv, fxr, fyv;
};

// Scalars of one stage: one thread gathers them per CTA -- per work item in an
// ensemble -- into shared memory, and the others read them after the next CTA
// barrier.  The constant ones come derived from the host (stage_args_derived);
// dt/dx is dt * (dtx_scale/dx) in the FAST builds (the FP64 divisions one
// thread made here, before the barrier the CTA's other threads wait at, cost
// 11 % of the FP32-mixed kernel's time at 128 cells per CTA; the product is
// within an ulp of the quotient) and the reference's dtx_scale * dt / dx in the
// parity build.
template <class T>
struct StageScalars {
  double glmf;        // GLM damping factor of the step (glm_ss2.f90:27)
  double dtx, dty;    // dtx_scale * dt / dx and / dy (rk.f90:22)
  T ch, gam, r1, r2;  // GLM speed, gamma, 1/(gamma-1), gamma/(gamma-1) (flux_solver.f90:38-39)
};
template <class T>
__device__ __forceinline__ void stage_scalars(const StageArgs& a, const StepState* st, StageScalars<T>& k) {
  const double dt = st->dt;
  k.glmf = st->glm_f;
  if constexpr (OMHD_FAST) {
    k.dtx = dt * a.sdx;
    k.dty = dt * a.sdy;
  } else {
    k.dtx = a.dtx_scale * dt / a.dx;
    k.dty = a.dtx_scale * dt / a.dy;
  }
  k.ch = to_face<T>(st->ch);
  if constexpr (sizeof(T) == 4) {
    k.gam = a.gamma_f;
    k.r1 = a.r1_f;
    k.r2 = a.r2_f;
  } else {
    k.gam = a.gamma;
    k.r1 = a.r1;
    k.r2 = a.r2;
  }
}

template <class T, class G>
__device__ __forceinline__ TileMem<T> tile_mem_separate(unsigned char* smem_raw) {
  TileMem<T> m;
  m.W = reinterpret_cast<T*>(smem_raw);
  m.SLx = m.W + NV * G::RX * G::RY;
  m.SRx = m.SLx + NV * G::NXS;
  m.SLy = m.SRx + NV * G::NXS;
  m.SRy = m.SLy + NV * G::NYS;
  m.FX = reinterpret_cast<double*>(m.SRy + NV * G::NYS);
  m.FY = m.FX + NV * G::NXF;
  m.fxv = G::NXF;
  m.fxr = G::TX + 1;
  m.fyv = G::NYF;
  return m;
}

// phase A: halo tile load + u2v (+ first GLM half in stage 1); threads t of n.
// STAGED: the conserved halo tile is already in shared memory (S, laid out as
// the TMA box: nine planes of RY rows of RX + 2 cells starting one cell left of
// the halo, so that the box starts on an even x), instead of in global memory.
template <class T, class G, bool STAGED = false>
__device__ __forceinline__ void phase_load(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t, int n,
                                           double glmf, const double* S = nullptr) {
  constexpr int TX = G::TX, TY = G::TY, RX = G::RX, RY = G::RY, PL = RX * RY;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * TY;
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const double f1g = a.gm1;  // u2v.f90:11, derived on the host
  const float f1g32 = a.gm1_f;
  T* W = m.W;
  // FP64: two cells per pass, both cells' loads issued before either is
  // converted, so their global-memory latencies overlap; FP32-mixed (two CTAs
  // per SM, 112 registers) one cell per pass
  constexpr int B = sizeof(T) == 8 ? 2 : 1;
  for (int q0 = t; q0 < PL; q0 += B * n) {
    double u[B][NV];
    bool act[B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int q = q0 + b * n;
      const int rx = q % RX, ry = q / RX;
      const bool cx_in = rx >= 2 && rx < TX + 2, cy_in = ry >= 2 && ry < TY + 2;
      // corners: only the diagonal neighbours are needed, by the resistive terms
      act[b] = q < PL && (cx_in || cy_in || (resist && rx != 0 && rx != RX - 1 && ry != 0 && ry != RY - 1));
      if (act[b]) {
        if constexpr (STAGED) {
          constexpr int SW = RX + 2;
#pragma unroll
          for (int v = 0; v < NV; ++v) u[b][v] = S[v * (SW * RY) + ry * SW + rx + 1];
        } else {
          const size_t c =
              (size_t)map_index(gi0 - 2 + rx, ix, perx) + (size_t)ix * map_index(gj0 - 2 + ry, jx, pery);
#pragma unroll
          for (int v = 0; v < NV; ++v) u[b][v] = __ldg(a.Uin + v * N + c);
        }
      }
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      if (!act[b]) continue;
      const int q = q0 + b * n;
      const int rx = q % RX, ry = q / RX;
      const bool cx_in = rx >= 2 && rx < TX + 2, cy_in = ry >= 2 && ry < TY + 2;
      const int gi = gi0 - 2 + rx, gj = gj0 - 2 + ry;
      double ps = u[b][PS];
      if (a.stage == 1) ps = glmf * ps;
      T w[NV];
      double pr, ro;
      u2v_cell<T, OMHD_FAST>(u[b], f1g, f1g32, ps, w, pr, ro);
#pragma unroll
      for (int v = 0; v < NV; ++v) W[v * PL + q] = w[v];
      if (cx_in && cy_in && gi <= ix - 2 && gj <= jx - 2) {  // owner check, u2v.f90:36-45
        if (!gt0_<OMHD_FAST>(pr))
          raise_error(a.err, OMHD_NEG_PRESSURE, gi + 1, gj + 1, 0, 0, pr);
        else if (!gt0_<OMHD_FAST>(ro))
          raise_error(a.err, OMHD_NEG_DENSITY, gi + 1, gj + 1, 0, 0, ro);
      }
    }
  }
}

// phase B: slopes in x (cells rx = 1..TX+2 on tile rows) and y (rows
// ry = 1..TY+2 on tile columns) -> face states of both directions
template <class T, class G, int TAPE>
__device__ __forceinline__ void phase_recon(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t, int n) {
  constexpr int TX = G::TX, TY = G::TY, RX = G::RX, RY = G::RY, PL = RX * RY;
  constexpr int NXS = G::NXS, NYS = G::NYS, XS = TX + 2;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * TY;
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const int lm = a.lm_type;
  const T* W = m.W;
  if constexpr (OMHD_FAST && sizeof(T) == 8 && TAPE != tape::kReplay) {
    if (lm == LM_MINMOD || lm == LM_MC) {
      // two neighbouring cells per item: wm, w0, w1, w2 give the three slopes
      // of both cells (their shared difference once), 4 loads instead of 6;
      // x pairs (cx, cx+1) of a row, y pairs (cy, cy+1) of a column
      constexpr int XP = XS / 2, NXP = NXS / 2, NYP = NYS / 2;
      static_assert(XS % 2 == 0 && (TY + 2) % 2 == 0, "cell pairs need even strip lengths");
      for (int p = t; p < NXP + NYP; p += n) {
        const bool xd = p < NXP;
        const int pp = xd ? p : p - NXP;
        // first cell of the pair: x (cx0, cy) / y (cx, cy0)
        const int ca = xd ? 2 * (pp % XP) : pp % TX, cb = xd ? pp / XP : 2 * (pp / TX);
        const int o = xd ? (cb + 2) * RX + (ca + 1) : (cb + 1) * RX + (ca + 2);
        const int st = xd ? 1 : RX;
        const int i0 = xd ? cb * XS + ca : cb * TX + ca, di = xd ? 1 : TX;
        double* dl = xd ? m.SLx : m.SLy;
        double* dr = xd ? m.SRx : m.SRy;
        const int sv = xd ? NXS : NYS;
        size_t tc0 = 0, tc1 = 0;
        bool own0 = false, own1 = false;
        unsigned char* tl = nullptr;
        if (TAPE == tape::kRecord && a.tlim) {
          // global cells of the pair; the tile owns cx/cy = 1..TX/TY
          const int gi = xd ? gi0 - 1 + ca : gi0 + ca, gj = xd ? gj0 + cb : gj0 - 1 + cb;
          const int gi1 = xd ? gi + 1 : gi, gj1 = xd ? gj : gj + 1;
          const int c0 = xd ? ca : cb, lim = xd ? TX : TY;
          own0 = c0 >= 1 && c0 <= lim && gi <= ix - 2 && gj <= jx - 2;
          own1 = c0 + 1 >= 1 && c0 + 1 <= lim && gi1 <= ix - 2 && gj1 <= jx - 2;
          tc0 = (size_t)tape_cell(gi, ix, perx) + (size_t)ix * tape_cell(gj, jx, pery);
          tc1 = (size_t)tape_cell(gi1, ix, perx) + (size_t)ix * tape_cell(gj1, jx, pery);
          tl = a.tlim + (size_t)(xd ? 0 : 1) * NV * N;
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double* w = W + v * PL + o;
          const double wm = w[-st], w0 = w[0], w1 = w[st], w2 = w[2 * st];
          const double d0 = w0 - wm, d1 = w1 - w0, d2 = w2 - w1;
          double l0, r0, l1, r1;
          unsigned char k0 = 0, k1 = 0;
          reconstruct_fp64_g<TAPE>(lm, d0, d1, wm, w0, w1, l0, r0, &k0);
          reconstruct_fp64_g<TAPE>(lm, d1, d2, w0, w1, w2, l1, r1, &k1);
          if (TAPE == tape::kRecord && tl) {
            if (own0) tl[v * N + tc0] = k0;
            if (own1) tl[v * N + tc1] = k1;
          }
          dl[v * sv + i0] = l0;
          dr[v * sv + i0] = r0;
          dl[v * sv + i0 + di] = l1;
          dr[v * sv + i0 + di] = r1;
        }
      }
      return;
    }
  }
  for (int q = t; q < NXS + NYS; q += n) {
    int o, st;
    T *dl, *dr;
    int qq;
    if (q < NXS) {
      const int cx = q % XS, cy = q / XS;
      o = (cy + 2) * RX + (cx + 1);
      st = 1;
      dl = m.SLx;
      dr = m.SRx;
      qq = q;
    } else {
      qq = q - NXS;
      const int cx = qq % TX, cy = qq / TX;
      o = (cy + 1) * RX + (cx + 2);
      st = RX;
      dl = m.SLy;
      dr = m.SRy;
    }
    if constexpr (TAPE == tape::kNone) {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        T l, r;
        reconstruct_t<T, OMHD_FAST>(lm, W[v * PL + o - st], W[v * PL + o], W[v * PL + o + st], l, r);
        dl[v * (q < NXS ? NXS : NYS) + qq] = l;
        dr[v * (q < NXS ? NXS : NYS) + qq] = r;
      }
    } else {
      // this cell's global index; x cells cx = 0..TX+1 of row cy, y cells
      // cy = 0..TY+1 of column cx (the tile owns cx/cy = 1..TX/TY)
      const bool xd = q < NXS;
      const int cx = xd ? q % XS : qq % TX, cy = xd ? q / XS : qq / TX;
      const int gi = xd ? gi0 - 1 + cx : gi0 + cx, gj = xd ? gj0 + cy : gj0 - 1 + cy;
      const bool own = (xd ? (cx >= 1 && cx <= TX) : (cy >= 1 && cy <= TY)) && gi <= ix - 2 && gj <= jx - 2;
      const size_t tc = (TAPE == tape::kReplay || a.tlim)
                            ? (size_t)tape_cell(gi, ix, perx) + (size_t)ix * tape_cell(gj, jx, pery)
                            : 0;
      unsigned char* tl = a.tlim ? a.tlim + (size_t)(xd ? 0 : 1) * NV * N : nullptr;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double l, r;
        unsigned char k = (TAPE == tape::kReplay) ? tl[v * N + tc] : 0;
        reconstruct_fp64<OMHD_FAST, TAPE>(lm, W[v * PL + o - st], W[v * PL + o], W[v * PL + o + st], l, r, &k);
        if (TAPE == tape::kRecord && own && tl) tl[v * N + tc] = k;
        dl[v * (xd ? NXS : NYS) + qq] = l;
        dr[v * (xd ? NXS : NYS) + qq] = r;
      }
    }
  }
}

// whether phase_walls changes a face state of this tile (a tile at a
// non-periodic edge); uniform over the CTA, so the barrier that follows the
// wall fixes is taken only by the tiles that have some
template <class G>
__device__ __forceinline__ bool tile_on_wall(const StageArgs& a, int bxi, int byi) {
  const int gi0 = 1 + bxi * G::TX, gj0 = 1 + byi * G::TY;
  const int clx = (a.ix - 2) - gi0 + 1, cly = (a.jx - 2) - gj0 + 1;
  const bool wx = a.bc_kind[0] != OMHD_BC_PERIODIC && (gi0 == 1 || (clx >= 1 && clx <= G::TX));
  const bool wy = a.bc_kind[2] != OMHD_BC_PERIODIC && (gj0 == 1 || (cly >= 1 && cly <= G::TY));
  return wx || wy;
}

// wall face fixes after phase B: x walls (2D_reconnection/bc.f90:136-165),
// y walls (2D_KH/bc.f90:55-83)
template <class T, class G>
__device__ __forceinline__ void phase_walls(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t, int n) {
  constexpr int TX = G::TX, TY = G::TY, NXS = G::NXS, NYS = G::NYS, XS = TX + 2;
  const int ix = a.ix, jx = a.jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * TY;
  if (a.bc_kind[0] != OMHD_BC_PERIODIC) {
    const int cl = (ix - 2) - gi0 + 1;  // cx of the last interior cell
    for (int k = t; k < TY * NV; k += n) {
      const int cy = k % TY, v = k / TY;
      if (gi0 == 1) {  // west face: VL = flip(VR)
        const T s = m.SRx[v * NXS + cy * XS + 1];
        m.SLx[v * NXS + cy * XS + 0] = ((a.bc_flip[0] >> v) & 1) ? -s : s;
      }
      if (cl >= 1 && cl <= TX) {  // east face: VR = flip(VL)
        const T s = m.SLx[v * NXS + cy * XS + cl];
        m.SRx[v * NXS + cy * XS + cl + 1] = ((a.bc_flip[1] >> v) & 1) ? -s : s;
      }
    }
  }
  if (a.bc_kind[2] != OMHD_BC_PERIODIC) {
    const int cl = (jx - 2) - gj0 + 1;
    // the last threads of the group, so that x and y fixes run side by side
    for (int k = n - 1 - t; k < TX * NV; k += n) {
      const int cx = k % TX, v = k / TX;
      if (gj0 == 1) {  // south face: VL = flip(VR)
        const T s = m.SRy[v * NYS + 1 * TX + cx];
        m.SLy[v * NYS + 0 * TX + cx] = ((a.bc_flip[2] >> v) & 1) ? -s : s;
      }
      if (cl >= 1 && cl <= TY) {  // north face: VR = flip(VL)
        const T s = m.SLy[v * NYS + cl * TX + cx];
        m.SRy[v * NYS + (cl + 1) * TX + cx] = ((a.bc_flip[3] >> v) & 1) ? -s : s;
      }
    }
  }
}

// y faces in x orientation: slot k of the rotated state holds component
// rot(k) (vx <- vy, vy <- vz, vz <- vx and the same for B, the order
// flux_solver.f90:62-70 uses for the y direction), and the x-oriented flux
// slot k belongs to component rot(k)
__device__ __forceinline__ constexpr int rot_y(int k) {
  return (k <= 2) ? (k + 1) % 3 : ((k >= 5 && k <= 7) ? 5 + (k - 4) % 3 : k);
}

// phase C for the FAST FP64 variant: the x faces (items 0..NXF-1) and the y
// faces (items NXF..NXF+NYF-1) through one x-oriented Riemann solver, the y
// faces' components rotated on load and back on store, so that the 544 faces
// of a 16x16 tile fill 17 whole warps (the per-direction form below pads each
// direction to whole warps: 18).
template <class T, int FLUX, class G, int TAPE>
__device__ __forceinline__ void phase_flux_rot(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t,
                                               int n, const StageScalars<T>& ks) {
  constexpr int TX = G::TX, RX = G::RX;
  constexpr int NXS = G::NXS, NYS = G::NYS, NXF = G::NXF, NYF = G::NYF, XS = TX + 2, XF = TX + 1;
  constexpr int PL = RX * G::RY;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * G::TY;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const T ch = ks.ch, gam = ks.gam, r1 = ks.r1, r2 = ks.r2;
  const T* W = m.W;
  for (int q = t; q < NXF + NYF; q += n) {
    const bool xd = q < NXF;
    const int qq = xd ? q : q - NXF;
    // x face (fx, cy): lower cell fx of x row cy; y face (cx, fy): lower cell
    // fy of y column cx
    const int fa = xd ? qq % XF : qq % TX, fb = xd ? qq / XF : qq / TX;
    const T* bl = xd ? m.SLx + fb * XS + fa : m.SLy + fb * TX + fa;
    const T* br = xd ? m.SRx + fb * XS + fa + 1 : m.SRy + (fb + 1) * TX + fa;
    const int sv = xd ? NXS : NYS;
    T L[NV], R[NV], Fo[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const int pv = (xd ? k : rot_y(k)) * sv;
      L[k] = bl[pv];
      R[k] = br[pv];
    }
    if constexpr (TAPE == tape::kNone) {
      riemann_flux<T, 1, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
    } else {
      size_t tc;
      if (xd) {  // face between cells gi0-1+fx and gi0+fx of row gj0+cy
        const int gl = gi0 - 1 + fa, gj = gj0 + fb;
        tc = (size_t)(gl < 0 ? 0 : (gl > ix - 2 ? ix - 2 : gl)) + (size_t)ix * (gj > jx - 2 ? jx - 2 : gj);
      } else {  // face between rows gj0-1+fy and gj0+fy of column gi0+cx
        const int gl = gj0 - 1 + fb, gi = gi0 + fa;
        tc = N + (size_t)(gi > ix - 2 ? ix - 2 : gi) + (size_t)ix * (gl < 0 ? 0 : (gl > jx - 2 ? jx - 2 : gl));
      }
      unsigned k = (TAPE == tape::kReplay) ? a.tface[tc] : 0u;
      riemann_flux<T, 1, FLUX, OMHD_FAST, TAPE>(L, R, ch, gam, r1, r2, Fo, &k);
      if (TAPE == tape::kRecord && a.tface) {
        const bool own = xd ? ((fa >= 1 || gi0 == 1) && gi0 - 1 + fa <= ix - 2 && gj0 + fb <= jx - 2)
                            : ((fb >= 1 || gj0 == 1) && gj0 - 1 + fb <= jx - 2 && gi0 + fa <= ix - 2);
        if (own) a.tface[tc] = (unsigned short)k;
      }
    }
    double F[NV];  // back to the grid's component order
#pragma unroll
    for (int k = 0; k < NV; ++k) F[rot_y(k)] = xd ? to_f64<T>(Fo[rot_y(k)]) : to_f64<T>(Fo[k]);
    if (resist) {
      if (xd) {  // 2D_reconnection/flux_resistive.f90:266-283
        const int fx = fa, cy = fb, g = gi0 - 1 + fx, gj = gj0 + cy;
        if (g >= 0 && g <= ix - 2 && gj <= jx - 2) {
          const int o = (cy + 2) * RX + (fx + 1);  // region index of cell g
          auto B = [&](int var, int dxo, int dyo) { return to_f64<T>(W[var * PL + o + dxo + dyo * RX]); };
          const double odx = 1.0 / a.dx;
          const double eta_dx = eta_at(a.eta_kind, a.xc[g] + 0.5 * a.dx, a.yc[gj], 0.0) * odx;
          const double JyS = -eta_dx * (B(BZ, 1, 0) - B(BZ, 0, 0));
          const double JzS = eta_dx * ((B(BY, 1, 0) - B(BY, 0, 0)) -
                                       0.25 * (B(BX, 0, 1) + B(BX, 1, 1) - B(BX, 0, -1) - B(BX, 1, -1)));
          F[EN] = F[EN] + 0.5 * (JyS * (B(BZ, 0, 0) + B(BZ, 1, 0)) - JzS * (B(BY, 0, 0) + B(BY, 1, 0)));
          F[BY] = F[BY] - JzS;
          F[BZ] = F[BZ] + JyS;
        }
      } else {  // 2D_reconnection/flux_resistive.f90:289-306
        const int cx = fa, fy = fb, gi = gi0 + cx, g = gj0 - 1 + fy;
        if (g >= 0 && g <= jx - 2 && gi <= ix - 2) {
          const int o = (fy + 1) * RX + (cx + 2);  // region index of cell (gi, g)
          auto B = [&](int var, int dxo, int dyo) { return to_f64<T>(W[var * PL + o + dxo + dyo * RX]); };
          const double odx = 1.0 / a.dx;
          const double eta_dx = eta_at(a.eta_kind, a.xc[gi], a.yc[g] + 0.5 * a.dx, 0.0) * odx;
          const double JxS = eta_dx * (B(BZ, 0, 1) - B(BZ, 0, 0));
          const double JzS = eta_dx * (0.25 * (B(BY, 1, 1) + B(BY, 1, 0) - B(BY, -1, 1) - B(BY, -1, 0)) -
                                       (B(BX, 0, 1) - B(BX, 0, 0)));
          F[EN] = F[EN] + 0.5 * (JzS * (B(BX, 0, 0) + B(BX, 0, 1)) - JxS * (B(BZ, 0, 0) + B(BZ, 0, 1)));
          F[BX] = F[BX] + JzS;
          F[BZ] = F[BZ] - JxS;
        }
      }
    }
    double* dst = xd ? m.FX + fb * m.fxr + fa : m.FY + fb * TX + fa;
    const int dv = xd ? m.fxv : m.fyv;
#pragma unroll
    for (int k = 0; k < NV; ++k) dst[k * dv] = F[k];
  }
}

// phase C: fluxes of all x faces (work items 0..NXFP-1, padded to whole
// warps) and all y faces (items NXFP..NXFP+NYF-1)
template <class T, int FLUX, class G, int TAPE>
__device__ __forceinline__ void phase_flux(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t, int n,
                                           const StageScalars<T>& ks) {
  if constexpr (OMHD_FAST && sizeof(T) == 8) {
    phase_flux_rot<T, FLUX, G, TAPE>(a, bxi, byi, m, t, n, ks);
    return;
  }
  constexpr int TX = G::TX, RX = G::RX;
  constexpr int NXS = G::NXS, NYS = G::NYS, NXF = G::NXF, NYF = G::NYF, NXFP = G::NXFP, XS = TX + 2;
  constexpr int PL = RX * G::RY;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * G::TY;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const T ch = ks.ch, gam = ks.gam, r1 = ks.r1, r2 = ks.r2;
  const T* W = m.W;
  constexpr int XF = TX + 1;
  for (int q = t; q < NXFP + NYF; q += n) {
    if (q < NXFP) {
      if (q >= NXF) continue;  // padding lanes
      const int fx = q % XF, cy = q / XF;
      T L[NV], R[NV], Fo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        L[v] = m.SLx[v * NXS + cy * XS + fx];
        R[v] = m.SRx[v * NXS + cy * XS + fx + 1];
      }
      if constexpr (TAPE == tape::kNone) {
        riemann_flux<T, 1, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
      } else {  // face between cells gi0-1+fx and gi0+fx of row gj0+cy
        const int gl = gi0 - 1 + fx, gj = gj0 + cy;
        const size_t tc = (size_t)(gl < 0 ? 0 : (gl > ix - 2 ? ix - 2 : gl)) + (size_t)ix * (gj > jx - 2 ? jx - 2 : gj);
        unsigned k = (TAPE == tape::kReplay) ? a.tface[tc] : 0u;
        riemann_flux<T, 1, FLUX, OMHD_FAST, TAPE>(L, R, ch, gam, r1, r2, Fo, &k);
        if (TAPE == tape::kRecord && a.tface && (fx >= 1 || gi0 == 1) && gl <= ix - 2 && gj <= jx - 2)
          a.tface[tc] = (unsigned short)k;
      }
      if (resist) {  // 2D_reconnection/flux_resistive.f90:266-283
        const int g = gi0 - 1 + fx, gj = gj0 + cy;
        if (g >= 0 && g <= ix - 2 && gj <= jx - 2) {
          const int o = (cy + 2) * RX + (fx + 1);  // region index of cell g
          auto B = [&](int var, int dxo, int dyo) { return to_f64<T>(W[var * PL + o + dxo + dyo * RX]); };
          const double odx = 1.0 / a.dx;
          const double eta_dx = eta_at(a.eta_kind, a.xc[g] + 0.5 * a.dx, a.yc[gj], 0.0) * odx;
          const double JyS = -eta_dx * (B(BZ, 1, 0) - B(BZ, 0, 0));
          const double JzS = eta_dx * ((B(BY, 1, 0) - B(BY, 0, 0)) -
                                       0.25 * (B(BX, 0, 1) + B(BX, 1, 1) - B(BX, 0, -1) - B(BX, 1, -1)));
          Fo[EN] = to_face<T>(to_f64<T>(Fo[EN]) + 0.5 * (JyS * (B(BZ, 0, 0) + B(BZ, 1, 0)) - JzS * (B(BY, 0, 0) + B(BY, 1, 0))));
          Fo[BY] = to_face<T>(to_f64<T>(Fo[BY]) - JzS);
          Fo[BZ] = to_face<T>(to_f64<T>(Fo[BZ]) + JyS);
        }
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) m.FX[v * m.fxv + cy * m.fxr + fx] = to_f64<T>(Fo[v]);
    } else {
      const int qq = q - NXFP;
      const int cx = qq % TX, fy = qq / TX;
      T L[NV], R[NV], Fo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        L[v] = m.SLy[v * NYS + fy * TX + cx];
        R[v] = m.SRy[v * NYS + (fy + 1) * TX + cx];
      }
      if constexpr (TAPE == tape::kNone) {
        riemann_flux<T, 2, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
      } else {  // face between rows gj0-1+fy and gj0+fy of column gi0+cx
        const int gl = gj0 - 1 + fy, gi = gi0 + cx;
        const size_t tc = (size_t)(gi > ix - 2 ? ix - 2 : gi) + (size_t)ix * (gl < 0 ? 0 : (gl > jx - 2 ? jx - 2 : gl));
        unsigned k = (TAPE == tape::kReplay) ? a.tface[N + tc] : 0u;
        riemann_flux<T, 2, FLUX, OMHD_FAST, TAPE>(L, R, ch, gam, r1, r2, Fo, &k);
        if (TAPE == tape::kRecord && a.tface && (fy >= 1 || gj0 == 1) && gl <= jx - 2 && gi <= ix - 2)
          a.tface[N + tc] = (unsigned short)k;
      }
      if (resist) {  // 2D_reconnection/flux_resistive.f90:289-306
        const int gi = gi0 + cx, g = gj0 - 1 + fy;
        if (g >= 0 && g <= jx - 2 && gi <= ix - 2) {
          const int o = (fy + 1) * RX + (cx + 2);  // region index of cell (gi, g)
          auto B = [&](int var, int dxo, int dyo) { return to_f64<T>(W[var * PL + o + dxo + dyo * RX]); };
          const double odx = 1.0 / a.dx;
          const double eta_dx = eta_at(a.eta_kind, a.xc[gi], a.yc[g] + 0.5 * a.dx, 0.0) * odx;
          const double JxS = eta_dx * (B(BZ, 0, 1) - B(BZ, 0, 0));
          const double JzS = eta_dx * (0.25 * (B(BY, 1, 1) + B(BY, 1, 0) - B(BY, -1, 1) - B(BY, -1, 0)) -
                                       (B(BX, 0, 1) - B(BX, 0, 0)));
          Fo[EN] = to_face<T>(to_f64<T>(Fo[EN]) + 0.5 * (JzS * (B(BX, 0, 0) + B(BX, 0, 1)) - JxS * (B(BZ, 0, 0) + B(BZ, 0, 1))));
          Fo[BX] = to_face<T>(to_f64<T>(Fo[BX]) + JzS);
          Fo[BZ] = to_face<T>(to_f64<T>(Fo[BZ]) - JxS);
        }
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) m.FY[v * m.fyv + fy * TX + cx] = to_f64<T>(Fo[v]);
    }
  }
}

// phase D: update, ghost fill, GLM, CFL of the tile's cells t, t+n, ...;
// returns this thread's largest CFL speed (stage 2) or 0
template <class T, class G>
__device__ __forceinline__ double phase_update(const StageArgs& a, int bxi, int byi, const TileMem<T>& m, int t,
                                               int n, const StageScalars<T>& ks) {
  constexpr int TX = G::TX, TY = G::TY;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int gi0 = 1 + bxi * TX, gj0 = 1 + byi * TY;
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const double gamma = a.gamma;
  const double f1g = a.gm1;
  // the argument block may live in global memory (ensembles), where a store to
  // the state could alias it: every pointer and scalar used in the loop is
  // read once, here
  double* const Uout = a.Uout;
  double* const Uhost = a.Uhost;
  const double* const Ubase = a.Ubase;
  const double* const U1 = a.U1;
  const double dtx = ks.dtx, dty = ks.dty, glmf = ks.glmf;
  const bool iso = a.iso, rk2 = a.stage == 1 || a.time_type == OMHD_TIME_RK2, stage2 = a.stage == 2;
  int flip[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) flip[q] = a.bc_flip[q];
  double vcell = 0.0;
  for (int k = t; k < TX * TY; k += n) {
    const int tx = k % TX, ty = k / TX;
    const int gi = gi0 + tx, gj = gj0 + ty;
    if (gi > ix - 2 || gj > jx - 2) continue;
    const size_t c = (size_t)gi + (size_t)ix * gj;
    double out[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      // F(i-1/2) - F(i+1/2) in FP64
      const double* fx = m.FX + v * m.fxv + ty * m.fxr + tx;
      const double dF = fx[0] - fx[1];
      const double gm = m.FY[v * m.fyv + ty * TX + tx], gp = m.FY[v * m.fyv + (ty + 1) * TX + tx];
      double d;
      if (iso)
        d = dtx * (dF + gm - gp);  // rk.f90:26-35 operation order
      else
        d = dtx * dF + dty * (gm - gp);
      double ub = Ubase[v * N + c];
      if (v == PS) ub = glmf * ub;
      if (rk2)
        out[v] = ub + d;  // rk_tvd21 / rk_std21 / rk_std22
      else
        out[v] = 0.5 * (ub + U1[v * N + c] + d);  // rk_tvd22 (rk.f90:56-66)
    }
    if (stage2) out[PS] = glmf * out[PS];  // second GLM half (main.f90:185)

    // owner-writes ghost fill (bc.f90 order: x sides, then y sides)
    int xt[3], yt[3], xf[3], yf[3], nxt = 1, nyt = 1;
    xt[0] = gi;
    xf[0] = 0;
    yt[0] = gj;
    yf[0] = 0;
    if (gi == 1) { xt[nxt] = perx ? ix - 1 : 0; xf[nxt] = perx ? 0 : flip[0]; ++nxt; }
    if (gi == ix - 2) { xt[nxt] = perx ? 0 : ix - 1; xf[nxt] = perx ? 0 : flip[1]; ++nxt; }
    if (gj == 1) { yt[nyt] = pery ? jx - 1 : 0; yf[nyt] = pery ? 0 : flip[2]; ++nyt; }
    if (gj == jx - 2) { yt[nyt] = pery ? 0 : jx - 1; yf[nyt] = pery ? 0 : flip[3]; ++nyt; }
    for (int b = 0; b < nyt; ++b)
      for (int q = 0; q < nxt; ++q) {
        const size_t cc = (size_t)xt[q] + (size_t)ix * yt[b];
        const int fm = xf[q] ^ yf[b];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double o = ((fm >> v) & 1) ? -out[v] : out[v];
          Uout[v * N + cc] = o;
          if (Uhost) Uhost[v * N + cc] = o;  // result straight to host memory
        }
      }

    if (stage2) {  // set_dt.f90:27-37 on the new state
      const double ro = out[RO];
      const double iro = rcp_<double, OMHD_FAST>(ro);  // one reciprocal for the three velocities
      const double vx = divr_<double, OMHD_FAST>(out[MX], ro, iro), vy = divr_<double, OMHD_FAST>(out[MY], ro, iro),
                   vz = divr_<double, OMHD_FAST>(out[MZ], ro, iro);
      const double rv2 = vx * out[MX] + vy * out[MY] + vz * out[MZ];
      const double B2 = out[BX] * out[BX] + out[BY] * out[BY] + out[BZ] * out[BZ];
      const double pr = f1g * (out[EN] - 0.5 * (rv2 + B2));
      const double f1 = gamma * pr;
      const double vfx = fast_speed<double, OMHD_FAST>(f1, B2, out[BX], ro);
      const double vfy = fast_speed<double, OMHD_FAST>(f1, B2, out[BY], ro);
      const double sx = fabs(vx) + vfx, sy = fabs(vy) + vfy;
      const double sc = lt_<double, OMHD_FAST>(sx, sy) ? sy : sx;  // fmax2(sx, sy)
      vcell = lt_<double, OMHD_FAST>(vcell, sc) ? sc : vcell;
    }
  }
  return vcell;
}

// One stage on one tile (tile coordinates bxi, byi) of the grid described by
// `a`, by all threads of the CTA; returns this thread's CFL speed of the
// updated cells (stage 2) or 0.  Three or four CTA-wide barriers.
template <class T, int FLUX, class G, int TAPE = tape::kNone>
__device__ __forceinline__ double stage2d_tile(const StageArgs& a, int bxi, int byi, unsigned char* smem_raw,
                                               const StageScalars<T>& ks) {
  const TileMem<T> m = tile_mem_separate<T, G>(smem_raw);
  const int tid = threadIdx.x;
  phase_load<T, G>(a, bxi, byi, m, tid, G::NT, ks.glmf);
  __syncthreads();
  phase_recon<T, G, TAPE>(a, bxi, byi, m, tid, G::NT);
  __syncthreads();
  if (tile_on_wall<G>(a, bxi, byi)) {
    phase_walls<T, G>(a, bxi, byi, m, tid, G::NT);
    __syncthreads();
  }
  phase_flux<T, FLUX, G, TAPE>(a, bxi, byi, m, tid, G::NT, ks);
  __syncthreads();
  return phase_update<T, G>(a, bxi, byi, m, tid, G::NT, ks);
}

// one CTA per tile of one grid
template <class T, int FLUX, int TAPE = tape::kNone>
__global__ void __launch_bounds__(GeoFor<T>::type::NT, sizeof(T) == 4 ? OMHD_MIXED_MIN_CTAS : 1)
    k_stage2d(const StageArgs a) {
  using G = typename GeoFor<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red32[32];
  __shared__ int skip;
  __shared__ StageScalars<T> ks;
  StepState* st = a.st;
  // one thread decides, so that the whole CTA leaves together (the error word
  // may be set by another CTA while this one starts)
  if (threadIdx.x == 0) {
    skip = st->done || *(volatile int*)&a.err->code;
    stage_scalars<T>(a, st, ks);
  }
  __syncthreads();
  if (skip) return;
  const double vcell = stage2d_tile<T, FLUX, G, TAPE>(a, blockIdx.x, blockIdx.y, smem_raw, ks);
  if (a.stage == 2) {
    const double bm = block_max_pos(vcell, red32);
    StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
    reduce_and_finalize(st, sc, a.err, bm, gridDim.x * gridDim.y, 1);
  }
}

// ---------------------------------------------------------------------------
// FP64 pipelined stage kernel: one persistent CTA per SM, warp-specialised.
// The flux phase C is FP64-pipe bound (~96 % of the pipe), while the load +
// u2v phase A, the slope phase B and the update phase D are latency bound
// (~50 %).  So NPW producer warps run A and B (+ wall fixes) of tile i+1
// while the 9 consumer warps run C and D of tile i: two face-state buffers in
// shared memory, handed over with named barriers (FULL[b]: producers arrive,
// consumers wait; EMPTY[b]: consumers arrive after D, producers wait before
// refilling b).  Fluxes overwrite the lower-cell face state that only their
// own face reads, so a buffer is 4 face-state arrays (83 KB) and the CTA holds
// W + 2 buffers = 195 KB.  Non-resistive 2D runs (the resistive terms read W
// in phase C, which the producers already refill).
// ---------------------------------------------------------------------------
using PipeGeo = Geo2<16, 16>;
constexpr int kPipeBarProd = 1, kPipeBarCons = 2, kPipeBarFull = 3, kPipeBarEmpty = 5;

__device__ __forceinline__ void named_bar_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void named_bar_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

constexpr size_t pipe_smem_bytes() {
  return sizeof(double) * (size_t)NV * (PipeGeo::RX * PipeGeo::RY + 2 * 2 * (PipeGeo::NXS + PipeGeo::NYS));
}
// TMA staging area after the two buffers: the conserved halo tile as one box of
// (RX + 2) x RY cells x 9 planes, 128-byte aligned (31.7 KB; 226.5 KB in all)
constexpr int kPipeBoxX = PipeGeo::RX + 2, kPipeBoxY = PipeGeo::RY;
constexpr unsigned kPipeBoxBytes = sizeof(double) * NV * kPipeBoxX * kPipeBoxY;
constexpr size_t pipe_stage_off() { return (pipe_smem_bytes() + 127) / 128 * 128; }
constexpr size_t pipe_smem_bytes_tma() { return pipe_stage_off() + 128 + kPipeBoxBytes; }
static_assert(pipe_smem_bytes_tma() <= 232448 - 512, "pipelined kernel exceeds the shared memory of one CTA");
static_assert((kPipeBoxX * 8) % 16 == 0, "TMA box rows must be whole 16-byte units");
// polls of a TMA completion before a tile is declared lost (well beyond any
// real transfer; the kernel then records OMHD_TIMEOUT and keeps its barrier
// protocol, so nothing waits forever)
constexpr uint32_t kTmaMaxPolls = 1u << 22;

__device__ __forceinline__ TileMem<double> pipe_mem(unsigned char* smem_raw, int b) {
  using G = PipeGeo;
  TileMem<double> m;
  m.W = reinterpret_cast<double*>(smem_raw);
  m.SLx = m.W + NV * G::RX * G::RY + (size_t)b * NV * 2 * (G::NXS + G::NYS);
  m.SRx = m.SLx + NV * G::NXS;
  m.SLy = m.SRx + NV * G::NXS;
  m.SRy = m.SLy + NV * G::NYS;
  m.FX = m.SLx;  // flux of x face (fx, cy) in the SLx slot of cell fx of row cy
  m.fxv = G::NXS;
  m.fxr = G::TX + 2;
  m.FY = m.SLy;  // flux of y face (cx, fy) in the SLy slot of cell fy of column cx
  m.fyv = G::NYS;
  return m;
}

template <int FLUX, int TAPE, int NPW>
__global__ void __launch_bounds__(NPW * 32 + PipeGeo::NT, 1)
    k_stage2d_pipe(const StageArgs a, const __grid_constant__ CUtensorMap tmap, const int use_tma) {
  using G = PipeGeo;
  constexpr int NP = NPW * 32, NC = G::NT, NTOT = NP + NC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ double red32[32];
  __shared__ __align__(8) uint64_t tma_bar;
  __shared__ int skip;
  __shared__ StageScalars<double> ks;
  StepState* st = a.st;
  if (threadIdx.x == 0) {
    skip = st->done || *(volatile int*)&a.err->code;
    stage_scalars<double>(a, st, ks);
  }
  __syncthreads();
  if (skip) return;
  const double glmf = ks.glmf;
  const int ntx = (a.ix - 2 + G::TX - 1) / G::TX;
  const int ntiles = ntx * ((a.jx - 2 + G::TY - 1) / G::TY);
  double vmax = 0.0;
  if (threadIdx.x < NP) {  // producers: A, B, wall fixes of tiles blockIdx.x, +gridDim.x, ...
    const int t = threadIdx.x;
    // TMA staging: a tile whose whole halo lies inside the array (no periodic
    // wrap, no wall clamp, no ragged edge) arrives as one 3D box load issued
    // by producer thread 0 while the producers work on the previous tile; the
    // other tiles take ordinary loads.  The box starts one cell left of the
    // halo so that its x coordinate is even (8-byte elements, 16-byte rule).
    unsigned char* s0 = smem_raw + pipe_stage_off();
    double* S = reinterpret_cast<double*>(s0 + ((128u - (smem_u32(s0) & 127u)) & 127u));  // 128-byte aligned
    auto staged = [&](int w) {
      if (!use_tma) return false;
      const int gi0 = 1 + (w % ntx) * G::TX, gj0 = 1 + (w / ntx) * G::TY;
      return gi0 >= 3 && gj0 >= 2 && gi0 - 2 + G::RX <= a.ix && gj0 - 2 + G::RY <= a.jx;
    };
    auto issue = [&](int w) {
      const int gi0 = 1 + (w % ntx) * G::TX, gj0 = 1 + (w / ntx) * G::TY;
      fence_proxy_async_smem();  // the producers' reads of S come before this write
      mbar_arrive_expect_tx(&tma_bar, kPipeBoxBytes);
      tma_load_3d(S, &tmap, gi0 - 3, gj0 - 2, 0, &tma_bar);
    };
    uint32_t tphase = 0;
    bool tma_lost = false;
    if (use_tma) {
      if (t == 0) mbar_init(&tma_bar, 1);
      named_bar_sync(kPipeBarProd, NP);
      if (t == 0 && (int)blockIdx.x < ntiles && staged(blockIdx.x)) issue(blockIdx.x);
    }
    int i = 0;
    for (int w = blockIdx.x; w < ntiles; w += gridDim.x, ++i) {
      const int b = i & 1;
      const TileMem<double> m = pipe_mem(smem_raw, b);
      if (i >= 2) named_bar_sync(kPipeBarEmpty + b, NTOT);  // consumers are done with buffer b
      if (i >= 1) named_bar_sync(kPipeBarProd, NP);         // W of the previous tile is read
      if (staged(w) && !tma_lost) {
        if (!mbar_wait_parity(&tma_bar, tphase & 1u, kTmaMaxPolls)) {
          tma_lost = true;  // recorded; the tile's results are void, the protocol goes on
          raise_error(a.err, OMHD_TIMEOUT, 1 + (w % ntx) * G::TX, 1 + (w / ntx) * G::TY, 0, 0, 0.0);
        }
        ++tphase;
        phase_load<double, G, true>(a, w % ntx, w / ntx, m, t, NP, glmf, S);
      } else {
        phase_load<double, G>(a, w % ntx, w / ntx, m, t, NP, glmf);
      }
      named_bar_sync(kPipeBarProd, NP);
      const int wn = w + (int)gridDim.x;
      if (t == 0 && !tma_lost && wn < ntiles && staged(wn)) issue(wn);
      phase_recon<double, G, TAPE>(a, w % ntx, w / ntx, m, t, NP);
      if (tile_on_wall<G>(a, w % ntx, w / ntx)) {
        named_bar_sync(kPipeBarProd, NP);
        phase_walls<double, G>(a, w % ntx, w / ntx, m, t, NP);
      }
      __threadfence_block();
      named_bar_arrive(kPipeBarFull + b, NTOT);
    }
    if (tma_lost && t == 0) mbar_wait_parity(&tma_bar, tphase & 1u, kTmaMaxPolls);  // a late copy lands first
  } else {  // consumers: C, D of the same tiles, one tile behind
    const int t = threadIdx.x - NP;
    const int nmine = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    int i = 0;
    for (int w = blockIdx.x; w < ntiles; w += gridDim.x, ++i) {
      const int b = i & 1;
      const TileMem<double> m = pipe_mem(smem_raw, b);
      named_bar_sync(kPipeBarFull + b, NTOT);
      phase_flux<double, FLUX, G, TAPE>(a, w % ntx, w / ntx, m, t, NC, ks);
      named_bar_sync(kPipeBarCons, NC);
      const double v = phase_update<double, G>(a, w % ntx, w / ntx, m, t, NC, ks);
      vmax = lt_<double, OMHD_FAST>(vmax, v) ? v : vmax;
      if (i + 2 < nmine) {  // the producers refill buffer b for tile i+2
        __threadfence_block();
        named_bar_arrive(kPipeBarEmpty + b, NTOT);
      }
    }
  }
  if (a.stage == 2) {
    const double bm = block_max_pos(vmax, red32);
    StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
    reduce_and_finalize(st, sc, a.err, bm, gridDim.x, 1);
  }
}

// producer warps of the pipelined kernel (a build-time constant, for tuning)
#ifndef OMHD_PIPE_PRODUCER_WARPS
#define OMHD_PIPE_PRODUCER_WARPS 3
#endif
template <int FLUX, int TAPE, int NPW = OMHD_PIPE_PRODUCER_WARPS>
int launch_pipe(const StageArgs& a, cudaStream_t s) {
  const size_t bytes = pipe_smem_bytes_tma();
  static std::atomic<unsigned long long> configured{0};
  int r = set_smem_attr_once(k_stage2d_pipe<FLUX, TAPE, NPW>, bytes, configured);
  if (r) return r;
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return (int)e;
  const int ntiles = ((a.ix - 2 + PipeGeo::TX - 1) / PipeGeo::TX) * ((a.jx - 2 + PipeGeo::TY - 1) / PipeGeo::TY);
  const int grid = ntiles < nsm ? ntiles : nsm;
  // the tensor map of this stage's input state (encoded on the host, passed by
  // value; an array TMA cannot address -- odd ix, unaligned base -- is loaded
  // with ordinary loads)
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof tmap);
  const int use_tma =
      tma_staging_enabled() && tma_encode_state_map(&tmap, a.Uin, a.ix, a.jx, NV, kPipeBoxX, kPipeBoxY) == 0;
  k_stage2d_pipe<FLUX, TAPE, NPW><<<grid, NPW * 32 + PipeGeo::NT, bytes, s>>>(a, tmap, use_tma);
  return (int)cudaGetLastError();
}

// Ensemble of independent 2D grids in one persistent launch: CTAs take the
// tiles of all grids from a work counter (*queue, zero at launch; work item
// w -> grid by binary search of the tile prefix sums), so members that are
// cheap this step (finished, or failed) leave no CTA idle; each grid keeps its
// own dt, step record and error word, and the CTA that finishes the last tile
// of a grid in stage 2 plans that grid's next step.
// FP32-mixed: two CTAs per SM for 288-thread tiles, four for 160-thread tiles
// (96 registers), hide the latency of the FP64 load and update phases and of
// the barriers behind each other's work
template <class T, int FLUX, class G>
__global__ void __launch_bounds__(G::NT, sizeof(T) == 4 ? (G::NT <= 160 ? 4 : 2) : 1)
    k_batch2d(const StageArgs* __restrict__ args,
                                                   const int* __restrict__ tile_start, int ngrids, int total_tiles,
                                                   int* __restrict__ queue) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red32[32];
  __shared__ unsigned int is_last;
  // the work item's descriptor, written by thread 0 before the barrier that
  // opens the item: two slots by item parity, so that thread 0 fills the next
  // item's slot while the other threads may still be reading this item's
  // (one barrier per item instead of three: every thread passes the opening
  // barrier of item i+1 only after finishing item i, so a slot is rewritten
  // only after every read of it)
  __shared__ int w_s[2], grid_s[2], skip_s[2];
  __shared__ StageScalars<T> ks[2];
  for (int it = 0;; ++it) {
    const int sl = it & 1;
    if (threadIdx.x == 0) {
      const int w = atomicAdd(queue, 1);
      w_s[sl] = w;
      if (w < total_tiles) {
        int lo = 0, hi = ngrids - 1;  // last grid with tile_start <= w
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (tile_start[mid] <= w)
            lo = mid;
          else
            hi = mid - 1;
        }
        grid_s[sl] = lo;
        const StageArgs& g = args[lo];
        skip_s[sl] = g.st->done || *(volatile int*)&g.err->code;
        stage_scalars<T>(g, g.st, ks[sl]);
      }
    }
    __syncthreads();
    const int w = w_s[sl];  // uniform over the CTA
    if (w >= total_tiles) break;
    const int lo = grid_s[sl];
    const StageArgs& a = args[lo];
    StepState* st = a.st;
    const int local = w - tile_start[lo];
    const int ntx = (a.ix - 2 + G::TX - 1) / G::TX;
    const int ntiles = ntx * ((a.jx - 2 + G::TY - 1) / G::TY);
    const bool skip = skip_s[sl];
    double vcell = 0.0;
    if (!skip) vcell = stage2d_tile<T, FLUX, G>(a, local % ntx, local / ntx, smem_raw, ks[sl]);
    if (!skip && a.stage == 2) {
      const double bm = block_max_pos(vcell, red32);
      if (threadIdx.x == 0) {
        atomic_max_pos_double(&st->vmax_acc, bm);
        __threadfence();
        is_last = (atomicAdd(&st->counter, 1u) == (unsigned)ntiles - 1) ? 1u : 0u;
      }
      __syncthreads();
      if (is_last && threadIdx.x == 0) {
        __threadfence();
        StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
        finalize_step(st, sc, a.err, 1);
      }
    }
    // no barrier here: the next item's opening barrier orders this item's reads
    // of shared memory before the next item's writes
  }
}

template <class T, int FLUX, int TAPE = tape::kNone>
int launch_one(const StageArgs& a, cudaStream_t s) {
  using G = typename GeoFor<T>::type;
  const size_t bytes = G::template smem_bytes<T>();
  static std::atomic<unsigned long long> configured{0};
  const int r = set_smem_attr_once(k_stage2d<T, FLUX, TAPE>, bytes, configured);
  if (r) return r;
  dim3 grid((a.ix - 2 + G::TX - 1) / G::TX, (a.jx - 2 + G::TY - 1) / G::TY);
  k_stage2d<T, FLUX, TAPE><<<grid, G::NT, bytes, s>>>(a);
  return (int)cudaGetLastError();
}

template <class T, int FLUX, class G>
int launch_batch_one(const StageArgs* args_dev, int* tile_start_dev, int ngrids, int total_tiles, int ctas,
                     cudaStream_t s) {
  const size_t bytes = G::template smem_bytes<T>();
  static std::atomic<unsigned long long> configured{0};
  const int r = set_smem_attr_once(k_batch2d<T, FLUX, G>, bytes, configured);
  if (r) return r;
  int* queue = tile_start_dev + ngrids + 1;  // work counter after the prefix sums
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int), s);
  if (e != cudaSuccess) return (int)e;
  k_batch2d<T, FLUX, G><<<ctas, G::NT, bytes, s>>>(args_dev, tile_start_dev, ngrids, total_tiles, queue);
  return (int)cudaGetLastError();
}

// Batched launch with one of the tile shapes the ensemble autotuner chooses
// from (HLLD only: the ensemble configuration's Riemann solver).
template <class T>
int launch_batch_variant(int flux, int tile_kind, const StageArgs* args, int* tile_start, int ngrids,
                         int total_tiles, int ctas, cudaStream_t s) {
  if (flux != FX_HLLD) return (int)cudaErrorNotSupported;
  switch (tile_kind) {
    case 0: return launch_batch_one<T, FX_HLLD, Geo2<32, 8>>(args, tile_start, ngrids, total_tiles, ctas, s);
    case 1: return launch_batch_one<T, FX_HLLD, Geo2<32, 4>>(args, tile_start, ngrids, total_tiles, ctas, s);
    case 2: return launch_batch_one<T, FX_HLLD, Geo2<16, 16>>(args, tile_start, ngrids, total_tiles, ctas, s);
    case 3: return launch_batch_one<T, FX_HLLD, Geo2<64, 4>>(args, tile_start, ngrids, total_tiles, ctas, s);
    default: return launch_batch_one<T, FX_HLLD, Geo2<16, 8>>(args, tile_start, ngrids, total_tiles, ctas, s);
  }
}

template <class T>
int launch_variant(const StageArgs& a, cudaStream_t s) {
  switch (a.flux_type) {
    case FX_LLF: return launch_one<T, FX_LLF>(a, s);
    case FX_HLL: return launch_one<T, FX_HLL>(a, s);
    case FX_HLLC: return launch_one<T, FX_HLLC>(a, s);
    case FX_HLLD: return launch_one<T, FX_HLLD>(a, s);
    default: return launch_one<T, FX_LHLLD>(a, s);
  }
}

}  // namespace OMHD_VARIANT
}  // namespace omhd
