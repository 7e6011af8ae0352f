// omhd_fused3d_pipe.cuh -- warp-specialised FP64 3D stage kernel (HLLD with
// minmod or MC, the FAST FP64 arithmetic).
//
// A CTA owns a TX x TY = 16 x 8 column and marches a chunk of ZC planes, like
// k_stage3d, but its warps are split as in the 2D pipelined kernel:
//   producers (3 warps), for plane p: load + u2v of plane p+2 into a ring of
//     five primitive planes, positivity of plane p, the x and y face states of
//     plane p (limiter.f90, paired cells) and the z face states of face p+1/2
//     (upper state of cell p, lower state of cell p+1), the x/y wall fixes and
//     the top z wall (the bc_for_F/G/H pattern of 3D_reconnection_gpu/bc.cuf);
//   consumers (9 warps), for plane p, one plane behind: the Riemann fluxes of
//     its 136 x faces, 144 y faces and the z face p+1/2 through one
//     x-oriented FP64 HLLD solver (y and z faces rotated into x orientation),
//     the resistive face terms (3D_reconnection_gpu/flux_resistive.cuf), and
//     the update of plane p (rk.f90) with the owner-writes ghost fill, GLM and
//     the CFL reduction in stage 2 (by the consumers that own cells; the others
//     go on to the next plane's faces meanwhile).
// Two face-state buffers change hands through named barriers (FULL[b]:
// producers arrive, consumers wait -- split into the consumers that own cells
// and the others; EMPTY[b]: consumers arrive when done with b, producers wait
// before refilling b); fluxes overwrite the lower-cell
// face state that only their own face reads; the z flux of face p-1/2 is kept
// per cell in shared memory (Fzm).  The ring holds planes p-1 .. p+3: the
// consumers read p-1 .. p+1 (resistive terms) while the producers write p+3
// into the slot of p-2, which the consumers released with plane p-1 (the same
// EMPTY barrier).  Producers and consumers walk the same plane sequence, so
// every barrier's arrive and sync counts match by construction and no CTA
// waits on another.
#pragma once
#include "omhd_fused3d.cuh"

namespace omhd {
namespace OMHD_VARIANT {
namespace d3p {

constexpr int TX = 16, TY = 8, NCELL = TX * TY;
constexpr int RX = TX + 4, RY = TY + 4, PL = RX * RY;
constexpr int NRING = 5;
constexpr int XS = TX + 2, NXS = TY * XS;  // x-reconstructed cells (rows of TX+2)
constexpr int NYS = (TY + 2) * TX;         // y-reconstructed cells (columns of TY+2)
constexpr int NXF = TY * (TX + 1), NYF = (TY + 1) * TX, NZF = NCELL;
// planes per CTA and the producer / consumer warp split (build-time constants, for tuning)
#ifndef OMHD_PIPE3D_ZCHUNK
#define OMHD_PIPE3D_ZCHUNK 128
#endif
#ifndef OMHD_PIPE3D_PRODUCER_WARPS
#define OMHD_PIPE3D_PRODUCER_WARPS 3
#endif
constexpr int ZC = OMHD_PIPE3D_ZCHUNK;
constexpr int NPW = OMHD_PIPE3D_PRODUCER_WARPS, NP = NPW * 32, NC = (12 - NPW) * 32, NTOT = NP + NC;
// named barriers: producers; per buffer b: FULL_OWN[b] (producers arrive, the
// consumers that own cells wait), FULL_NON[b] (producers arrive, the other
// consumers wait), EMPTY[b] (all consumers arrive, producers wait) and
// CONS[b] (the cell owners wait for every consumer's fluxes; the others only
// arrive).  The consumers without cells thus start plane p+1's faces while the
// owners update plane p; each barrier is used again two planes later, and the
// producers can re-arm a buffer's barriers only after EMPTY[b], which the
// owners release after their update, so no generation is overtaken.
constexpr int kBarProd = 1, kBarFull = 3, kBarEmpty = 5, kBarCons = 7, kBarFullNon = 9;
constexpr int NOWN = NCELL, NNON = NC - NCELL;  // consumer threads that own a cell / own none
static_assert(NOWN % 32 == 0 && NNON % 32 == 0 && NNON > 0, "owner split must be whole warps");
// one buffer: SLx, SRx [NV][NXS], SLy, SRy [NV][NYS], SLz, SRz [NV][NZF]
constexpr int BUF = NV * 2 * (NXS + NYS + NZF);
constexpr size_t kSmemDoubles = (size_t)NRING * NV * PL + 2 * (size_t)BUF + (size_t)NV * NCELL;
constexpr size_t smem_bytes() { return sizeof(double) * kSmemDoubles; }
static_assert(smem_bytes() + 2048 <= 232448, "3D pipelined kernel exceeds the shared memory of one CTA");
static_assert(XS % 2 == 0 && (TY + 2) % 2 == 0, "paired reconstruction needs even strips");

__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// y faces in x orientation: slot k holds component rot_y(k) (vn <- vy,
// vt1 <- vz, vt2 <- vx and the same for B: flux_solver.f90:62-70 for dir 2)
__device__ __forceinline__ constexpr int rot_y(int k) {
  return (k <= 2) ? (k + 1) % 3 : ((k >= 5 && k <= 7) ? 5 + (k - 4) % 3 : k);
}
// z faces in x orientation: slot k holds component rot_z(k) (vn <- vz,
// vt1 <- vx, vt2 <- vy and the same for B: flux_solver.f90:62-70 for dir 3)
__device__ __forceinline__ constexpr int rot_z(int k) {
  return (k <= 2) ? (k + 2) % 3 : ((k >= 5 && k <= 7) ? 5 + (k - 3) % 3 : k);
}

struct Buf {
  double *SLx, *SRx, *SLy, *SRy, *SLz, *SRz;
};
__device__ __forceinline__ Buf buf_at(double* base) {
  Buf b;
  b.SLx = base;
  b.SRx = b.SLx + NV * NXS;
  b.SLy = b.SRx + NV * NXS;
  b.SRy = b.SLy + NV * NYS;
  b.SLz = b.SRy + NV * NYS;
  b.SRz = b.SLz + NV * NZF;
  return b;
}

__device__ __forceinline__ int ring_slot(int k) { return ((k % NRING) + NRING) % NRING; }

// load + u2v of plane gk (mapped by the z boundary) into its ring slot; threads t of n
__device__ __forceinline__ void load_plane(const StageArgs& a, double* W, int gk, int gi0, int gj0, bool perx,
                                           bool pery, bool perz, bool resist, double glmf, int t, int n) {
  const int ix = a.ix, jx = a.jx, kx = a.kx;
  const size_t N = (size_t)ix * jx * kx;
  const double f1g = a.gamma - 1;
  const int mk = d3::map_idx(gk, kx, perz);
  double* Ws = W + (size_t)ring_slot(gk) * NV * PL;
  for (int q = t; q < PL; q += n) {
    const int rx = q % RX, ry = q / RX;
    const bool cx_in = rx >= 2 && rx < TX + 2, cy_in = ry >= 2 && ry < TY + 2;
    if (!cx_in && !cy_in) {  // corners: only the diagonal neighbours, for the resistive terms
      if (!resist || rx == 0 || rx == RX - 1 || ry == 0 || ry == RY - 1) continue;
    }
    const size_t c = (size_t)d3::map_idx(gi0 - 2 + rx, ix, perx) +
                     (size_t)ix * ((size_t)d3::map_idx(gj0 - 2 + ry, jx, pery) + (size_t)jx * mk);
    const double* U = a.Uin;
    double u[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[v] = __ldg(U + v * N + c);
    const double ro = u[RO];
    const double iro = rcp_<double, true>(ro);  // one reciprocal for the three velocities
    const double vx = divr_<double, true>(u[MX], ro, iro), vy = divr_<double, true>(u[MY], ro, iro),
                 vz = divr_<double, true>(u[MZ], ro, iro);  // 3D_basic/u2v.f90:24
    const double rv2 = vx * u[MX] + vy * u[MY] + vz * u[MZ];
    const double B2 = u[BX] * u[BX] + u[BY] * u[BY] + u[BZ] * u[BZ];
    const double pr = f1g * (u[EN] - 0.5 * (rv2 + B2));
    Ws[VX * PL + q] = vx;
    Ws[VY * PL + q] = vy;
    Ws[VZ * PL + q] = vz;
    Ws[PR * PL + q] = pr;
    Ws[RO * PL + q] = ro;
    Ws[BX * PL + q] = u[BX];
    Ws[BY * PL + q] = u[BY];
    Ws[BZ * PL + q] = u[BZ];
    Ws[PS * PL + q] = (a.stage == 1) ? glmf * u[PS] : u[PS];
  }
}

template <int FLUX>
__global__ void __launch_bounds__(NTOT, 1) k_stage3d_pipe(const StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* W = reinterpret_cast<double*>(smem_raw);  // [NRING][NV][PL]
  double* bufbase = W + (size_t)NRING * NV * PL;
  double* Fzm = bufbase + 2 * (size_t)BUF;  // [NV][NCELL]: z flux of face p-1/2
  __shared__ double red32[32];
  __shared__ double ex_c[TX + 2], ex_f[TX + 2], ez_c[ZC + 2], ez_f[ZC + 2];
  __shared__ int skip;

  StepState* st = a.st;
  if (threadIdx.x == 0) skip = st->done || *(volatile int*)&a.err->code;
  __syncthreads();
  if (skip) return;
  const double dt = st->dt, chd = st->ch, glmf = st->glm_f;
  const int ix = a.ix, jx = a.jx, kx = a.kx;
  const size_t N = (size_t)ix * jx * kx;
  const int gi0 = 1 + blockIdx.x * TX, gj0 = 1 + blockIdx.y * TY;
  const int k0 = 1 + blockIdx.z * ZC;
  const int k1 = min(k0 + ZC - 1, kx - 2);
  const int nplanes = k1 - k0 + 1;
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const bool perz = a.bc_kind[4] == OMHD_BC_PERIODIC;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const double gamma = a.gamma;
  const double r1 = 1.0 / (gamma - 1.0), r2 = gamma / (gamma - 1.0);
  const int lm = a.lm_type;
  const bool sep_eta = a.eta_kind == OMHD_ETA_HARRIS_XZ;
  const double inv_dx = 1.0 / a.dx;
  auto Wv = [&](int k, int v, int o) -> double { return W[(size_t)ring_slot(k) * NV * PL + v * PL + o]; };

  // separable Harris resistivity: exp(-x^2/4) over this column's x cells and
  // faces, exp(-z^2/4) over this chunk's z cells and faces (as k_stage3d)
  if (sep_eta) {
    for (int q = threadIdx.x; q < 2 * (TX + 2) + 2 * (ZC + 2); q += NTOT) {
      if (q < 2 * (TX + 2)) {
        const int p = q % (TX + 2);
        const double x = a.xc[min(gi0 - 1 + p, ix - 1)] + (q >= TX + 2 ? 0.5 * a.dx : 0.0);
        (q < TX + 2 ? ex_c : ex_f)[p] = exp(-(x * x) / 4.0);
      } else {
        const int r = q - 2 * (TX + 2), p = r % (ZC + 2);
        const double z = a.zc[min(k0 - 1 + p, kx - 1)] + (r >= ZC + 2 ? 0.5 * a.dx : 0.0);
        (r < ZC + 2 ? ez_c : ez_f)[p] = exp(-(z * z) / 4.0);
      }
    }
  }
  __syncthreads();
  // eta/dx at the face of kind `face` (1: x, 2: y, 3: z) whose lower cell is
  // (gi, gj, kk); xo indexes the x tables (x faces: face index, else cell + 1)
  auto eta_of = [&](int face, int xo, int kk, int gi, int gj) -> double {
    if (sep_eta)
      return d3::harris_eta_dx((face == 1 ? ex_f : ex_c)[xo], (face == 3 ? ez_f : ez_c)[kk - k0 + 1], inv_dx);
    return d3::eta3(a.eta_kind, a.xc[gi] + (face == 1 ? 0.5 * a.dx : 0.0), a.yc[gj] + (face == 2 ? 0.5 * a.dx : 0.0),
                    a.zc[kk] + (face == 3 ? 0.5 * a.dx : 0.0)) /
           a.dx;
  };

  double vmax = 0.0;
  if (threadIdx.x < NP) {
    // ======================= producers =======================
    const int t = threadIdx.x;
    // prologue: planes k0-2 .. k0+1, and the z flux of face k0-1/2 into Fzm
    for (int p = k0 - 2; p <= k0 + 1; ++p) load_plane(a, W, p, gi0, gj0, perx, pery, perz, resist, glmf, t, NP);
    bar_sync(kBarProd, NP);
    for (int c = t; c < NCELL; c += NP) {
      const int tx = c % TX, ty = c / TX;
      const int o = (ty + 2) * RX + (tx + 2);
      double L[NV], R[NV], Fo[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const int v = rot_z(k);
        const double wm = Wv(k0 - 2, v, o), w0 = Wv(k0 - 1, v, o), w1 = Wv(k0, v, o), w2 = Wv(k0 + 1, v, o);
        const double d0 = w0 - wm, d1 = w1 - w0, d2 = w2 - w1;
        double l0, r0, l1, r1_;
        reconstruct_fp64_g(lm, d0, d1, wm, w0, w1, l0, r0);
        reconstruct_fp64_g(lm, d1, d2, w0, w1, w2, l1, r1_);
        L[k] = l0;   // upper state of cell k0-1
        R[k] = r1_;  // lower state of cell k0
      }
      if (!perz && k0 == 1) {  // bottom wall: VL = flip(VR)
#pragma unroll
        for (int k = 0; k < NV; ++k) L[k] = ((a.bc_flip[4] >> rot_z(k)) & 1) ? -R[k] : R[k];
      }
      riemann_flux<double, 1, FLUX, true>(L, R, chd, gamma, r1, r2, Fo);
      double F[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) F[rot_z(k)] = Fo[k];
      const int gi = gi0 + tx, gj = gj0 + ty;
      if (resist && gi <= ix - 2 && gj <= jx - 2) {  // flux_resistive.cuf:121-135, face k0-1/2
        const int k = k0 - 1;
        auto B = [&](int var, int dxo, int dyo, int dzo) { return Wv(k + dzo, var, o + dxo + dyo * RX); };
        const double eta_dx = eta_of(3, tx + 1, k, gi, gj);
        const double JyS = (B(BX, 0, 0, 1) - B(BX, 0, 0, 0)) -
                           0.25 * (B(BZ, 1, 0, 0) + B(BZ, 1, 0, 1) - B(BZ, -1, 0, 0) - B(BZ, -1, 0, 1));
        const double JxS = -(B(BY, 0, 0, 1) - B(BY, 0, 0, 0)) +
                           0.25 * (B(BZ, 0, 1, 0) + B(BZ, 0, 1, 1) - B(BZ, 0, -1, 0) - B(BZ, 0, -1, 1));
        F[EN] = F[EN] + 0.5 * eta_dx * (JxS * (B(BY, 0, 0, 0) + B(BY, 0, 0, 1)) - JyS * (B(BX, 0, 0, 0) + B(BX, 0, 0, 1)));
        F[BX] = F[BX] - eta_dx * JyS;
        F[BY] = F[BY] + eta_dx * JxS;
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) Fzm[v * NCELL + c] = F[v];
    }
    const bool xwalls = !perx, ywalls = !pery;
    for (int i = 0; i < nplanes; ++i) {
      const int p = k0 + i, b = i & 1;
      const Buf m = buf_at(bufbase + (size_t)b * BUF);
      if (i >= 2) bar_sync(kBarEmpty + b, NTOT);  // consumers are done with plane p-2 (and its buffer)
      load_plane(a, W, p + 2, gi0, gj0, perx, pery, perz, resist, glmf, t, NP);
      bar_sync(kBarProd, NP);
      // positivity of plane p's own cells (3D_basic/u2v.f90:36-45)
      for (int c = t; c < NCELL; c += NP) {
        const int tx = c % TX, ty = c / TX, gi = gi0 + tx, gj = gj0 + ty;
        if (gi > ix - 2 || gj > jx - 2) continue;
        const int o = (ty + 2) * RX + (tx + 2);
        const double ro = Wv(p, RO, o), pr = Wv(p, PR, o);
        if (!gt0_<true>(pr))
          raise_error(a.err, OMHD_NEG_PRESSURE, gi + 1, gj + 1, p + 1, 0, pr);
        else if (!gt0_<true>(ro))
          raise_error(a.err, OMHD_NEG_DENSITY, gi + 1, gj + 1, p + 1, 0, ro);
      }
      // face states: x pairs (cells 2a, 2a+1 of a row), y pairs (cells 2a,
      // 2a+1 of a column), z pairs (cells p, p+1 of a column)
      constexpr int XP = XS / 2, NXP = NXS / 2, NYP = NYS / 2;
      const double* Wp = W + (size_t)ring_slot(p) * NV * PL;
      for (int q = t; q < NXP + NYP + NZF; q += NP) {
        if (q < NXP + NYP) {
          const bool xd = q < NXP;
          const int pp = xd ? q : q - NXP;
          const int ca = xd ? 2 * (pp % XP) : pp % TX, cb = xd ? pp / XP : 2 * (pp / TX);
          const int o = xd ? (cb + 2) * RX + (ca + 1) : (cb + 1) * RX + (ca + 2);
          const int stp = xd ? 1 : RX;
          const int i0 = xd ? cb * XS + ca : cb * TX + ca, di = xd ? 1 : TX;
          double* dl = xd ? m.SLx : m.SLy;
          double* dr = xd ? m.SRx : m.SRy;
          const int sv = xd ? NXS : NYS;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const double* w = Wp + v * PL + o;
            const double wm = w[-stp], w0 = w[0], w1 = w[stp], w2 = w[2 * stp];
            const double d0 = w0 - wm, d1 = w1 - w0, d2 = w2 - w1;
            double l0, r0, l1, r1_;
            reconstruct_fp64_g(lm, d0, d1, wm, w0, w1, l0, r0);
            reconstruct_fp64_g(lm, d1, d2, w0, w1, w2, l1, r1_);
            dl[v * sv + i0] = l0;
            dr[v * sv + i0] = r0;
            dl[v * sv + i0 + di] = l1;
            dr[v * sv + i0 + di] = r1_;
          }
        } else {
          const int c = q - NXP - NYP;
          const int tx = c % TX, ty = c / TX;
          const int o = (ty + 2) * RX + (tx + 2);
          const bool top = !perz && p == kx - 2;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const double wm = Wv(p - 1, v, o), w0 = Wv(p, v, o), w1 = Wv(p + 1, v, o), w2 = Wv(p + 2, v, o);
            const double d0 = w0 - wm, d1 = w1 - w0, d2 = w2 - w1;
            double l0, r0, l1, r1_;
            reconstruct_fp64_g(lm, d0, d1, wm, w0, w1, l0, r0);
            reconstruct_fp64_g(lm, d1, d2, w0, w1, w2, l1, r1_);
            m.SLz[v * NZF + c] = l0;  // upper state of cell p
            // lower state of cell p+1; at the top wall VR = flip(VL)
            m.SRz[v * NZF + c] = top ? (((a.bc_flip[5] >> v) & 1) ? -l0 : l0) : r1_;
          }
        }
      }
      if (xwalls || ywalls) {  // x walls (bc_for_F), y walls (bc_for_G)
        bar_sync(kBarProd, NP);
        for (int q = t; q < NV * (TY + TX); q += NP) {
          const int v = q / (TY + TX), r = q % (TY + TX);
          if (r < TY) {
            if (!xwalls) continue;
            const int cy = r;
            if (gi0 == 1) {
              const double s = m.SRx[v * NXS + cy * XS + 1];
              m.SLx[v * NXS + cy * XS + 0] = ((a.bc_flip[0] >> v) & 1) ? -s : s;
            }
            const int cl = (ix - 2) - gi0 + 1;
            if (cl >= 1 && cl <= TX) {
              const double s = m.SLx[v * NXS + cy * XS + cl];
              m.SRx[v * NXS + cy * XS + cl + 1] = ((a.bc_flip[1] >> v) & 1) ? -s : s;
            }
          } else {
            if (!ywalls) continue;
            const int cx = r - TY;
            if (gj0 == 1) {
              const double s = m.SRy[v * NYS + 1 * TX + cx];
              m.SLy[v * NYS + 0 * TX + cx] = ((a.bc_flip[2] >> v) & 1) ? -s : s;
            }
            const int cl = (jx - 2) - gj0 + 1;
            if (cl >= 1 && cl <= TY) {
              const double s = m.SLy[v * NYS + cl * TX + cx];
              m.SRy[v * NYS + (cl + 1) * TX + cx] = ((a.bc_flip[3] >> v) & 1) ? -s : s;
            }
          }
        }
      }
      __threadfence_block();
      bar_arrive(kBarFull + b, NP + NOWN);
      bar_arrive(kBarFullNon + b, NP + NNON);
    }
  } else {
    // ======================= consumers =======================
    const int t = threadIdx.x - NP;
    const double dtx = a.dtx_scale * dt / a.dx, dty = a.dtx_scale * dt / a.dy, dtz = a.dtx_scale * dt / a.dz;
    const double f1g = gamma - 1;
    for (int i = 0; i < nplanes; ++i) {
      const int p = k0 + i, b = i & 1;
      const Buf m = buf_at(bufbase + (size_t)b * BUF);
      if (t < NOWN)
        bar_sync(kBarFull + b, NP + NOWN);
      else
        bar_sync(kBarFullNon + b, NP + NNON);
      // ---- fluxes of the 136 x, 144 y and 128 z faces, x-oriented ----
      for (int q = t; q < NXF + NYF + NZF; q += NC) {
        const int dir = q < NXF ? 1 : (q < NXF + NYF ? 2 : 3);
        double* bl;
        const double* br;
        int sv;
        int fa, fb;  // x: (fx, cy); y: (cx, fy); z: (cell, -)
        if (dir == 1) {
          fa = q % (TX + 1), fb = q / (TX + 1);
          bl = m.SLx + fb * XS + fa;
          br = m.SRx + fb * XS + fa + 1;
          sv = NXS;
        } else if (dir == 2) {
          const int qq = q - NXF;
          fa = qq % TX, fb = qq / TX;
          bl = m.SLy + fb * TX + fa;
          br = m.SRy + (fb + 1) * TX + fa;
          sv = NYS;
        } else {
          fa = q - NXF - NYF, fb = 0;
          bl = m.SLz + fa;
          br = m.SRz + fa;
          sv = NZF;
        }
        double L[NV], R[NV], Fo[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const int v = dir == 1 ? k : (dir == 2 ? rot_y(k) : rot_z(k));
          L[k] = bl[v * sv];
          R[k] = br[v * sv];
        }
        riemann_flux<double, 1, FLUX, true>(L, R, chd, gamma, r1, r2, Fo);
        double F[NV];  // back to the grid's component order (constant indices: registers)
        if (dir == 1) {
#pragma unroll
          for (int k = 0; k < NV; ++k) F[k] = Fo[k];
        } else if (dir == 2) {
#pragma unroll
          for (int k = 0; k < NV; ++k) F[rot_y(k)] = Fo[k];
        } else {
#pragma unroll
          for (int k = 0; k < NV; ++k) F[rot_z(k)] = Fo[k];
        }
        if (resist) {
          if (dir == 1) {  // flux_resistive.cuf:87-101
            const int g = gi0 - 1 + fa, gj = gj0 + fb;
            if (g >= 0 && g <= ix - 2 && gj <= jx - 2) {
              const int o = (fb + 2) * RX + (fa + 1);
              auto B = [&](int var, int dxo, int dyo, int dzo) { return Wv(p + dzo, var, o + dxo + dyo * RX); };
              const double eta_dx = eta_of(1, fa, p, g, gj);
              const double JyS = -(B(BZ, 1, 0, 0) - B(BZ, 0, 0, 0)) +
                                 0.25 * (B(BX, 0, 0, 1) + B(BX, 1, 0, 1) - B(BX, 0, 0, -1) - B(BX, 1, 0, -1));
              const double JzS = (B(BY, 1, 0, 0) - B(BY, 0, 0, 0)) -
                                 0.25 * (B(BX, 0, 1, 0) + B(BX, 1, 1, 0) - B(BX, 0, -1, 0) - B(BX, 1, -1, 0));
              F[EN] = F[EN] + 0.5 * eta_dx * (JyS * (B(BZ, 0, 0, 0) + B(BZ, 1, 0, 0)) - JzS * (B(BY, 0, 0, 0) + B(BY, 1, 0, 0)));
              F[BY] = F[BY] - eta_dx * JzS;
              F[BZ] = F[BZ] + eta_dx * JyS;
            }
          } else if (dir == 2) {  // flux_resistive.cuf:104-118
            const int gii = gi0 + fa, g = gj0 - 1 + fb;
            if (g >= 0 && g <= jx - 2 && gii <= ix - 2) {
              const int o = (fb + 1) * RX + (fa + 2);
              auto B = [&](int var, int dxo, int dyo, int dzo) { return Wv(p + dzo, var, o + dxo + dyo * RX); };
              const double eta_dx = eta_of(2, fa + 1, p, gii, g);
              const double JxS = (B(BZ, 0, 1, 0) - B(BZ, 0, 0, 0)) -
                                 0.25 * (B(BY, 0, 0, 1) + B(BY, 0, 1, 1) - B(BY, 0, 0, -1) - B(BY, 0, 1, -1));
              const double JzS = -(B(BX, 0, 1, 0) - B(BX, 0, 0, 0)) +
                                 0.25 * (B(BY, 1, 0, 0) + B(BY, 1, 1, 0) - B(BY, -1, 0, 0) - B(BY, -1, 1, 0));
              F[EN] = F[EN] + 0.5 * eta_dx * (JzS * (B(BX, 0, 0, 0) + B(BX, 0, 1, 0)) - JxS * (B(BZ, 0, 0, 0) + B(BZ, 0, 1, 0)));
              F[BX] = F[BX] + eta_dx * JzS;
              F[BZ] = F[BZ] - eta_dx * JxS;
            }
          } else {  // flux_resistive.cuf:121-135, face p+1/2
            const int tx = fa % TX, ty = fa / TX, gi = gi0 + tx, gj = gj0 + ty;
            if (gi <= ix - 2 && gj <= jx - 2) {
              const int o = (ty + 2) * RX + (tx + 2);
              auto B = [&](int var, int dxo, int dyo, int dzo) { return Wv(p + dzo, var, o + dxo + dyo * RX); };
              const double eta_dx = eta_of(3, tx + 1, p, gi, gj);
              const double JyS = (B(BX, 0, 0, 1) - B(BX, 0, 0, 0)) -
                                 0.25 * (B(BZ, 1, 0, 0) + B(BZ, 1, 0, 1) - B(BZ, -1, 0, 0) - B(BZ, -1, 0, 1));
              const double JxS = -(B(BY, 0, 0, 1) - B(BY, 0, 0, 0)) +
                                 0.25 * (B(BZ, 0, 1, 0) + B(BZ, 0, 1, 1) - B(BZ, 0, -1, 0) - B(BZ, 0, -1, 1));
              F[EN] = F[EN] + 0.5 * eta_dx * (JxS * (B(BY, 0, 0, 0) + B(BY, 0, 0, 1)) - JyS * (B(BX, 0, 0, 0) + B(BX, 0, 0, 1)));
              F[BX] = F[BX] - eta_dx * JyS;
              F[BY] = F[BY] + eta_dx * JxS;
            }
          }
        }
        // the flux replaces the lower-cell face state, which only this face reads
#pragma unroll
        for (int v = 0; v < NV; ++v) bl[v * sv] = F[v];
      }
      // Only threads t < NCELL update cells.  The others have no further use of
      // this buffer: they signal both barriers without waiting (bar.arrive
      // counts toward the same totals) and go on to the next plane's faces,
      // which overlaps the update.
      if (t >= NOWN) {
        bar_arrive(kBarCons + b, NC);
        if (i + 2 < nplanes) {
          __threadfence_block();
          bar_arrive(kBarEmpty + b, NTOT);
        }
        continue;
      }
      bar_sync(kBarCons + b, NC);
      // ---- update plane p ----
      for (int c = t; c < NCELL; c += NC) {
        const int tx = c % TX, ty = c / TX;
        const int gi = gi0 + tx, gj = gj0 + ty;
        if (gi > ix - 2 || gj > jx - 2) continue;
        const size_t cc0 = (size_t)gi + (size_t)ix * ((size_t)gj + (size_t)jx * p);
        double out[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double acc = m.SLx[v * NXS + ty * XS + tx] - m.SLx[v * NXS + ty * XS + tx + 1];
          const double gm = m.SLy[v * NYS + ty * TX + tx], gp = m.SLy[v * NYS + (ty + 1) * TX + tx];
          const double fzm = Fzm[v * NCELL + c], fzp = m.SLz[v * NZF + c];
          Fzm[v * NCELL + c] = fzp;  // face p+1/2 is the next plane's lower face
          double d;
          if (a.iso)
            d = dtx * (acc + gm - gp + fzm - fzp);  // 3D_basic/rk.f90:26-35 order
          else
            d = dtx * acc + dty * (gm - gp) + dtz * (fzm - fzp);
          double ub = a.Ubase[v * N + cc0];
          if (v == PS) ub = glmf * ub;
          if (a.stage == 1 || a.time_type == OMHD_TIME_RK2)
            out[v] = ub + d;
          else
            out[v] = 0.5 * (ub + a.U1[v * N + cc0] + d);
        }
        if (a.stage == 2) out[PS] = glmf * out[PS];
        int xt[3], yt[3], zt[3], xf[3], yf[3], zf[3], nxt = 1, nyt = 1, nzt = 1;
        xt[0] = gi; xf[0] = 0; yt[0] = gj; yf[0] = 0; zt[0] = p; zf[0] = 0;
        if (gi == 1) { xt[nxt] = perx ? ix - 1 : 0; xf[nxt] = perx ? 0 : a.bc_flip[0]; ++nxt; }
        if (gi == ix - 2) { xt[nxt] = perx ? 0 : ix - 1; xf[nxt] = perx ? 0 : a.bc_flip[1]; ++nxt; }
        if (gj == 1) { yt[nyt] = pery ? jx - 1 : 0; yf[nyt] = pery ? 0 : a.bc_flip[2]; ++nyt; }
        if (gj == jx - 2) { yt[nyt] = pery ? 0 : jx - 1; yf[nyt] = pery ? 0 : a.bc_flip[3]; ++nyt; }
        if (p == 1) { zt[nzt] = perz ? kx - 1 : 0; zf[nzt] = perz ? 0 : a.bc_flip[4]; ++nzt; }
        if (p == kx - 2) { zt[nzt] = perz ? 0 : kx - 1; zf[nzt] = perz ? 0 : a.bc_flip[5]; ++nzt; }
        for (int e = 0; e < nzt; ++e)
          for (int bb = 0; bb < nyt; ++bb)
            for (int qx = 0; qx < nxt; ++qx) {
              const size_t cc = (size_t)xt[qx] + (size_t)ix * ((size_t)yt[bb] + (size_t)jx * zt[e]);
              const int fm = xf[qx] ^ yf[bb] ^ zf[e];
#pragma unroll
              for (int v = 0; v < NV; ++v) {
                const double o = ((fm >> v) & 1) ? -out[v] : out[v];
                a.Uout[v * N + cc] = o;
                if (a.Uhost) a.Uhost[v * N + cc] = o;  // result straight to host memory
              }
            }
        if (a.stage == 2) {  // 3D_basic/set_dt.f90:27-43 on the new state
          const double ro = out[RO];
          const double iro = rcp_<double, true>(ro);
          const double vx = divr_<double, true>(out[MX], ro, iro), vy = divr_<double, true>(out[MY], ro, iro),
                       vz = divr_<double, true>(out[MZ], ro, iro);
          const double rv2 = vx * out[MX] + vy * out[MY] + vz * out[MZ];
          const double B2 = out[BX] * out[BX] + out[BY] * out[BY] + out[BZ] * out[BZ];
          const double pr = f1g * (out[EN] - 0.5 * (rv2 + B2));
          const double f1 = gamma * pr;
          // fmax2 of the three speeds and of the running max, compared on the
          // integer pipe (same results)
          const double sx = fabs(vx) + fast_speed<double, true>(f1, B2, out[BX], ro);
          const double sy = fabs(vy) + fast_speed<double, true>(f1, B2, out[BY], ro);
          const double sz = fabs(vz) + fast_speed<double, true>(f1, B2, out[BZ], ro);
          double s = lt_<double, true>(sx, sy) ? sy : sx;
          s = lt_<double, true>(s, sz) ? sz : s;
          vmax = lt_<double, true>(s, vmax) ? vmax : s;
        }
      }
      if (i + 2 < nplanes) {  // the producers refill buffer b for plane p+2
        __threadfence_block();
        bar_arrive(kBarEmpty + b, NTOT);
      }
    }
  }
  if (a.stage == 2) {
    const double bm = block_max_pos(vmax, red32);
    StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
    reduce_and_finalize(st, sc, a.err, bm, gridDim.x * gridDim.y * gridDim.z, 1);
  }
}

template <int FLUX>
int launch_pipe3d(const StageArgs& a, cudaStream_t s) {
  const size_t bytes = smem_bytes();
  static std::atomic<unsigned long long> configured{0};
  const int r = set_smem_attr_once(k_stage3d_pipe<FLUX>, bytes, configured);
  if (r) return r;
  dim3 grid((a.ix - 2 + TX - 1) / TX, (a.jx - 2 + TY - 1) / TY, (a.kx - 2 + ZC - 1) / ZC);
  k_stage3d_pipe<FLUX><<<grid, NTOT, bytes, s>>>(a);
  return (int)cudaGetLastError();
}

}  // namespace d3p
}  // namespace OMHD_VARIANT
}  // namespace omhd
