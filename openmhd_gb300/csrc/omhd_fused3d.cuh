// omhd_fused3d.cuh -- one fused kernel per TVD-RK2 stage for 3D grids.
//
// A CTA owns a TX x TY column of interior cells and marches it through a
// chunk of z planes.  A ring of four primitive planes (k-1 .. k+2, each with
// a two-cell x/y halo) lives in shared memory, so the conserved->primitive
// recovery of every plane is done once per CTA; per plane the CTA
//   - loads and converts plane k+2 (u2v.f90, first GLM half in stage 1),
//   - builds x and y face states and fluxes of plane k in shared memory
//     (limiter.f90, flux_solver.f90, bc_for_F/G face fixes),
//   - reconstructs cell k+1 in z and solves the z face k+1/2 in registers,
//     carrying the z flux of face k-1/2 from the previous plane,
//   - updates plane k (rk.f90), fills ghosts by owner writes (bc),
//     applies the second GLM half and the CFL reduction in stage 2.
// Resistive fluxes (3D_reconnection_gpu/flux_resistive.cuf) are added at
// each face from cell-centred B in the ring.
#pragma once
#include "omhd_fused.h"
#include "omhd_step.cuh"

#ifndef OMHD_VARIANT
#error "define OMHD_VARIANT before including omhd_fused3d.cuh"
#endif

namespace omhd {
namespace OMHD_VARIANT {
namespace d3 {

// column of the one-role kernel (build-time constants, for tuning)
#ifndef OMHD_3D_TILE_X
#define OMHD_3D_TILE_X 32
#endif
#ifndef OMHD_3D_TILE_Y
#define OMHD_3D_TILE_Y 8
#endif
#ifndef OMHD_3D_MIXED_MIN_CTAS  // resident CTAs per SM the FP32-mixed 3D kernel is built for
#define OMHD_3D_MIXED_MIN_CTAS 2
#endif
constexpr int TX = OMHD_3D_TILE_X, TY = OMHD_3D_TILE_Y, NT = TX * TY;
static_assert(TY * NV <= NT - TX, "the x and y wall fixes use disjoint threads");
constexpr int RX = TX + 4, RY = TY + 4, PL = RX * RY;  // plane of the halo tile
constexpr int NRING = 4;
constexpr int XS = TX + 2, NXS3 = TY * XS;        // cells reconstructed in x (a row strip per tile row)
constexpr int NYS3 = (TY + 2) * TX;               // cells reconstructed in y
constexpr int XF = TX + 1, NXF3 = TY * XF;        // x faces
constexpr int NXFP3 = (NXF3 + 31) / 32 * 32;      // x faces padded to whole warps
constexpr int NYF3 = (TY + 1) * TX;               // y faces
constexpr int ZCHUNK = 64;  // z planes marched by one CTA

// ring of NRING primitive planes, then the x and y face states of one plane;
// each face's flux overwrites the lower-cell face state that only it reads
template <class T>
constexpr size_t smem3d_bytes() {
  return sizeof(T) * (size_t)NV * (NRING * PL + 2 * NXS3 + 2 * NYS3);
}

__device__ __forceinline__ int map_idx(int g, int n, bool periodic) {
  if (g >= 0 && g < n) return g;
  if (periodic) {
    const int P = n - 2;
    int r = (g - 1) % P;
    if (r < 0) r += P;
    return r + 1;
  }
  return g < 0 ? 0 : n - 1;
}

__device__ __forceinline__ double eta3(int kind, double x, double y, double z) {
  if (kind == OMHD_ETA_RECON2D) {  // 2D_reconnection/flux_resistive.f90:1-16 (as coded in the 3D GPU driver)
    const double Rm1 = 60.0, Rm0 = 1000.0;
    const double eta0 = 1.0 / Rm0;
    const double eta01 = (Rm0 - Rm1) / (Rm0 * Rm1);
    const double c = cosh(fmin2(sqrt(x * x + y * y), 25.0));
    return eta0 + eta01 * (1.0 / (c * c));
  }
  if (kind == OMHD_ETA_HARRIS_XZ) return 1.0e-3 + (1.0 / 60.0) * exp(-(x * x + z * z) / 4.0);
  return 0.0;
}

// eta / dx of the Harris resistivity, eta = 1e-3 + exp(-(x^2+z^2)/4)/60, from
// the factors ex = exp(-x^2/4) and ez = exp(-z^2/4), in the arithmetic type R
template <class R>
__device__ __forceinline__ R harris_eta_dx(R ex, R ez, R inv_dx) {
  return (R(1.0e-3) + R(1.0 / 60.0) * (ex * ez)) * inv_dx;
}

// Resistive terms of the FP32-mixed kernels (flux_resistive.cuf:87-135) in
// binary32, added to the binary32 face flux they belong to.  Each current
// component is a difference of cell-centred B across the face plus a quarter
// of a four-point transverse difference; the four-point sums are formed as two
// neighbour differences, which binary32 subtracts exactly when the neighbours
// are within a factor of two (Sterbenz), so the current keeps its relative
// precision where it is small.  b(var, dx, dy, dz) reads B of the cell at that
// offset from the face's lower cell; the face normal is axis n (1, 2, 3).
template <int n, class BF>
__device__ __forceinline__ void resist_face_f32(const BF& b, float eta_dx, float (&Fo)[NV]) {
  if constexpr (n == 1) {  // x face (:87-101)
    const float JyS = (b(BZ, 0, 0, 0) - b(BZ, 1, 0, 0)) +
                      0.25f * ((b(BX, 0, 0, 1) - b(BX, 0, 0, -1)) + (b(BX, 1, 0, 1) - b(BX, 1, 0, -1)));
    const float JzS = (b(BY, 1, 0, 0) - b(BY, 0, 0, 0)) -
                      0.25f * ((b(BX, 0, 1, 0) - b(BX, 0, -1, 0)) + (b(BX, 1, 1, 0) - b(BX, 1, -1, 0)));
    Fo[EN] += 0.5f * eta_dx * (JyS * (b(BZ, 0, 0, 0) + b(BZ, 1, 0, 0)) - JzS * (b(BY, 0, 0, 0) + b(BY, 1, 0, 0)));
    Fo[BY] -= eta_dx * JzS;
    Fo[BZ] += eta_dx * JyS;
  } else if constexpr (n == 2) {  // y face (:104-118)
    const float JxS = (b(BZ, 0, 1, 0) - b(BZ, 0, 0, 0)) -
                      0.25f * ((b(BY, 0, 0, 1) - b(BY, 0, 0, -1)) + (b(BY, 0, 1, 1) - b(BY, 0, 1, -1)));
    const float JzS = (b(BX, 0, 0, 0) - b(BX, 0, 1, 0)) +
                      0.25f * ((b(BY, 1, 0, 0) - b(BY, -1, 0, 0)) + (b(BY, 1, 1, 0) - b(BY, -1, 1, 0)));
    Fo[EN] += 0.5f * eta_dx * (JzS * (b(BX, 0, 0, 0) + b(BX, 0, 1, 0)) - JxS * (b(BZ, 0, 0, 0) + b(BZ, 0, 1, 0)));
    Fo[BX] += eta_dx * JzS;
    Fo[BZ] -= eta_dx * JxS;
  } else {  // z face (:121-135)
    const float JyS = (b(BX, 0, 0, 1) - b(BX, 0, 0, 0)) -
                      0.25f * ((b(BZ, 1, 0, 0) - b(BZ, -1, 0, 0)) + (b(BZ, 1, 0, 1) - b(BZ, -1, 0, 1)));
    const float JxS = (b(BY, 0, 0, 0) - b(BY, 0, 0, 1)) +
                      0.25f * ((b(BZ, 0, 1, 0) - b(BZ, 0, -1, 0)) + (b(BZ, 0, 1, 1) - b(BZ, 0, -1, 1)));
    Fo[EN] += 0.5f * eta_dx * (JxS * (b(BY, 0, 0, 0) + b(BY, 0, 0, 1)) - JyS * (b(BX, 0, 0, 0) + b(BX, 0, 0, 1)));
    Fo[BX] -= eta_dx * JyS;
    Fo[BY] += eta_dx * JxS;
  }
}

// Load + convert one z plane (global index gk, any value; mapped by the z bc)
// of the halo tile into ring slot `slot`.
template <class T>
__device__ __forceinline__ void load_plane(const StageArgs& a, T* W, int slot, int gk, int gi0, int gj0, bool perx,
                                           bool pery, bool perz, bool resist, double glmf, bool own_plane) {
  const int ix = a.ix, jx = a.jx, kx = a.kx;
  const size_t N = (size_t)ix * jx * kx;
  const double f1g = a.gm1;  // derived on the host
  const float f1g32 = a.gm1_f;
  const int mk = map_idx(gk, kx, perz);
  T* Ws = W + (size_t)slot * NV * PL;
  for (int q = threadIdx.x; q < PL; q += NT) {
    const int rx = q % RX, ry = q / RX;
    const bool cx_in = rx >= 2 && rx < TX + 2, cy_in = ry >= 2 && ry < TY + 2;
    if (!cx_in && !cy_in) {
      if (!resist || rx == 0 || rx == RX - 1 || ry == 0 || ry == RY - 1) continue;
    }
    const int gi = gi0 - 2 + rx, gj = gj0 - 2 + ry;
    const size_t c = (size_t)map_idx(gi, ix, perx) + (size_t)ix * ((size_t)map_idx(gj, jx, pery) + (size_t)jx * mk);
    const double* U = a.Uin;
    double u[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[v] = U[v * N + c];
    double ps = u[PS];
    if (a.stage == 1) ps = glmf * ps;
    T w[NV];
    double pr, ro;
    u2v_cell<T, OMHD_FAST>(u, f1g, f1g32, ps, w, pr, ro);  // 3D_basic/u2v.f90
#pragma unroll
    for (int v = 0; v < NV; ++v) Ws[v * PL + q] = w[v];
    if (own_plane && cx_in && cy_in && gi <= ix - 2 && gj <= jx - 2) {  // u2v.f90:36-45, owner check
      if (!(pr > 0.0))
        raise_error(a.err, OMHD_NEG_PRESSURE, gi + 1, gj + 1, gk + 1, 0, pr);
      else if (!(ro > 0.0))
        raise_error(a.err, OMHD_NEG_DENSITY, gi + 1, gj + 1, gk + 1, 0, ro);
    }
  }
}

// FP32 face arithmetic: two CTAs per SM (registers capped at 128, 97 KB of
// shared memory each), so that one CTA's FP64 loads, updates and barriers
// overlap the other's face work.
template <class T, int FLUX>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? OMHD_3D_MIXED_MIN_CTAS : 1) k_stage3d(const StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* W = reinterpret_cast<T*>(smem_raw);  // [NRING][NV][PL]
  T* SLx = W + NRING * NV * PL;  // [NV][NXS3]; x fluxes in place
  T* SRx = SLx + NV * NXS3;
  T* SLy = SRx + NV * NXS3;      // [NV][NYS3]; y fluxes in place
  T* SRy = SLy + NV * NYS3;
  __shared__ double red32[32];
  __shared__ int skip;

  StepState* st = a.st;
  // one thread decides, so that the whole CTA leaves together
  if (threadIdx.x == 0) skip = st->done || *(volatile int*)&a.err->code;
  __syncthreads();
  if (skip) return;
  const double dt = st->dt, chd = st->ch, glmf = st->glm_f;
  const int ix = a.ix, jx = a.jx, kx = a.kx;
  const size_t N = (size_t)ix * jx * kx;
  const int tid = threadIdx.x;
  const int gi0 = 1 + blockIdx.x * TX, gj0 = 1 + blockIdx.y * TY;
  const int k0 = 1 + blockIdx.z * ZCHUNK;
  const int k1 = min(k0 + ZCHUNK - 1, kx - 2);
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const bool perz = a.bc_kind[4] == OMHD_BC_PERIODIC;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const double gamma = a.gamma;
  // gamma constants derived on the host (stage_args_derived)
  const double f1g = a.gm1;
  const T ch = to_face<T>(chd);
  T gam, r1, r2;
  if constexpr (sizeof(T) == 4) {
    gam = a.gamma_f;
    r1 = a.r1_f;
    r2 = a.r2_f;
  } else {
    gam = gamma;
    r1 = a.r1;
    r2 = a.r2;
  }
  const int lm = a.lm_type;
  const int tx = tid % TX, ty = tid / TX;
  const int gi = gi0 + tx, gj = gj0 + ty;
  const bool own = gi <= ix - 2 && gj <= jx - 2;
  const int oc = (ty + 2) * RX + (tx + 2);  // own column in a ring plane
  // dt/dx as dt * (dtx_scale/dx) in the FAST builds (within an ulp), the
  // reference's division in the parity build
  const double dtx = OMHD_FAST ? dt * a.sdx : a.dtx_scale * dt / a.dx;
  const double dty = OMHD_FAST ? dt * a.sdy : a.dtx_scale * dt / a.dy;
  const double dtz = OMHD_FAST ? dt * a.sdz : a.dtx_scale * dt / a.dz;
  auto slot = [](int k) { return ((k % NRING) + NRING) % NRING; };
  auto Wv = [&](int k, int v, int o) -> T { return W[(size_t)slot(k) * NV * PL + v * PL + o]; };

  // The Harris resistivity is separable in x and z: in the FAST builds its
  // exponential is tabulated over this CTA's x columns (cell centres ex_c and
  // x faces ex_f, index q = i - gi0 + 1) and z chunk (ez_c, ez_f at z faces,
  // index p = k - k0 + 1), one exp per entry instead of one per face.
  __shared__ T ex_c[TX + 2], ex_f[TX + 2], ez_c[ZCHUNK + 2], ez_f[ZCHUNK + 2];
  const bool sep_eta = OMHD_FAST && a.eta_kind == OMHD_ETA_HARRIS_XZ;
  const double inv_dx = 1.0 / a.dx;
  const T inv_dx_t = T(inv_dx);
  if (sep_eta) {
    for (int q = tid; q < 2 * (TX + 2) + 2 * (ZCHUNK + 2); q += NT) {
      if (q < 2 * (TX + 2)) {
        const int p = q % (TX + 2);
        const double x = a.xc[min(gi0 - 1 + p, ix - 1)] + (q >= TX + 2 ? 0.5 * a.dx : 0.0);
        (q < TX + 2 ? ex_c : ex_f)[p] = to_face<T>(exp(-(x * x) / 4.0));
      } else {
        const int r = q - 2 * (TX + 2), p = r % (ZCHUNK + 2);
        const double z = a.zc[min(k0 - 1 + p, kx - 1)] + (r >= ZCHUNK + 2 ? 0.5 * a.dx : 0.0);
        (r < ZCHUNK + 2 ? ez_c : ez_f)[p] = to_face<T>(exp(-(z * z) / 4.0));
      }
    }
  }

  // ---- prologue: planes k0-2 .. k0+1, z face k0-1/2, cached upper state of cell k0 ----
  for (int p = k0 - 2; p <= k0 + 1; ++p)
    load_plane<T>(a, W, slot(p), p, gi0, gj0, perx, pery, perz, resist, glmf, p == k0);
  __syncthreads();
  T sLc[NV];  // z-upper face state of the current cell (k)
  double Fzp[NV];  // z flux through face k-1/2
  {
    T L[NV], R[NV], Fo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      T l, r;
      reconstruct_t<T, OMHD_FAST>(lm, Wv(k0 - 2, v, oc), Wv(k0 - 1, v, oc), Wv(k0, v, oc), l, r);
      L[v] = l;  // upper state of cell k0-1
      reconstruct_t<T, OMHD_FAST>(lm, Wv(k0 - 1, v, oc), Wv(k0, v, oc), Wv(k0 + 1, v, oc), l, r);
      R[v] = r;  // lower state of cell k0
      sLc[v] = l;
    }
    if (!perz && k0 == 1) {  // bottom wall: VL = flip(VR)  (3D_reconnection_gpu/bc.cuf bc_for_H pattern)
#pragma unroll
      for (int v = 0; v < NV; ++v) L[v] = ((a.bc_flip[4] >> v) & 1) ? -R[v] : R[v];
    }
    riemann_flux<T, 3, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
#pragma unroll
    for (int v = 0; v < NV; ++v) Fzp[v] = to_f64<T>(Fo[v]);
    if (resist && own) {  // z face k0-1/2 (flux_resistive.cuf:121-135)
      const int k = k0 - 1;
      if constexpr (sizeof(T) == 4) {
        auto b = [&](int var, int dxo, int dyo, int dzo) { return Wv(k + dzo, var, oc + dxo + dyo * RX); };
        const float eta_dx = sep_eta ? harris_eta_dx<T>(ex_c[tx + 1], ez_f[0], inv_dx_t)
                                     : narrow_f64(eta3(a.eta_kind, a.xc[gi], a.yc[gj], a.zc[k] + 0.5 * a.dx) / a.dx);
        resist_face_f32<3>(b, eta_dx, Fo);
#pragma unroll
        for (int v = 0; v < NV; ++v) Fzp[v] = to_f64<T>(Fo[v]);
      } else {
        auto B = [&](int var, int dxo, int dyo, int dzo) { return to_f64<T>(Wv(k + dzo, var, oc + dxo + dyo * RX)); };
        const double eta_dx = sep_eta ? harris_eta_dx<double>(ex_c[tx + 1], ez_f[0], inv_dx)
                                      : eta3(a.eta_kind, a.xc[gi], a.yc[gj], a.zc[k] + 0.5 * a.dx) / a.dx;
        const double JyS = (B(BX, 0, 0, 1) - B(BX, 0, 0, 0)) -
                           0.25 * (B(BZ, 1, 0, 0) + B(BZ, 1, 0, 1) - B(BZ, -1, 0, 0) - B(BZ, -1, 0, 1));
        const double JxS = -(B(BY, 0, 0, 1) - B(BY, 0, 0, 0)) +
                           0.25 * (B(BZ, 0, 1, 0) + B(BZ, 0, 1, 1) - B(BZ, 0, -1, 0) - B(BZ, 0, -1, 1));
        Fzp[EN] = Fzp[EN] + 0.5 * eta_dx * (JxS * (B(BY, 0, 0, 0) + B(BY, 0, 0, 1)) - JyS * (B(BX, 0, 0, 0) + B(BX, 0, 0, 1)));
        Fzp[BX] = Fzp[BX] - eta_dx * JyS;
        Fzp[BY] = Fzp[BY] + eta_dx * JxS;
      }
    }
  }
  double vloc = 0.0;

  for (int k = k0; k <= k1; ++k) {
    // Three CTA barriers per plane (plus one where a wall fix is needed).  The
    // ring slot of plane k+2 held plane k-2, whose last readers (the resistive
    // terms of plane k-1) finished before the previous plane's flux barrier;
    // the face arrays are rewritten only after the barrier that follows this
    // load, which every thread reaches after its reads of the previous plane's
    // fluxes.  The prologue's z face reads plane k0-2: one barrier before the
    // first load.
    if (k == k0) __syncthreads();
    load_plane<T>(a, W, slot(k + 2), k + 2, gi0, gj0, perx, pery, perz, resist, glmf, false);
    __syncthreads();
    if (k > k0) {
      // positivity of the current plane's own cells (u2v.f90:36-45); plane k0
      // was checked at load time in the prologue
      if (own) {
        const double ro = to_f64<T>(Wv(k, RO, oc)), pr = to_f64<T>(Wv(k, PR, oc));
        if (pr <= 0)
          raise_error(a.err, OMHD_NEG_PRESSURE, gi + 1, gj + 1, k + 1, 0, pr);
        else if (ro <= 0)
          raise_error(a.err, OMHD_NEG_DENSITY, gi + 1, gj + 1, k + 1, 0, ro);
      }
    }
    const T* Wk = W + (size_t)slot(k) * NV * PL;

    // ---- x and y face states of plane k, one phase ----
    for (int q = tid; q < NXS3 + NYS3; q += NT) {
      const bool xd = q < NXS3;
      const int qq = xd ? q : q - NXS3;
      int o, st;
      if (xd) {  // x row cy, cells cx = 0..TX+1 (tile columns -1..TX)
        const int cx = qq % XS, cy = qq / XS;
        o = (cy + 2) * RX + (cx + 1);
        st = 1;
      } else {  // y column cx, cells cy = 0..TY+1 (tile rows -1..TY)
        const int cx = qq % TX, cy = qq / TX;
        o = (cy + 1) * RX + (cx + 2);
        st = RX;
      }
      T* dl = xd ? SLx : SLy;
      T* dr = xd ? SRx : SRy;
      const int sv = xd ? NXS3 : NYS3;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        T l, r;
        reconstruct_t<T, OMHD_FAST>(lm, Wk[v * PL + o - st], Wk[v * PL + o], Wk[v * PL + o + st], l, r);
        dl[v * sv + qq] = l;
        dr[v * sv + qq] = r;
      }
    }
    __syncthreads();
    if (!perx || !pery) {  // wall face fixes, x by the first threads, y by the last
      if (!perx && tid < TY * NV) {
        const int cy = tid % TY, v = tid / TY;
        if (gi0 == 1) {
          const T s = SRx[v * NXS3 + cy * XS + 1];
          SLx[v * NXS3 + cy * XS + 0] = ((a.bc_flip[0] >> v) & 1) ? -s : s;
        }
        const int cl = (ix - 2) - gi0 + 1;
        if (cl >= 1 && cl <= TX) {
          const T s = SLx[v * NXS3 + cy * XS + cl];
          SRx[v * NXS3 + cy * XS + cl + 1] = ((a.bc_flip[1] >> v) & 1) ? -s : s;
        }
      }
      if (!pery && tid >= NT - TX) {
        const int cx = tid - (NT - TX);
        const int cl = (jx - 2) - gj0 + 1;
        for (int v = 0; v < NV; ++v) {
          if (gj0 == 1) {
            const T s = SRy[v * NYS3 + 1 * TX + cx];
            SLy[v * NYS3 + 0 * TX + cx] = ((a.bc_flip[2] >> v) & 1) ? -s : s;
          }
          if (cl >= 1 && cl <= TY) {
            const T s = SLy[v * NYS3 + cl * TX + cx];
            SRy[v * NYS3 + (cl + 1) * TX + cx] = ((a.bc_flip[3] >> v) & 1) ? -s : s;
          }
        }
      }
      __syncthreads();
    }

    // ---- x and y fluxes of plane k, one phase (x faces padded to whole
    // warps, so that no warp mixes directions); each flux replaces the
    // lower-cell face state that only its own face reads ----
    for (int q = tid; q < NXFP3 + NYF3; q += NT) {
      if (q < NXFP3) {
        if (q >= NXF3) continue;  // padding lanes
        const int fx = q % XF, cy = q / XF;
        T L[NV], R[NV], Fo[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          L[v] = SLx[v * NXS3 + cy * XS + fx];
          R[v] = SRx[v * NXS3 + cy * XS + fx + 1];
        }
        riemann_flux<T, 1, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
        if (resist) {  // flux_resistive.cuf:87-101
          const int g = gi0 - 1 + fx, gjj = gj0 + cy;
          if (g >= 0 && g <= ix - 2 && gjj <= jx - 2) {
            const int o = (cy + 2) * RX + (fx + 1);
            if constexpr (sizeof(T) == 4) {
              auto b = [&](int var, int dxo, int dyo, int dzo) { return Wv(k + dzo, var, o + dxo + dyo * RX); };
              const float eta_dx = sep_eta ? harris_eta_dx<T>(ex_f[fx], ez_c[k - k0 + 1], inv_dx_t)
                                           : narrow_f64(eta3(a.eta_kind, a.xc[g] + 0.5 * a.dx, a.yc[gjj], a.zc[k]) / a.dx);
              resist_face_f32<1>(b, eta_dx, Fo);
            } else {
              auto B = [&](int var, int dxo, int dyo, int dzo) { return to_f64<T>(Wv(k + dzo, var, o + dxo + dyo * RX)); };
              const double eta_dx = sep_eta ? harris_eta_dx<double>(ex_f[fx], ez_c[k - k0 + 1], inv_dx)
                                            : eta3(a.eta_kind, a.xc[g] + 0.5 * a.dx, a.yc[gjj], a.zc[k]) / a.dx;
              const double JyS = -(B(BZ, 1, 0, 0) - B(BZ, 0, 0, 0)) +
                                 0.25 * (B(BX, 0, 0, 1) + B(BX, 1, 0, 1) - B(BX, 0, 0, -1) - B(BX, 1, 0, -1));
              const double JzS = (B(BY, 1, 0, 0) - B(BY, 0, 0, 0)) -
                                 0.25 * (B(BX, 0, 1, 0) + B(BX, 1, 1, 0) - B(BX, 0, -1, 0) - B(BX, 1, -1, 0));
              Fo[EN] = Fo[EN] + 0.5 * eta_dx * (JyS * (B(BZ, 0, 0, 0) + B(BZ, 1, 0, 0)) - JzS * (B(BY, 0, 0, 0) + B(BY, 1, 0, 0)));
              Fo[BY] = Fo[BY] - eta_dx * JzS;
              Fo[BZ] = Fo[BZ] + eta_dx * JyS;
            }
          }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) SLx[v * NXS3 + cy * XS + fx] = Fo[v];
      } else {
        const int qq = q - NXFP3;
        const int cx = qq % TX, fy = qq / TX;
        T L[NV], R[NV], Fo[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          L[v] = SLy[v * NYS3 + fy * TX + cx];
          R[v] = SRy[v * NYS3 + (fy + 1) * TX + cx];
        }
        riemann_flux<T, 2, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
        if (resist) {  // flux_resistive.cuf:104-118
          const int gii = gi0 + cx, g = gj0 - 1 + fy;
          if (g >= 0 && g <= jx - 2 && gii <= ix - 2) {
            const int o = (fy + 1) * RX + (cx + 2);
            if constexpr (sizeof(T) == 4) {
              auto b = [&](int var, int dxo, int dyo, int dzo) { return Wv(k + dzo, var, o + dxo + dyo * RX); };
              const float eta_dx = sep_eta ? harris_eta_dx<T>(ex_c[cx + 1], ez_c[k - k0 + 1], inv_dx_t)
                                           : narrow_f64(eta3(a.eta_kind, a.xc[gii], a.yc[g] + 0.5 * a.dx, a.zc[k]) / a.dx);
              resist_face_f32<2>(b, eta_dx, Fo);
            } else {
              auto B = [&](int var, int dxo, int dyo, int dzo) { return to_f64<T>(Wv(k + dzo, var, o + dxo + dyo * RX)); };
              const double eta_dx = sep_eta ? harris_eta_dx<double>(ex_c[cx + 1], ez_c[k - k0 + 1], inv_dx)
                                            : eta3(a.eta_kind, a.xc[gii], a.yc[g] + 0.5 * a.dx, a.zc[k]) / a.dx;
              const double JxS = (B(BZ, 0, 1, 0) - B(BZ, 0, 0, 0)) -
                                 0.25 * (B(BY, 0, 0, 1) + B(BY, 0, 1, 1) - B(BY, 0, 0, -1) - B(BY, 0, 1, -1));
              const double JzS = -(B(BX, 0, 1, 0) - B(BX, 0, 0, 0)) +
                                 0.25 * (B(BY, 1, 0, 0) + B(BY, 1, 1, 0) - B(BY, -1, 0, 0) - B(BY, -1, 1, 0));
              Fo[EN] = Fo[EN] + 0.5 * eta_dx * (JzS * (B(BX, 0, 0, 0) + B(BX, 0, 1, 0)) - JxS * (B(BZ, 0, 0, 0) + B(BZ, 0, 1, 0)));
              Fo[BX] = Fo[BX] + eta_dx * JzS;
              Fo[BZ] = Fo[BZ] - eta_dx * JxS;
            }
          }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) SLy[v * NYS3 + fy * TX + cx] = Fo[v];
      }
    }
    // ---- z face k+1/2 in registers: it reads only the ring, so the FP64 build
    // solves it before the flux barrier (threads with no face left in the last
    // round of x/y faces solve their z face meanwhile: 1 % faster on Harris
    // 512x256x512); the FP32 build, after the barrier (3 % faster there) ----
    double Fzc[NV];
    T sLn[NV];
    auto z_face = [&]() {
      T L[NV], R[NV], Fo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        T l, r;
        reconstruct_t<T, OMHD_FAST>(lm, Wv(k, v, oc), Wv(k + 1, v, oc), Wv(k + 2, v, oc), l, r);
        L[v] = sLc[v];
        R[v] = r;
        sLn[v] = l;
      }
      if (!perz && k == kx - 2) {  // top wall: VR = flip(VL)
#pragma unroll
        for (int v = 0; v < NV; ++v) R[v] = ((a.bc_flip[5] >> v) & 1) ? -L[v] : L[v];
      }
      riemann_flux<T, 3, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
#pragma unroll
      for (int v = 0; v < NV; ++v) Fzc[v] = to_f64<T>(Fo[v]);
      if (resist && own) {  // flux_resistive.cuf:121-135
        if constexpr (sizeof(T) == 4) {
          auto b = [&](int var, int dxo, int dyo, int dzo) { return Wv(k + dzo, var, oc + dxo + dyo * RX); };
          const float eta_dx = sep_eta ? harris_eta_dx<T>(ex_c[tx + 1], ez_f[k - k0 + 1], inv_dx_t)
                                       : narrow_f64(eta3(a.eta_kind, a.xc[gi], a.yc[gj], a.zc[k] + 0.5 * a.dx) / a.dx);
          resist_face_f32<3>(b, eta_dx, Fo);
#pragma unroll
          for (int v = 0; v < NV; ++v) Fzc[v] = to_f64<T>(Fo[v]);
        } else {
          auto B = [&](int var, int dxo, int dyo, int dzo) { return to_f64<T>(Wv(k + dzo, var, oc + dxo + dyo * RX)); };
          const double eta_dx = sep_eta ? harris_eta_dx<double>(ex_c[tx + 1], ez_f[k - k0 + 1], inv_dx)
                                        : eta3(a.eta_kind, a.xc[gi], a.yc[gj], a.zc[k] + 0.5 * a.dx) / a.dx;
          const double JyS = (B(BX, 0, 0, 1) - B(BX, 0, 0, 0)) -
                             0.25 * (B(BZ, 1, 0, 0) + B(BZ, 1, 0, 1) - B(BZ, -1, 0, 0) - B(BZ, -1, 0, 1));
          const double JxS = -(B(BY, 0, 0, 1) - B(BY, 0, 0, 0)) +
                             0.25 * (B(BZ, 0, 1, 0) + B(BZ, 0, 1, 1) - B(BZ, 0, -1, 0) - B(BZ, 0, -1, 1));
          Fzc[EN] = Fzc[EN] + 0.5 * eta_dx * (JxS * (B(BY, 0, 0, 0) + B(BY, 0, 0, 1)) - JyS * (B(BX, 0, 0, 0) + B(BX, 0, 0, 1)));
          Fzc[BX] = Fzc[BX] - eta_dx * JyS;
          Fzc[BY] = Fzc[BY] + eta_dx * JxS;
        }
      }
    };
    if constexpr (sizeof(T) == 8) z_face();

    __syncthreads();
    double acc[NV], gm[NV], gp[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      acc[v] = to_f64<T>(SLx[v * NXS3 + ty * XS + tx]) - to_f64<T>(SLx[v * NXS3 + ty * XS + tx + 1]);
      gm[v] = to_f64<T>(SLy[v * NYS3 + ty * TX + tx]);
      gp[v] = to_f64<T>(SLy[v * NYS3 + (ty + 1) * TX + tx]);
    }
    if constexpr (sizeof(T) == 4) z_face();

    // ---- update plane k ----
    if (own) {
      const size_t c = (size_t)gi + (size_t)ix * ((size_t)gj + (size_t)jx * k);
      double out[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double d;
        if (a.iso)
          d = dtx * (acc[v] + gm[v] - gp[v] + Fzp[v] - Fzc[v]);  // 3D_basic/rk.f90:26-35 order
        else
          d = dtx * acc[v] + dty * (gm[v] - gp[v]) + dtz * (Fzp[v] - Fzc[v]);
        double ub = a.Ubase[v * N + c];
        if (v == PS) ub = glmf * ub;
        if (a.stage == 1 || a.time_type == OMHD_TIME_RK2)
          out[v] = ub + d;
        else
          out[v] = 0.5 * (ub + a.U1[v * N + c] + d);
      }
      if (a.stage == 2) out[PS] = glmf * out[PS];
      int xt[3], yt[3], zt[3], xf[3], yf[3], zf[3], nxt = 1, nyt = 1, nzt = 1;
      xt[0] = gi; xf[0] = 0; yt[0] = gj; yf[0] = 0; zt[0] = k; zf[0] = 0;
      if (gi == 1) { xt[nxt] = perx ? ix - 1 : 0; xf[nxt] = perx ? 0 : a.bc_flip[0]; ++nxt; }
      if (gi == ix - 2) { xt[nxt] = perx ? 0 : ix - 1; xf[nxt] = perx ? 0 : a.bc_flip[1]; ++nxt; }
      if (gj == 1) { yt[nyt] = pery ? jx - 1 : 0; yf[nyt] = pery ? 0 : a.bc_flip[2]; ++nyt; }
      if (gj == jx - 2) { yt[nyt] = pery ? 0 : jx - 1; yf[nyt] = pery ? 0 : a.bc_flip[3]; ++nyt; }
      if (k == 1) { zt[nzt] = perz ? kx - 1 : 0; zf[nzt] = perz ? 0 : a.bc_flip[4]; ++nzt; }
      if (k == kx - 2) { zt[nzt] = perz ? 0 : kx - 1; zf[nzt] = perz ? 0 : a.bc_flip[5]; ++nzt; }
      for (int e = 0; e < nzt; ++e)
        for (int b = 0; b < nyt; ++b)
          for (int q = 0; q < nxt; ++q) {
            const size_t cc = (size_t)xt[q] + (size_t)ix * ((size_t)yt[b] + (size_t)jx * zt[e]);
            const int fm = xf[q] ^ yf[b] ^ zf[e];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              const double o = ((fm >> v) & 1) ? -out[v] : out[v];
              a.Uout[v * N + cc] = o;
              if (a.Uhost) a.Uhost[v * N + cc] = o;  // result straight to host memory
            }
          }
      if (a.stage == 2) {  // 3D_basic/set_dt.f90:27-43 on the new state
        const double ro = out[RO];
        const double iro = rcp_<double, OMHD_FAST>(ro);  // one reciprocal for the three velocities
        const double vx = divr_<double, OMHD_FAST>(out[MX], ro, iro), vy = divr_<double, OMHD_FAST>(out[MY], ro, iro), vz = divr_<double, OMHD_FAST>(out[MZ], ro, iro);
        const double rv2 = vx * out[MX] + vy * out[MY] + vz * out[MZ];
        const double B2 = out[BX] * out[BX] + out[BY] * out[BY] + out[BZ] * out[BZ];
        const double pr = f1g * (out[EN] - 0.5 * (rv2 + B2));
        const double f1 = gamma * pr;
        // fmax2 of the three speeds and of the running max, the comparisons on
        // the integer pipe in the FAST builds (same results)
        const double sx = fabs(vx) + fast_speed<double, OMHD_FAST>(f1, B2, out[BX], ro);
        const double sy = fabs(vy) + fast_speed<double, OMHD_FAST>(f1, B2, out[BY], ro);
        const double sz = fabs(vz) + fast_speed<double, OMHD_FAST>(f1, B2, out[BZ], ro);
        double s = lt_<double, OMHD_FAST>(sx, sy) ? sy : sx;
        s = lt_<double, OMHD_FAST>(s, sz) ? sz : s;
        vloc = lt_<double, OMHD_FAST>(s, vloc) ? vloc : s;
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      Fzp[v] = Fzc[v];
      sLc[v] = sLn[v];
    }
  }
  if (a.stage == 2) {
    const double bm = block_max_pos(vloc, red32);
    StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
    reduce_and_finalize(st, sc, a.err, bm, gridDim.x * gridDim.y * gridDim.z, 1);
  }
}

template <class T, int FLUX>
int launch_one3d(const StageArgs& a, cudaStream_t s) {
  const size_t bytes = smem3d_bytes<T>();
  static std::atomic<unsigned long long> configured{0};
  const int r = set_smem_attr_once(k_stage3d<T, FLUX>, bytes, configured);
  if (r) return r;
  dim3 grid((a.ix - 2 + TX - 1) / TX, (a.jx - 2 + TY - 1) / TY, (a.kx - 2 + ZCHUNK - 1) / ZCHUNK);
  k_stage3d<T, FLUX><<<grid, NT, bytes, s>>>(a);
  return (int)cudaGetLastError();
}

template <class T>
int launch_variant3d(const StageArgs& a, cudaStream_t s) {
  switch (a.flux_type) {
    case FX_LLF: return launch_one3d<T, FX_LLF>(a, s);
    case FX_HLL: return launch_one3d<T, FX_HLL>(a, s);
    case FX_HLLC: return launch_one3d<T, FX_HLLC>(a, s);
    case FX_HLLD: return launch_one3d<T, FX_HLLD>(a, s);
    default: return launch_one3d<T, FX_LHLLD>(a, s);
  }
}

}  // namespace d3
}  // namespace OMHD_VARIANT
}  // namespace omhd
