// omhd_fused2d.cuh -- one fused kernel per TVD-RK2 stage for 2D grids.
//
// A CTA owns a TX x TY tile of interior cells and stages the tile plus a
// two-cell halo of the state in shared memory.  Inside the CTA:
//   A  load + conserved->primitive recovery (u2v.f90) of the halo tile,
//      stage 1 applies the first GLM half (glm_ss2.f90) on the fly;
//   B  x-direction slope limiting (limiter.f90) -> face states, wall fix;
//   C  x-face Riemann fluxes (flux_solver.f90) [+ resistive terms];
//   D  x flux differences kept in registers (FP64);
//   E/F the same in y;
//   G  Runge-Kutta update (rk.f90), ghost-cell fill by the owner of each
//      source cell (bc.f90), stage 2 applies the second GLM half and reduces
//      the next step's CFL speed (set_dt.f90); the last CTA plans the next
//      step on the device.
// Per stage this reads the state once (plus halo) and writes it once: the
// face states and fluxes of the reference (VL, VR, F, G) never reach HBM.
//
// Included by one translation unit per arithmetic variant; OMHD_VARIANT names
// the namespace so that instantiations built with different floating-point
// flags never collide at link time.
#pragma once
#include "omhd_fused.h"
#include "omhd_step.cuh"

#ifndef OMHD_VARIANT
#error "define OMHD_VARIANT before including omhd_fused2d.cuh"
#endif

namespace omhd {
namespace OMHD_VARIANT {

constexpr int TX = 32, TY = 8, NT = TX * TY;
constexpr int RX = TX + 4, RY = TY + 4;
constexpr int SFACE = (TY * (TX + 2) > (TY + 2) * TX) ? TY * (TX + 2) : (TY + 2) * TX;
constexpr int SFLUX = (TY * (TX + 1) > (TY + 1) * TX) ? TY * (TX + 1) : (TY + 1) * TX;

template <class T>
constexpr size_t smem2d_bytes() {
  return sizeof(T) * (size_t)NV * (RY * RX + 2 * SFACE + SFLUX);
}

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

template <class T, int FLUX>
__global__ void __launch_bounds__(NT) k_stage2d(const StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* W = reinterpret_cast<T*>(smem_raw);  // [NV][RY][RX] primitive halo tile
  T* SL = W + NV * RY * RX;               // [NV][SFACE] upper-face states of cells
  T* SR = SL + NV * SFACE;                // [NV][SFACE] lower-face states of cells
  T* FB = SR + NV * SFACE;                // [NV][SFLUX] face fluxes
  __shared__ double red32[32];

  StepState* st = a.st;
  if (st->done || *(volatile int*)&a.err->code) return;
  const double dt = st->dt, chd = st->ch, glmf = st->glm_f;
  const int ix = a.ix, jx = a.jx;
  const size_t N = (size_t)ix * jx;
  const int tid = threadIdx.x;
  const int gi0 = 1 + blockIdx.x * TX, gj0 = 1 + blockIdx.y * TY;
  const bool perx = a.bc_kind[0] == OMHD_BC_PERIODIC, pery = a.bc_kind[2] == OMHD_BC_PERIODIC;
  const bool resist = a.eta_kind != OMHD_ETA_NONE;
  const double gamma = a.gamma;
  const double f1g = gamma - 1;  // u2v.f90:11
  const T ch = T(chd), gam = T(gamma);
  const T r1 = T(1.0 / (gamma - 1.0)), r2 = T(gamma / (gamma - 1.0));
  const int lm = a.lm_type;

  // ---- A: halo tile load + u2v (+ first GLM half in stage 1) ----
  for (int q = tid; q < RX * RY; q += NT) {
    const int rx = q % RX, ry = q / RX;
    const bool cx_in = rx >= 2 && rx < TX + 2, cy_in = ry >= 2 && ry < TY + 2;
    if (!cx_in && !cy_in) {
      // corners: only the diagonal neighbours are needed, by the resistive terms
      if (!resist || rx == 0 || rx == RX - 1 || ry == 0 || ry == RY - 1) continue;
    }
    const int gi = gi0 - 2 + rx, gj = gj0 - 2 + ry;
    const size_t c = (size_t)map_index(gi, ix, perx) + (size_t)ix * map_index(gj, jx, pery);
    const double* U = a.Uin;
    const double ro = U[RO * N + c];
    const double mx = U[MX * N + c], my = U[MY * N + c], mz = U[MZ * N + c];
    const double vx = div_<double, OMHD_FAST>(mx, ro), vy = div_<double, OMHD_FAST>(my, ro),
                 vz = div_<double, OMHD_FAST>(mz, ro);  // u2v.f90:24
    const double rv2 = vx * mx + vy * my + vz * mz;
    const double bx = U[BX * N + c], by = U[BY * N + c], bz = U[BZ * N + c];
    const double B2 = bx * bx + by * by + bz * bz;
    const double pr = f1g * (U[EN * N + c] - 0.5 * (rv2 + B2));  // u2v.f90:27
    double ps = U[PS * N + c];
    if (a.stage == 1) ps = glmf * ps;
    const int o = ry * RX + rx;
    W[VX * RY * RX + o] = T(vx);
    W[VY * RY * RX + o] = T(vy);
    W[VZ * RY * RX + o] = T(vz);
    W[PR * RY * RX + o] = T(pr);
    W[RO * RY * RX + o] = T(ro);
    W[BX * RY * RX + o] = T(bx);
    W[BY * RY * RX + o] = T(by);
    W[BZ * RY * RX + o] = T(bz);
    W[PS * RY * RX + o] = T(ps);
    if (cx_in && cy_in && gi <= ix - 2 && gj <= jx - 2) {  // owner check, u2v.f90:36-45
      if (pr <= 0)
        raise_error(a.err, OMHD_NEG_PRESSURE, gi + 1, gj + 1, 0, 0, pr);
      else if (ro <= 0)
        raise_error(a.err, OMHD_NEG_DENSITY, gi + 1, gj + 1, 0, 0, ro);
    }
  }
  __syncthreads();

  // ---- B: x slopes for cells rx = 1 .. TX+2 on tile rows ----
  constexpr int XS = TX + 2;  // face-state row length in the x pass
  for (int q = tid; q < TY * XS; q += NT) {
    const int cx = q % XS, cy = q / XS;
    const int o = (cy + 2) * RX + (cx + 1);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      T l, r;
      reconstruct<T>(lm, W[v * RY * RX + o - 1], W[v * RY * RX + o], W[v * RY * RX + o + 1], l, r);
      SL[v * SFACE + q] = l;
      SR[v * SFACE + q] = r;
    }
  }
  __syncthreads();
  // wall face fix (2D_KH/bc.f90:42-51 pattern; 2D_reconnection/bc.f90:136-165)
  if (!perx) {
    if (gi0 == 1 && tid < TY * NV) {  // west face: VL = flip(VR)
      const int cy = tid % TY, v = tid / TY;
      const T s = SR[v * SFACE + cy * XS + 1];
      SL[v * SFACE + cy * XS + 0] = ((a.bc_flip[0] >> v) & 1) ? -s : s;
    }
    const int cl = (ix - 2) - gi0 + 1;  // cx of the last interior cell
    if (cl >= 1 && cl <= TX && tid < TY * NV) {  // east face: VR = flip(VL)
      const int cy = tid % TY, v = tid / TY;
      const T s = SL[v * SFACE + cy * XS + cl];
      SR[v * SFACE + cy * XS + cl + 1] = ((a.bc_flip[1] >> v) & 1) ? -s : s;
    }
    __syncthreads();
  }

  // ---- C: x-face fluxes ----
  constexpr int XF = TX + 1;
  for (int q = tid; q < TY * XF; q += NT) {
    const int fx = q % XF, cy = q / XF;
    T L[NV], R[NV], Fo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      L[v] = SL[v * SFACE + cy * XS + fx];
      R[v] = SR[v * SFACE + cy * XS + fx + 1];
    }
    riemann_flux<T, 1, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
    if (resist) {  // 2D_reconnection/flux_resistive.f90:266-283
      const int g = gi0 - 1 + fx, gj = gj0 + cy;
      if (g >= 0 && g <= ix - 2 && gj <= jx - 2) {
        const int o = (cy + 2) * RX + (fx + 1);  // region index of cell g
        auto B = [&](int var, int dxo, int dyo) { return double(W[var * RY * RX + o + dxo + dyo * RX]); };
        const double odx = 1.0 / a.dx;
        const double eta_dx = eta_at(a.eta_kind, a.xc[g] + 0.5 * a.dx, a.yc[gj], 0.0) * odx;
        const double JyS = -eta_dx * (B(BZ, 1, 0) - B(BZ, 0, 0));
        const double JzS = eta_dx * ((B(BY, 1, 0) - B(BY, 0, 0)) -
                                     0.25 * (B(BX, 0, 1) + B(BX, 1, 1) - B(BX, 0, -1) - B(BX, 1, -1)));
        Fo[EN] = T(double(Fo[EN]) + 0.5 * (JyS * (B(BZ, 0, 0) + B(BZ, 1, 0)) - JzS * (B(BY, 0, 0) + B(BY, 1, 0))));
        Fo[BY] = T(double(Fo[BY]) - JzS);
        Fo[BZ] = T(double(Fo[BZ]) + JyS);
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) FB[v * SFLUX + q] = Fo[v];
  }
  __syncthreads();

  // ---- D: x flux differences, F(i-1/2) - F(i+1/2), in FP64 ----
  const int tx = tid % TX, ty = tid / TX;
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
    acc[v] = double(FB[v * SFLUX + ty * XF + tx]) - double(FB[v * SFLUX + ty * XF + tx + 1]);
  __syncthreads();

  // ---- E: y slopes for rows ry = 1 .. TY+2 on tile columns ----
  for (int q = tid; q < (TY + 2) * TX; q += NT) {
    const int cx = q % TX, cy = q / TX;
    const int o = (cy + 1) * RX + (cx + 2);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      T l, r;
      reconstruct<T>(lm, W[v * RY * RX + o - RX], W[v * RY * RX + o], W[v * RY * RX + o + RX], l, r);
      SL[v * SFACE + q] = l;
      SR[v * SFACE + q] = r;
    }
  }
  __syncthreads();
  if (!pery) {
    if (gj0 == 1 && tid < TX) {  // south face: VL = flip(VR)   (2D_KH/bc.f90:61-70)
      for (int v = 0; v < NV; ++v) {
        const T s = SR[v * SFACE + 1 * TX + tid];
        SL[v * SFACE + 0 * TX + tid] = ((a.bc_flip[2] >> v) & 1) ? -s : s;
      }
    }
    const int cl = (jx - 2) - gj0 + 1;
    if (cl >= 1 && cl <= TY && tid < TX) {  // north face: VR = flip(VL)  (2D_KH/bc.f90:72-81)
      for (int v = 0; v < NV; ++v) {
        const T s = SL[v * SFACE + cl * TX + tid];
        SR[v * SFACE + (cl + 1) * TX + tid] = ((a.bc_flip[3] >> v) & 1) ? -s : s;
      }
    }
    __syncthreads();
  }

  // ---- F: y-face fluxes ----
  for (int q = tid; q < (TY + 1) * TX; q += NT) {
    const int cx = q % TX, fy = q / TX;
    T L[NV], R[NV], Fo[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      L[v] = SL[v * SFACE + fy * TX + cx];
      R[v] = SR[v * SFACE + (fy + 1) * TX + cx];
    }
    riemann_flux<T, 2, FLUX, OMHD_FAST>(L, R, ch, gam, r1, r2, Fo);
    if (resist) {  // 2D_reconnection/flux_resistive.f90:289-306
      const int gi = gi0 + cx, g = gj0 - 1 + fy;
      if (g >= 0 && g <= jx - 2 && gi <= ix - 2) {
        const int o = (fy + 1) * RX + (cx + 2);  // region index of cell (gi, g)
        auto B = [&](int var, int dxo, int dyo) { return double(W[var * RY * RX + o + dxo + dyo * RX]); };
        const double odx = 1.0 / a.dx;
        const double eta_dx = eta_at(a.eta_kind, a.xc[gi], a.yc[g] + 0.5 * a.dx, 0.0) * odx;
        const double JxS = eta_dx * (B(BZ, 0, 1) - B(BZ, 0, 0));
        const double JzS = eta_dx * (0.25 * (B(BY, 1, 1) + B(BY, 1, 0) - B(BY, -1, 1) - B(BY, -1, 0)) -
                                     (B(BX, 0, 1) - B(BX, 0, 0)));
        Fo[EN] = T(double(Fo[EN]) + 0.5 * (JzS * (B(BX, 0, 0) + B(BX, 0, 1)) - JxS * (B(BZ, 0, 0) + B(BZ, 0, 1))));
        Fo[BX] = T(double(Fo[BX]) + JzS);
        Fo[BZ] = T(double(Fo[BZ]) - JxS);
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) FB[v * SFLUX + q] = Fo[v];
  }
  __syncthreads();

  // ---- G: update, ghost fill, GLM, CFL ----
  const int gi = gi0 + tx, gj = gj0 + ty;
  double vcell = 0.0;
  if (gi <= ix - 2 && gj <= jx - 2) {
    const double dtx = a.dtx_scale * dt / a.dx, dty = a.dtx_scale * dt / a.dy;
    const size_t c = (size_t)gi + (size_t)ix * gj;
    double out[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double gm = double(FB[v * SFLUX + ty * TX + tx]), gp = double(FB[v * SFLUX + (ty + 1) * TX + tx]);
      double d;
      if (a.iso)
        d = dtx * (acc[v] + gm - gp);  // rk.f90:26-35 operation order
      else
        d = dtx * acc[v] + dty * (gm - gp);
      double ub = a.Ubase[v * N + c];
      if (v == PS) ub = glmf * ub;
      if (a.stage == 1 || a.time_type == OMHD_TIME_RK2)
        out[v] = ub + d;  // rk_tvd21 / rk_std21 / rk_std22
      else
        out[v] = 0.5 * (ub + a.U1[v * N + c] + d);  // rk_tvd22 (rk.f90:56-66)
    }
    if (a.stage == 2) out[PS] = glmf * out[PS];  // second GLM half (main.f90:185)

    // owner-writes ghost fill (bc.f90 order: x sides, then y sides)
    int xt[3], yt[3], xf[3], yf[3], nxt = 1, nyt = 1;
    xt[0] = gi; xf[0] = 0;
    yt[0] = gj; yf[0] = 0;
    if (gi == 1) { xt[nxt] = perx ? ix - 1 : 0; xf[nxt] = perx ? 0 : a.bc_flip[0]; ++nxt; }
    if (gi == ix - 2) { xt[nxt] = perx ? 0 : ix - 1; xf[nxt] = perx ? 0 : a.bc_flip[1]; ++nxt; }
    if (gj == 1) { yt[nyt] = pery ? jx - 1 : 0; yf[nyt] = pery ? 0 : a.bc_flip[2]; ++nyt; }
    if (gj == jx - 2) { yt[nyt] = pery ? 0 : jx - 1; yf[nyt] = pery ? 0 : a.bc_flip[3]; ++nyt; }
    for (int b = 0; b < nyt; ++b)
      for (int q = 0; q < nxt; ++q) {
        const size_t cc = (size_t)xt[q] + (size_t)ix * yt[b];
        const int fm = xf[q] ^ yf[b];
#pragma unroll
        for (int v = 0; v < NV; ++v) a.Uout[v * N + cc] = ((fm >> v) & 1) ? -out[v] : out[v];
      }

    if (a.stage == 2) {  // set_dt.f90:27-37 on the new state
      const double ro = out[RO];
      const double vx = div_<double, OMHD_FAST>(out[MX], ro), vy = div_<double, OMHD_FAST>(out[MY], ro), vz = div_<double, OMHD_FAST>(out[MZ], ro);
      const double rv2 = vx * out[MX] + vy * out[MY] + vz * out[MZ];
      const double B2 = out[BX] * out[BX] + out[BY] * out[BY] + out[BZ] * out[BZ];
      const double pr = f1g * (out[EN] - 0.5 * (rv2 + B2));
      const double f1 = gamma * pr;
      const double vfx = fast_speed<double, OMHD_FAST>(f1, B2, out[BX], ro);
      const double vfy = fast_speed<double, OMHD_FAST>(f1, B2, out[BY], ro);
      vcell = fmax2(fabs(vx) + vfx, fabs(vy) + vfy);
    }
  }
  if (a.stage == 2) {
    const double bm = block_max_pos(vcell, red32);
    StepConsts sc{a.cfl, a.dmin, a.dx, a.eta_kind};
    reduce_and_finalize(st, sc, a.err, bm, gridDim.x * gridDim.y, 1);
  }
}

template <class T, int FLUX>
int launch_one(const StageArgs& a, cudaStream_t s) {
  const size_t bytes = smem2d_bytes<T>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_stage2d<T, FLUX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return (int)e;
    configured = true;
  }
  dim3 grid((a.ix - 2 + TX - 1) / TX, (a.jx - 2 + TY - 1) / TY);
  k_stage2d<T, FLUX><<<grid, NT, bytes, s>>>(a);
  return (int)cudaGetLastError();
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
