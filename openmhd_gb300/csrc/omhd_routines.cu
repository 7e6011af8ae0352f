// omhd_routines.cu -- routine-level kernels behind the reference-compatible
// entry points (one kernel per reference routine, one thread per cell or
// face).  This translation unit is compiled with --fmad=false: each
// expression is the reference's sequence of IEEE-754 double operations, so
// these entry points reproduce a serial FP64 run of the reference routines.
#include <cmath>
#include <cstring>
#include <vector>

#include "omhd_common.cuh"
#include "omhd_riemann.cuh"
#include "omhd_runtime.h"

namespace omhd {
namespace {

constexpr int TPB = 256;

__device__ __forceinline__ int lo_of(int n) { return (n < 2 ? n : 2) - 1; }
__device__ __forceinline__ int hi_of(int n) { return (n - 1 > 1 ? n - 1 : 1) - 1; }

// ---------------- u2v (2D_basic/u2v.f90:20-31) ----------------
__global__ void k_u2v(const double* __restrict__ U, double* __restrict__ V, size_t n, double f1,
                      DevError* err) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double ro = U[RO * n + c];
  const double mx = U[MX * n + c], my = U[MY * n + c], mz = U[MZ * n + c];
  const double vx = mx / ro, vy = my / ro, vz = mz / ro;
  const double rv2 = vx * mx + vy * my + vz * mz;
  const double bx = U[BX * n + c], by = U[BY * n + c], bz = U[BZ * n + c];
  const double B2 = bx * bx + by * by + bz * bz;
  const double pr = f1 * (U[EN * n + c] - 0.5 * (rv2 + B2));
  V[VX * n + c] = vx;
  V[VY * n + c] = vy;
  V[VZ * n + c] = vz;
  V[PR * n + c] = pr;
  if (pr <= 0) raise_error(err, OMHD_NEG_PRESSURE, 0, 0, 0, 0, pr);
  if (ro <= 0) raise_error(err, OMHD_NEG_DENSITY, 0, 0, 0, 0, ro);
}

// ---------------- limiter (2D_basic/limiter.f90) ----------------
// one thread per cell m along a line in direction `d`; lines cover the
// interior range of the two other axes (limiter.f90:30-46).
__global__ void k_limiter(const double* __restrict__ wk, double* __restrict__ wL, double* __restrict__ wR,
                          int ix, int jx, int kx, int d, int type) {
  const int ext[3] = {ix, jx, kx};
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  const int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
  const int lo1 = lo_of(ext[a1]), n1 = hi_of(ext[a1]) - lo1 + 1;
  const int lo2 = lo_of(ext[a2]), n2 = hi_of(ext[a2]) - lo2 + 1;
  const int nd = ext[d];
  const long long total = (long long)nd * n1 * n2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int m = (int)(t % nd);
  const long long line = t / nd;
  const int q1 = lo1 + (int)(line % n1);
  const int q2 = lo2 + (int)(line / n1);
  const size_t base = (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
  const size_t s = stride[d];
  if (type == LM_FLAT) {  // :54-71
    if (m < nd - 1) {
      wL[base + m * s] = wk[base + m * s];
      wR[base + m * s] = wk[base + (m + 1) * s];
    }
    return;
  }
  if (m == 0) {
    wL[base] = wk[base];  // :82
  } else if (m == nd - 1) {
    wR[base + (nd - 2) * s] = wk[base + (nd - 1) * s];  // :103
  } else {
    double l, r;
    reconstruct<double>(type, wk[base + (m - 1) * s], wk[base + m * s], wk[base + (m + 1) * s], l, r);
    wR[base + (m - 1) * s] = r;
    wL[base + m * s] = l;
  }
}

// ---------------- flux_solver (2D_basic/flux_solver.f90) ----------------
template <int DIR, int TYPE>
__global__ void k_flux(double* __restrict__ F, const double* __restrict__ VL, const double* __restrict__ VR,
                       double ch, double gamma, int ix, int jx, int kx, int is, int ni, int js, int nj,
                       int ks, int nk) {
  const long long total = (long long)ni * nj * nk;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int i = is + (int)(t % ni);
  const int j = js + (int)((t / ni) % nj);
  const int k = ks + (int)(t / ((long long)ni * nj));
  const size_t n = (size_t)ix * jx * kx;
  const size_t c = (size_t)i + (size_t)ix * ((size_t)j + (size_t)jx * k);
  double L[NV], R[NV], Fo[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    L[v] = VL[v * n + c];
    R[v] = VR[v * n + c];
  }
  const double r1 = 1.0 / (gamma - 1.0), r2 = gamma / (gamma - 1.0);
  riemann_flux<double, DIR, TYPE>(L, R, ch, gamma, r1, r2, Fo);
#pragma unroll
  for (int v = 0; v < NV; ++v) F[v * n + c] = Fo[v];
}

template <int DIR>
void launch_flux(int type, double* F, const double* VL, const double* VR, double ch, double gamma, int ix,
                 int jx, int kx, int is, int ni, int js, int nj, int ks, int nk, cudaStream_t st) {
  const long long total = (long long)ni * nj * nk;
  if (total <= 0) return;
  const int blocks = ceil_div(total, 128);
  switch (type) {
    case FX_LLF: k_flux<DIR, FX_LLF><<<blocks, 128, 0, st>>>(F, VL, VR, ch, gamma, ix, jx, kx, is, ni, js, nj, ks, nk); break;
    case FX_HLL: k_flux<DIR, FX_HLL><<<blocks, 128, 0, st>>>(F, VL, VR, ch, gamma, ix, jx, kx, is, ni, js, nj, ks, nk); break;
    case FX_HLLC: k_flux<DIR, FX_HLLC><<<blocks, 128, 0, st>>>(F, VL, VR, ch, gamma, ix, jx, kx, is, ni, js, nj, ks, nk); break;
    case FX_HLLD: k_flux<DIR, FX_HLLD><<<blocks, 128, 0, st>>>(F, VL, VR, ch, gamma, ix, jx, kx, is, ni, js, nj, ks, nk); break;
    default: k_flux<DIR, FX_LHLLD><<<blocks, 128, 0, st>>>(F, VL, VR, ch, gamma, ix, jx, kx, is, ni, js, nj, ks, nk); break;
  }
}

// ---------------- rk (2D_basic/rk.f90, 3D_basic/rk.f90) ----------------
// mode 0 tvd21, 1 tvd22, 2 std21, 3 std22; dtx = dt/dx (std21: 0.5*dt/dx)
__global__ void k_rk(int mode, double* __restrict__ U, double* __restrict__ U1, const double* __restrict__ F,
                     const double* __restrict__ G, const double* __restrict__ H, double dtx, int ix, int jx,
                     int kx, int nd) {
  const int ni = ix - 2, nj = jx - 2, nk = (nd == 3) ? kx - 2 : 1;
  const long long per = (long long)ni * nj * nk;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per * NV) return;
  const int m = (int)(t / per);
  const long long r = t % per;
  const int i = 1 + (int)(r % ni);
  const int j = 1 + (int)((r / ni) % nj);
  const int k = (nd == 3 ? 1 : 0) + (int)(r / ((long long)ni * nj));
  const size_t n = (size_t)ix * jx * kx;
  const size_t sy = ix, sz = (size_t)ix * jx;
  const size_t q = (size_t)m * n + (size_t)i + sy * j + sz * k;
  double d;
  if (nd == 3)
    d = dtx * (F[q - 1] - F[q] + G[q - sy] - G[q] + H[q - sz] - H[q]);
  else
    d = dtx * (F[q - 1] - F[q] + G[q - sy] - G[q]);
  if (mode == 1)
    U[q] = 0.5 * (U[q] + U1[q] + d);
  else if (mode == 3)
    U[q] = U[q] + d;
  else
    U1[q] = U[q] + d;
}

// ---------------- glm_ss2 (2D_basic/glm_ss2.f90:27-34) ----------------
__global__ void k_scale(double* __restrict__ a, size_t n, double f) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) a[c] = f * a[c];
}

// ---------------- set_dt (2D_basic/set_dt.f90:27-52) ----------------
__device__ __forceinline__ double cell_speed(const double* U, const double* V, size_t n, size_t c, int nd,
                                             double gamma) {
  const double bx = U[BX * n + c], by = U[BY * n + c], bz = U[BZ * n + c];
  const double ro = U[RO * n + c];
  const double B2 = bx * bx + by * by + bz * bz;
  const double f1 = gamma * V[PR * n + c];
  const double vfx = fast_speed(f1, B2, bx, ro);
  const double vfy = fast_speed(f1, B2, by, ro);
  double s = fmax2(fabs(V[VX * n + c]) + vfx, fabs(V[VY * n + c]) + vfy);
  if (nd == 3) {
    const double vfz = fast_speed(f1, B2, bz, ro);
    s = fmax2(s, fabs(V[VZ * n + c]) + vfz);
  }
  return s;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax2(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax2(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

__global__ void k_set_dt(const double* __restrict__ U, const double* __restrict__ V, int ix, int jx, int kx,
                         int nd, double gamma, unsigned long long* accum) {
  const int is = lo_of(ix), ni = hi_of(ix) - is + 1;
  const int js = lo_of(jx), nj = hi_of(jx) - js + 1;
  const int ks = lo_of(kx), nk = hi_of(kx) - ks + 1;
  const long long total = (long long)ni * nj * nk;
  const size_t n = (size_t)ix * jx * kx;
  double v = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = is + (int)(t % ni);
    const int j = js + (int)((t / ni) % nj);
    const int k = ks + (int)(t / ((long long)ni * nj));
    const size_t c = (size_t)i + (size_t)ix * ((size_t)j + (size_t)jx * k);
    v = fmax2(cell_speed(U, V, n, c, nd, gamma), v);
  }
  v = block_max(v);
  if (threadIdx.x == 0) atomic_max_pos_double(accum, v);
}

// ---------------- bc (2D_basic/bc.f90 and wall variants) ----------------
__global__ void k_bc_axis(double* __restrict__ U, int ix, int jx, int kx, int axis, int kind, int flip_lo,
                          int flip_hi) {
  const int ext[3] = {ix, jx, kx};
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
  const long long plane = (long long)ext[a1] * ext[a2];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= plane * NV) return;
  const int v = (int)(t / plane);
  const long long p = t % plane;
  const int q1 = (int)(p % ext[a1]), q2 = (int)(p / ext[a1]);
  const size_t n = (size_t)ix * jx * kx;
  const size_t b = (size_t)v * n + (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
  const size_t s = stride[axis];
  const int nx = ext[axis];
  if (kind == OMHD_BC_PERIODIC) {
    const double a = U[b + 1 * s], z = U[b + (size_t)(nx - 2) * s];
    U[b + (size_t)(nx - 1) * s] = a;  // U(ix) = U(2)
    U[b] = z;                         // U(1) = U(ix-1)
  } else {
    const double a = U[b + 1 * s], z = U[b + (size_t)(nx - 2) * s];
    U[b] = ((flip_lo >> v) & 1) ? -a : a;
    U[b + (size_t)(nx - 1) * s] = ((flip_hi >> v) & 1) ? -z : z;
  }
}

// ---------------- face-state fix ----------------
__global__ void k_facefix(double* __restrict__ VL, double* __restrict__ VR, int ix, int jx, int kx, int axis,
                          int kind_lo, int flip_lo, int kind_hi, int flip_hi) {
  const int ext[3] = {ix, jx, kx};
  const size_t stride[3] = {1, (size_t)ix, (size_t)ix * jx};
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
  const long long plane = (long long)ext[a1] * ext[a2];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= plane * NV) return;
  const int v = (int)(t / plane);
  const long long p = t % plane;
  const int q1 = (int)(p % ext[a1]), q2 = (int)(p / ext[a1]);
  const size_t n = (size_t)ix * jx * kx;
  const size_t b = (size_t)v * n + (size_t)q1 * stride[a1] + (size_t)q2 * stride[a2];
  const size_t fl = (size_t)(ext[axis] - 2) * stride[axis];
  if (kind_lo == OMHD_BC_PERIODIC) {
    VR[b + fl] = VR[b];  // VR(ix-1) = VR(1)
    VL[b] = VL[b + fl];  // VL(1) = VL(ix-1)
  } else {
    const double s0 = VR[b];
    VL[b] = ((flip_lo >> v) & 1) ? -s0 : s0;
    const double s1 = VL[b + fl];
    VR[b + fl] = ((flip_hi >> v) & 1) ? -s1 : s1;
  }
  (void)kind_hi;
}

// ---------------- resistivity ----------------
__device__ __forceinline__ double eta_of(int kind, double x, double y, double z) {
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

// 2D_reconnection/flux_resistive.f90:27-115
__global__ void k_resist2d(double* __restrict__ F, const double* __restrict__ U, const double* __restrict__ x,
                           const double* __restrict__ y, double dx, int ix, int jx, int dir, int eta_kind) {
  const int is = (dir == 1) ? 0 : 1, ni = ix - 1 - is;
  const int js = (dir == 2) ? 0 : 1, nj = jx - 1 - js;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj) return;
  const int i = is + (int)(t % ni), j = js + (int)(t / ni);
  const size_t n = (size_t)ix * jx;
  const size_t c = (size_t)i + (size_t)ix * j, sx = 1, sy = ix;
  const double* Bx = U + BX * n;
  const double* By = U + BY * n;
  const double* Bz = U + BZ * n;
  const double odx = 1.0 / dx;
  if (dir == 1) {
    const double eta_dx = eta_of(eta_kind, x[i] + 0.5 * dx, y[j], 0.0) * odx;
    const double JyS = -eta_dx * (Bz[c + sx] - Bz[c]);
    const double JzS =
        eta_dx * ((By[c + sx] - By[c]) - 0.25 * (Bx[c + sy] + Bx[c + sx + sy] - Bx[c - sy] - Bx[c + sx - sy]));
    F[EN * n + c] = F[EN * n + c] + 0.5 * (JyS * (Bz[c] + Bz[c + sx]) - JzS * (By[c] + By[c + sx]));
    F[BY * n + c] = F[BY * n + c] - JzS;
    F[BZ * n + c] = F[BZ * n + c] + JyS;
  } else {
    const double eta_dx = eta_of(eta_kind, x[i], y[j] + 0.5 * dx, 0.0) * odx;
    const double JxS = eta_dx * (Bz[c + sy] - Bz[c]);
    const double JzS =
        eta_dx * (0.25 * (By[c + sx + sy] + By[c + sx] - By[c - sx + sy] - By[c - sx]) - (Bx[c + sy] - Bx[c]));
    F[EN * n + c] = F[EN * n + c] + 0.5 * (JzS * (Bx[c] + Bx[c + sy]) - JxS * (Bz[c] + Bz[c + sy]));
    F[BX * n + c] = F[BX * n + c] + JzS;
    F[BZ * n + c] = F[BZ * n + c] - JxS;
  }
}

// 3D_reconnection_gpu/flux_resistive.cuf:45-137
__global__ void k_resist3d(double* __restrict__ F, const double* __restrict__ U, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, double dx, int ix, int jx,
                           int kx, int dir, int eta_kind) {
  const int is = (dir == 1) ? 0 : 1, ni = ix - 1 - is;
  const int js = (dir == 2) ? 0 : 1, nj = jx - 1 - js;
  const int ks = (dir == 3) ? 0 : 1, nk = kx - 1 - ks;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * nk) return;
  const int i = is + (int)(t % ni), j = js + (int)((t / ni) % nj), k = ks + (int)(t / ((long long)ni * nj));
  const size_t n = (size_t)ix * jx * kx;
  const size_t sx = 1, sy = ix, sz = (size_t)ix * jx;
  const size_t c = (size_t)i + sy * j + sz * k;
  const double* Bx = U + BX * n;
  const double* By = U + BY * n;
  const double* Bz = U + BZ * n;
  double xx = x[i], yy = y[j], zz = z[k];
  if (dir == 1) xx = x[i] + 0.5 * dx;
  if (dir == 2) yy = y[j] + 0.5 * dx;
  if (dir == 3) zz = z[k] + 0.5 * dx;
  const double eta_dx = eta_of(eta_kind, xx, yy, zz) / dx;
  if (dir == 1) {
    const double JyS = -(Bz[c + sx] - Bz[c]) + 0.25 * (Bx[c + sz] + Bx[c + sx + sz] - Bx[c - sz] - Bx[c + sx - sz]);
    const double JzS = (By[c + sx] - By[c]) - 0.25 * (Bx[c + sy] + Bx[c + sx + sy] - Bx[c - sy] - Bx[c + sx - sy]);
    F[EN * n + c] = F[EN * n + c] + 0.5 * eta_dx * (JyS * (Bz[c] + Bz[c + sx]) - JzS * (By[c] + By[c + sx]));
    F[BY * n + c] = F[BY * n + c] - eta_dx * JzS;
    F[BZ * n + c] = F[BZ * n + c] + eta_dx * JyS;
  } else if (dir == 2) {
    const double JxS = (Bz[c + sy] - Bz[c]) - 0.25 * (By[c + sz] + By[c + sy + sz] - By[c - sz] - By[c + sy - sz]);
    const double JzS = -(Bx[c + sy] - Bx[c]) + 0.25 * (By[c + sx] + By[c + sx + sy] - By[c - sx] - By[c - sx + sy]);
    F[EN * n + c] = F[EN * n + c] + 0.5 * eta_dx * (JzS * (Bx[c] + Bx[c + sy]) - JxS * (Bz[c] + Bz[c + sy]));
    F[BX * n + c] = F[BX * n + c] + eta_dx * JzS;
    F[BZ * n + c] = F[BZ * n + c] - eta_dx * JxS;
  } else {
    const double JyS = (Bx[c + sz] - Bx[c]) - 0.25 * (Bz[c + sx] + Bz[c + sx + sz] - Bz[c - sx] - Bz[c - sx + sz]);
    const double JxS = -(By[c + sz] - By[c]) + 0.25 * (Bz[c + sy] + Bz[c + sy + sz] - Bz[c - sy] - Bz[c - sy + sz]);
    F[EN * n + c] = F[EN * n + c] + 0.5 * eta_dx * (JxS * (By[c] + By[c + sz]) - JyS * (Bx[c] + Bx[c + sz]));
    F[BX * n + c] = F[BX * n + c] - eta_dx * JyS;
    F[BY * n + c] = F[BY * n + c] + eta_dx * JxS;
  }
}

double g_gamma = 5.0 / 3.0;  // param.h:3

bool dims_ok(int ix, int jx, int kx) { return ix >= 1 && jx >= 1 && kx >= 1; }

// read the device error word, reset it, and build the reference message
int collect_u2v_error(const double* Ud, const double* Vd, int ix, int jx, int kx) {
  DevError h;
  cudaStream_t st = lib_stream();
  DevError* de = lib_dev_error();
  if (cuda_status(cudaMemcpyAsync(&h, de, sizeof h, cudaMemcpyDeviceToHost, st), "u2v status")) return OMHD_CUDA_ERR;
  if (cuda_status(cudaStreamSynchronize(st), "u2v synchronize")) return OMHD_CUDA_ERR;
  if (h.code == 0) return OMHD_OK;
  cudaMemsetAsync(de, 0, sizeof(DevError), st);
  // minloc over the whole plane (u2v.f90:35-36, :40-41); first occurrence in
  // array element order
  const size_t n = (size_t)ix * jx * kx;
  std::vector<double> plane(n);
  const bool pres = h.code == OMHD_NEG_PRESSURE;
  const double* src = pres ? (Vd + PR * n) : (Ud + RO * n);
  // a negative pressure wins over a negative density, as in the reference
  if (!pres) {
    std::vector<double> pl(n);
    cudaMemcpy(pl.data(), Vd + PR * n, n * sizeof(double), cudaMemcpyDeviceToHost);
    for (size_t c = 0; c < n; ++c)
      if (pl[c] <= 0) {
        src = Vd + PR * n;
        h.code = OMHD_NEG_PRESSURE;
        break;
      }
  }
  cudaMemcpy(plane.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost);
  size_t best = 0;
  for (size_t c = 1; c < n; ++c)
    if (plane[c] < plane[best]) best = c;
  const int i = (int)(best % ix) + 1, j = (int)((best / ix) % jx) + 1, k = (int)(best / ((size_t)ix * jx)) + 1;
  char msg[160];
  char loc[48];
  if (kx > 1)
    snprintf(loc, sizeof loc, "%d %d %d", i, j, k);
  else
    snprintf(loc, sizeof loc, "%d %d", i, j);
  if (h.code == OMHD_NEG_PRESSURE)
    snprintf(msg, sizeof msg, "negative pressure at %s P: %.17g", loc, plane[best]);
  else
    snprintf(msg, sizeof msg, "negative density at %s rho: %.17g", loc, plane[best]);
  set_host_error(h.code, i, j, kx > 1 ? k : 0, plane[best], msg);
  return h.code;
}

int do_u2v(const double* U, double* V, int ix, int jx, int kx) {
  if (!dims_ok(ix, jx, kx)) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  const double* Ud = a.add(U, NV * n, true, false);
  double* Vd = a.add(V, 4 * n, false, true);
  if (a.status()) return a.status();
  DevError* de = lib_dev_error();
  if (!de) return OMHD_CUDA_ERR;
  k_u2v<<<ceil_div(n, TPB), TPB, 0, lib_stream()>>>(Ud, Vd, n, g_gamma - 1, de);
  int st = collect_u2v_error(Ud, Vd, ix, jx, kx);
  int st2 = a.finish();
  return st ? st : st2;
}

int do_limiter(const double* wk, double* wL, double* wR, int ix, int jx, int kx, int dir, int type, int nd) {
  if (!dims_ok(ix, jx, kx) || dir < 1 || dir > nd || type < 0 || type > 4) {
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, type < 0 || type > 4 ? "unknown limiter" : "bad limiter argument");
    return OMHD_BAD_ARG;
  }
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  const double* wkd = a.add(wk, n, true, false);
  double* wLd = a.add(wL, n, true, true);
  double* wRd = a.add(wR, n, true, true);
  if (a.status()) return a.status();
  const int ext[3] = {ix, jx, kx};
  const int d = dir - 1;
  auto cnt = [](int e) { return ((e - 1 > 1 ? e - 1 : 1) - 1) - ((e < 2 ? e : 2) - 1) + 1; };
  const long long total = (long long)ext[d] * cnt(ext[(d + 1) % 3]) * cnt(ext[(d + 2) % 3]);
  if (total > 0) k_limiter<<<ceil_div(total, TPB), TPB, 0, lib_stream()>>>(wkd, wLd, wRd, ix, jx, kx, d, type);
  return a.finish();
}

int do_flux(double* F, const double* VL, const double* VR, double ch, int ix, int jx, int kx, int dir, int type,
            int nd) {
  if (!dims_ok(ix, jx, kx) || dir < 1 || dir > nd || type < 0 || type > 4) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  double* Fd = a.add(F, NV * n, false, true);
  const double* VLd = a.add(VL, NV * n, true, false);
  const double* VRd = a.add(VR, NV * n, true, false);
  if (a.status()) return a.status();
  cudaStream_t st = lib_stream();
  cudaMemsetAsync(Fd, 0, NV * n * sizeof(double), st);  // flux_solver.f90:57
  auto lo = [](int e) { return (e < 2 ? e : 2) - 1; };
  auto cnt = [](int e) { return ((e - 1 > 1 ? e - 1 : 1) - 1) - ((e < 2 ? e : 2) - 1) + 1; };
  int is = lo(ix), ni = cnt(ix), js = lo(jx), nj = cnt(jx), ks = lo(kx), nk = cnt(kx);
  if (dir == 1) { is = 0; ni = ix - 1; }
  if (dir == 2) { js = 0; nj = jx - 1; }
  if (dir == 3) { ks = 0; nk = kx - 1; }
  if (dir == 1) launch_flux<1>(type, Fd, VLd, VRd, ch, g_gamma, ix, jx, kx, is, ni, js, nj, ks, nk, st);
  if (dir == 2) launch_flux<2>(type, Fd, VLd, VRd, ch, g_gamma, ix, jx, kx, is, ni, js, nj, ks, nk, st);
  if (dir == 3) launch_flux<3>(type, Fd, VLd, VRd, ch, g_gamma, ix, jx, kx, is, ni, js, nj, ks, nk, st);
  return a.finish();
}

int do_rk(int mode, double* U, double* U1, const double* F, const double* G, const double* H, double dt, double dx,
          int ix, int jx, int kx, int nd) {
  if (!dims_ok(ix, jx, kx)) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  const bool u_out = (mode == 1 || mode == 3);
  double* Ud = a.add(U, NV * n, true, u_out);
  double* U1d = (mode == 3) ? nullptr : a.add(U1, NV * n, true, !u_out);
  const double* Fd = a.add(F, NV * n, true, false);
  const double* Gd = a.add(G, NV * n, true, false);
  const double* Hd = (nd == 3) ? a.add(H, NV * n, true, false) : nullptr;
  if (a.status()) return a.status();
  const double dtx = (mode == 2) ? 0.5 * dt / dx : dt / dx;  // rk.f90:22, :76
  const long long per = (long long)(ix - 2) * (jx - 2) * (nd == 3 ? kx - 2 : 1);
  if (per > 0)
    k_rk<<<ceil_div(per * NV, TPB), TPB, 0, lib_stream()>>>(mode, Ud, U1d, Fd, Gd, Hd, dtx, ix, jx, kx, nd);
  return a.finish();
}

int do_glm(double* U, double ch, double dt, int ix, int jx, int kx) {
  if (!dims_ok(ix, jx, kx)) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  double* Ud = a.add(U, NV * n, true, true);
  if (a.status()) return a.status();
  const double cr = 0.2;                           // glm_ss2.f90:15
  const double f1 = std::exp(-(0.5 * dt * ch / cr));  // glm_ss2.f90:27 (host libm, like the reference)
  k_scale<<<ceil_div(n, TPB), TPB, 0, lib_stream()>>>(Ud + PS * n, n, f1);
  return a.finish();
}

int do_set_dt(const double* U, const double* V, double* vmax, double* dt, double dx, double cfl, int ix, int jx,
              int kx, int nd) {
  if (!dims_ok(ix, jx, kx) || !vmax || !dt) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  const double* Ud = a.add(U, NV * n, true, false);
  const double* Vd = a.add(V, 4 * n, true, false);
  if (a.status()) return a.status();
  unsigned long long* acc = lib_dev_accum();
  if (!acc) return OMHD_CUDA_ERR;
  cudaStream_t st = lib_stream();
  cudaMemsetAsync(acc, 0, sizeof(unsigned long long), st);
  auto cnt = [](int e) { return ((e - 1 > 1 ? e - 1 : 1) - 1) - ((e < 2 ? e : 2) - 1) + 1; };
  const long long total = (long long)cnt(ix) * cnt(jx) * cnt(kx);
  int blocks = ceil_div(total, TPB);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_set_dt<<<blocks, TPB, 0, st>>>(Ud, Vd, ix, jx, kx, nd, g_gamma, acc);
  unsigned long long bits = 0;
  if (cuda_status(cudaMemcpyAsync(&bits, acc, sizeof bits, cudaMemcpyDeviceToHost, st), "set_dt readback"))
    return OMHD_CUDA_ERR;
  int s2 = a.finish();
  if (cuda_status(cudaStreamSynchronize(st), "set_dt synchronize")) return OMHD_CUDA_ERR;
  if (s2) return s2;
  double vm;
  memcpy(&vm, &bits, sizeof vm);
  if (total <= 0) vm = -1.0;
  *vmax = vm;
  *dt = cfl * dx / vm;  // set_dt.f90:52
  if (*dt < 1.0e-7) {   // set_dt.f90:55-65
    char msg[160];
    snprintf(msg, sizeof msg, " dt is too small : %.17g < %.17g   velocity is : %.17g%s", *dt, 1.0e-7, vm,
             vm < 0 ? " (Potential error in OpenMP/reduction ...)" : "");
    set_host_error(OMHD_DT_TOO_SMALL, 0, 0, 0, *dt, msg);
    return OMHD_DT_TOO_SMALL;
  }
  return OMHD_OK;
}

int do_bc(double* U, int ix, int jx, int kx, int nd, const int* kind, const int* flip) {
  if (!dims_ok(ix, jx, kx) || !kind || !flip) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  double* Ud = a.add(U, NV * n, true, true);
  if (a.status()) return a.status();
  const int ext[3] = {ix, jx, kx};
  for (int axis = 0; axis < nd; ++axis) {
    const long long plane = (long long)ext[(axis + 1) % 3] * ext[(axis + 2) % 3];
    const int kd = kind[2 * axis];
    k_bc_axis<<<ceil_div(plane * NV, TPB), TPB, 0, lib_stream()>>>(Ud, ix, jx, kx, axis, kd, flip[2 * axis],
                                                                   flip[2 * axis + 1]);
  }
  return a.finish();
}

int do_facefix(double* VL, double* VR, int ix, int jx, int kx, int nd, int dir, int kl, int fl, int kh, int fh) {
  if (!dims_ok(ix, jx, kx) || dir < 1 || dir > nd) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  double* VLd = a.add(VL, NV * n, true, true);
  double* VRd = a.add(VR, NV * n, true, true);
  if (a.status()) return a.status();
  const int ext[3] = {ix, jx, kx};
  const int axis = dir - 1;
  const long long plane = (long long)ext[(axis + 1) % 3] * ext[(axis + 2) % 3];
  k_facefix<<<ceil_div(plane * NV, TPB), TPB, 0, lib_stream()>>>(VLd, VRd, ix, jx, kx, axis, kl, fl, kh, fh);
  return a.finish();
}

int do_resist(double* F, const double* U, const double* x, const double* y, const double* z, double dx, int ix,
              int jx, int kx, int nd, int dir, int eta_kind) {
  if (!dims_ok(ix, jx, kx) || dir < 1 || dir > nd) return OMHD_BAD_ARG;
  const size_t n = (size_t)ix * jx * kx;
  ArgSet a;
  double* Fd = a.add(F, NV * n, true, true);
  const double* Ud = a.add(U, NV * n, true, false);
  const double* xd = a.add(x, ix, true, false);
  const double* yd = a.add(y, jx, true, false);
  const double* zd = (nd == 3) ? a.add(z, kx, true, false) : nullptr;
  if (a.status()) return a.status();
  if (nd == 2) {
    const int ni = (dir == 1) ? ix - 1 : ix - 2, nj = (dir == 2) ? jx - 1 : jx - 2;
    const long long total = (long long)ni * nj;
    if (total > 0)
      k_resist2d<<<ceil_div(total, TPB), TPB, 0, lib_stream()>>>(Fd, Ud, xd, yd, dx, ix, jx, dir, eta_kind);
  } else {
    const long long total = (long long)((dir == 1) ? ix - 1 : ix - 2) * ((dir == 2) ? jx - 1 : jx - 2) *
                            ((dir == 3) ? kx - 1 : kx - 2);
    if (total > 0)
      k_resist3d<<<ceil_div(total, TPB), TPB, 0, lib_stream()>>>(Fd, Ud, xd, yd, zd, dx, ix, jx, kx, dir,
                                                                 eta_kind);
  }
  return a.finish();
}

int rec(int st) {
  if (st != OMHD_OK) {
    char msg[64];
    snprintf(msg, sizeof msg, "openmhd_gb300 routine failed with status %d", st);
    set_host_error(st, 0, 0, 0, 0.0, msg);
  }
  return st;
}

}  // namespace
}  // namespace omhd

using namespace omhd;

extern "C" {

int omhd_u2v_2d(const double* U, double* V, int ix, int jx) { return rec(do_u2v(U, V, ix, jx, 1)); }
int omhd_u2v_3d(const double* U, double* V, int ix, int jx, int kx) { return rec(do_u2v(U, V, ix, jx, kx)); }

int omhd_limiter_2d(const double* wk, double* wL, double* wR, int ix, int jx, int dir, int type) {
  return rec(do_limiter(wk, wL, wR, ix, jx, 1, dir, type, 2));
}
int omhd_limiter_3d(const double* wk, double* wL, double* wR, int ix, int jx, int kx, int dir, int type) {
  return rec(do_limiter(wk, wL, wR, ix, jx, kx, dir, type, 3));
}

int omhd_flux_solver_2d(double* F, const double* VL, const double* VR, double ch, int ix, int jx, int dir,
                        int type) {
  return rec(do_flux(F, VL, VR, ch, ix, jx, 1, dir, type, 2));
}
int omhd_flux_solver_3d(double* F, const double* VL, const double* VR, double ch, int ix, int jx, int kx, int dir,
                        int type) {
  return rec(do_flux(F, VL, VR, ch, ix, jx, kx, dir, type, 3));
}

int omhd_rk_tvd21_2d(const double* U, double* U1, const double* F, const double* G, double dt, double dx, int ix,
                     int jx) {
  return rec(do_rk(0, const_cast<double*>(U), U1, F, G, nullptr, dt, dx, ix, jx, 1, 2));
}
int omhd_rk_tvd22_2d(double* U, const double* U1, const double* F, const double* G, double dt, double dx, int ix,
                     int jx) {
  return rec(do_rk(1, U, const_cast<double*>(U1), F, G, nullptr, dt, dx, ix, jx, 1, 2));
}
int omhd_rk_std21_2d(const double* U, double* U1, const double* F, const double* G, double dt, double dx, int ix,
                     int jx) {
  return rec(do_rk(2, const_cast<double*>(U), U1, F, G, nullptr, dt, dx, ix, jx, 1, 2));
}
int omhd_rk_std22_2d(double* U, const double* F, const double* G, double dt, double dx, int ix, int jx) {
  return rec(do_rk(3, U, nullptr, F, G, nullptr, dt, dx, ix, jx, 1, 2));
}
int omhd_rk_tvd21_3d(const double* U, double* U1, const double* F, const double* G, const double* H, double dt,
                     double dx, int ix, int jx, int kx) {
  return rec(do_rk(0, const_cast<double*>(U), U1, F, G, H, dt, dx, ix, jx, kx, 3));
}
int omhd_rk_tvd22_3d(double* U, const double* U1, const double* F, const double* G, const double* H, double dt,
                     double dx, int ix, int jx, int kx) {
  return rec(do_rk(1, U, const_cast<double*>(U1), F, G, H, dt, dx, ix, jx, kx, 3));
}
int omhd_rk_std21_3d(const double* U, double* U1, const double* F, const double* G, const double* H, double dt,
                     double dx, int ix, int jx, int kx) {
  return rec(do_rk(2, const_cast<double*>(U), U1, F, G, H, dt, dx, ix, jx, kx, 3));
}
int omhd_rk_std22_3d(double* U, const double* F, const double* G, const double* H, double dt, double dx, int ix,
                     int jx, int kx) {
  return rec(do_rk(3, U, nullptr, F, G, H, dt, dx, ix, jx, kx, 3));
}

int omhd_glm_ss2_2d(double* U, double ch, double dt, int ix, int jx) { return rec(do_glm(U, ch, dt, ix, jx, 1)); }
int omhd_glm_ss2_3d(double* U, double ch, double dt, int ix, int jx, int kx) {
  return rec(do_glm(U, ch, dt, ix, jx, kx));
}

int omhd_set_dt_2d(const double* U, const double* V, double* vmax, double* dt, double dx, double cfl, int ix,
                   int jx) {
  return do_set_dt(U, V, vmax, dt, dx, cfl, ix, jx, 1, 2);
}
int omhd_set_dt_3d(const double* U, const double* V, double* vmax, double* dt, double dx, double cfl, int ix,
                   int jx, int kx) {
  return do_set_dt(U, V, vmax, dt, dx, cfl, ix, jx, kx, 3);
}

int omhd_set_dt_resistive(double* dt, double dx, double cfl, int eta_kind) {
  if (!dt) return OMHD_BAD_ARG;
  if (eta_kind == OMHD_ETA_RECON2D) {
    const double Rm1 = 60.0;  // 2D_reconnection/flux_resistive.f90:19-21
    *dt = fmin2(*dt, 0.5 * cfl * Rm1 * (dx * dx));
  } else if (eta_kind == OMHD_ETA_HARRIS_XZ) {
    const double eta_max = 1.0e-3 + 1.0 / 60.0;
    *dt = fmin2(*dt, 0.5 * cfl / eta_max * (dx * dx));
  }
  return OMHD_OK;
}

int omhd_bc_2d(double* U, int ix, int jx, const int kind[4], const int flip[4]) {
  return rec(do_bc(U, ix, jx, 1, 2, kind, flip));
}
int omhd_bc_3d(double* U, int ix, int jx, int kx, const int kind[6], const int flip[6]) {
  return rec(do_bc(U, ix, jx, kx, 3, kind, flip));
}

int omhd_facefix_2d(double* VL, double* VR, int ix, int jx, int dir, int kl, int fl, int kh, int fh) {
  return rec(do_facefix(VL, VR, ix, jx, 1, 2, dir, kl, fl, kh, fh));
}
int omhd_facefix_3d(double* VL, double* VR, int ix, int jx, int kx, int dir, int kl, int fl, int kh, int fh) {
  return rec(do_facefix(VL, VR, ix, jx, kx, 3, dir, kl, fl, kh, fh));
}

int omhd_flux_resistive_2d(double* F, const double* U, const double* x, const double* y, double dx, int ix, int jx,
                           int dir, int eta_kind) {
  return rec(do_resist(F, U, x, y, nullptr, dx, ix, jx, 1, 2, dir, eta_kind));
}
int omhd_flux_resistive_3d(double* F, const double* U, const double* x, const double* y, const double* z,
                           double dx, int ix, int jx, int kx, int dir, int eta_kind) {
  return rec(do_resist(F, U, x, y, z, dx, ix, jx, kx, 3, dir, eta_kind));
}

// ---- gfortran link-level drop-ins for the 2D drivers ----
void u2v_(const double* U, double* V, const int* ix, const int* jx) { finish_status(omhd_u2v_2d(U, V, *ix, *jx)); }
void limiter_(const double* wk, double* wL, double* wR, const int* ix, const int* jx, const int* dir,
              const int* type) {
  finish_status(omhd_limiter_2d(wk, wL, wR, *ix, *jx, *dir, *type));
}
void flux_solver_(double* F, const double* VL, const double* VR, const double* ch, const int* ix, const int* jx,
                  const int* dir, const int* type) {
  finish_status(omhd_flux_solver_2d(F, VL, VR, *ch, *ix, *jx, *dir, *type));
}
void rk_tvd21_(const double* U, double* U1, const double* F, const double* G, const double* dt, const double* dx,
               const int* ix, const int* jx) {
  finish_status(omhd_rk_tvd21_2d(U, U1, F, G, *dt, *dx, *ix, *jx));
}
void rk_tvd22_(double* U, const double* U1, const double* F, const double* G, const double* dt, const double* dx,
               const int* ix, const int* jx) {
  finish_status(omhd_rk_tvd22_2d(U, U1, F, G, *dt, *dx, *ix, *jx));
}
void rk_std21_(const double* U, double* U1, const double* F, const double* G, const double* dt, const double* dx,
               const int* ix, const int* jx) {
  finish_status(omhd_rk_std21_2d(U, U1, F, G, *dt, *dx, *ix, *jx));
}
void rk_std22_(double* U, const double* F, const double* G, const double* dt, const double* dx, const int* ix,
               const int* jx) {
  finish_status(omhd_rk_std22_2d(U, F, G, *dt, *dx, *ix, *jx));
}
void glm_ss2_(double* U, const double* ch, const double* dt, const int* ix, const int* jx) {
  finish_status(omhd_glm_ss2_2d(U, *ch, *dt, *ix, *jx));
}
void set_dt_(const double* U, const double* V, double* vmax, double* dt, const double* dx, const double* cfl,
             const int* ix, const int* jx) {
  finish_status(omhd_set_dt_2d(U, V, vmax, dt, *dx, *cfl, *ix, *jx));
}
void bc_(double* U, const int* ix, const int* jx) {
  const int kind[4] = {OMHD_BC_PERIODIC, OMHD_BC_PERIODIC, OMHD_BC_PERIODIC, OMHD_BC_PERIODIC};
  const int flip[4] = {0, 0, 0, 0};
  finish_status(omhd_bc_2d(U, *ix, *jx, kind, flip));
}
void flux_resistive_(double* F, const double* U, const double* x, const double* y, const double* dx, const int* ix,
                     const int* jx, const int* dir) {
  finish_status(omhd_flux_resistive_2d(F, U, x, y, *dx, *ix, *jx, *dir, OMHD_ETA_RECON2D));
}
void set_dt_resistive_(double* dt, const double* dx, const double* cfl) {
  omhd_set_dt_resistive(dt, *dx, *cfl, OMHD_ETA_RECON2D);
}

}  // extern "C"
