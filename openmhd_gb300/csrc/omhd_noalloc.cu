// omhd_noalloc.cu -- a fused 2D step that allocates no device memory.
//
// Some callers cannot call cudaMalloc: drivers embedded in an application
// whose framework owns the whole device memory pool and hands out only its
// own buffers, and long-running jobs that must reserve every byte when the
// program loads rather than in the middle of a run.  For them this file
// keeps the scratch of the fused step -- the stage buffer U1, the device step
// record, the error word and the cell-centre coordinates -- in one file-scope
// static __device__ array of fixed size, OMHD_NOALLOC_SCRATCH_DOUBLES doubles
// (32 MiB).  Every GPU that loads the library holds that array until the
// process exits.  The caller still passes the state (inputs and outputs).
//
// The array is shared by every call: calls that overlap on the GPU (two
// streams, or two host threads) race on it.  Whatever must start at zero
// (step record, error word) is cleared by each call.
//
// Set-up: the first call on a device, with that device current, looks up the
// device address of the array with cudaGetSymbolAddress and caches it per
// device; that first call should therefore come before any stream capture.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "omhd_common.cuh"
#include "omhd_fused.h"
#include "omhd_runtime.h"
#include "omhd_step.cuh"

#define OMHD_NOALLOC_SCRATCH_DOUBLES (4u * 1024u * 1024u)

namespace omhd {
namespace {

static __device__ __align__(256) double g_noalloc_scratch[OMHD_NOALLOC_SCRATCH_DOUBLES];

// layout inside the array (in doubles, each part 256-byte aligned)
constexpr size_t kRecordOff = 0;    // StepState
constexpr size_t kErrorOff = 32;    // DevError
constexpr size_t kCoordOff = 64;    // x (ix), then y (jx)
constexpr size_t kTPB = 256;

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
int g_sm_count[kMaxDevices] = {0};

inline size_t align32(size_t n) { return (n + 31) & ~size_t(31); }

// ghost fill of one axis (bc.f90 and wall variants)
__global__ void k_na_bc_axis(double* __restrict__ U, int ix, int jx, int axis, int kind, int flip_lo, int flip_hi) {
  const int ext[2] = {ix, jx};
  const size_t stride[2] = {1, (size_t)ix};
  const int other = 1 - axis;
  const long long line = ext[other];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= line * NV) return;
  const int v = (int)(t / line);
  const int q = (int)(t % line);
  const size_t n = (size_t)ix * jx;
  const size_t b = (size_t)v * n + (size_t)q * stride[other];
  const size_t s = stride[axis];
  const int nx = ext[axis];
  const double lo = U[b + s], hi = U[b + (size_t)(nx - 2) * s];
  if (kind == OMHD_BC_PERIODIC) {
    U[b + (size_t)(nx - 1) * s] = lo;
    U[b] = hi;
  } else {
    U[b] = ((flip_lo >> v) & 1) ? -lo : lo;
    U[b + (size_t)(nx - 1) * s] = ((flip_hi >> v) & 1) ? -hi : hi;
  }
}

// CFL speed of the incoming state (set_dt.f90:27-52) and device planning of
// the first step, into the step record in the static array
__global__ void k_na_plan(const double* __restrict__ U, int ix, int jx, double gamma, StepState* st, DevError* err,
                          StepConsts sc) {
  __shared__ double red32[32];
  const int ni = ix - 2, nj = jx - 2;
  const long long total = (long long)ni * nj;
  const size_t n = (size_t)ix * jx;
  const double f1g = gamma - 1;
  double v = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const size_t c = (size_t)(1 + t % ni) + (size_t)ix * (size_t)(1 + t / ni);
    const double ro = U[RO * n + c];
    const double mx = U[MX * n + c], my = U[MY * n + c], mz = U[MZ * n + c];
    const double vx = mx / ro, vy = my / ro, vz = mz / ro;
    const double rv2 = vx * mx + vy * my + vz * mz;
    const double bx = U[BX * n + c], by = U[BY * n + c], bz = U[BZ * n + c];
    const double B2 = bx * bx + by * by + bz * bz;
    const double pr = f1g * (U[EN * n + c] - 0.5 * (rv2 + B2));
    const double f1 = gamma * pr;
    v = fmax2(fmax2(fabs(vx) + fast_speed(f1, B2, bx, ro), fabs(vy) + fast_speed(f1, B2, by, ro)), v);
  }
  const double bm = block_max_pos(v, red32);
  reduce_and_finalize(st, sc, err, bm, gridDim.x, 0);
}

__global__ void k_na_coords(double* x, int ix, double x0, double dx, double* y, int jx, double y0, double dy) {
  x[0] = x0 - dx / 2;
  for (int i = 1; i < ix; ++i) x[i] = x[i - 1] + dx;
  y[0] = y0 - dy / 2;
  for (int j = 1; j < jx; ++j) y[j] = y[j - 1] + dy;
}

// Once per device, with that device current: the device address of the
// static scratch array (a host-side reference to the symbol is not a device
// address and must never be handed to a kernel).
int scratch_address(double** out, int* sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    set_host_error(OMHD_CUDA_ERR, 0, 0, 0, 0.0, "no-alloc step: no usable current CUDA device");
    return OMHD_CUDA_ERR;
  }
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      char msg[160];
      snprintf(msg, sizeof msg, "no-alloc step: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      cudaGetLastError();
      set_host_error(OMHD_CUDA_ERR, 0, 0, 0, 0.0, msg);
      return OMHD_CUDA_ERR;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
      cudaGetLastError();
      set_host_error(OMHD_CUDA_ERR, 0, 0, 0, 0.0, "no-alloc step: cannot read the device's SM count");
      return OMHD_CUDA_ERR;
    }
    g_sm_count[dev] = n;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  *sms = g_sm_count[dev];
  return OMHD_OK;
}

}  // namespace
}  // namespace omhd

using namespace omhd;

extern "C" {

size_t omhd_step2d_noalloc_max_doubles(void) { return OMHD_NOALLOC_SCRATCH_DOUBLES; }

int omhd_step2d_noalloc(double* U, const omhd_config* cfg, double t0, int nsteps, void* stream,
                        omhd_step_info* info) {
  if (!U || !cfg || nsteps < 0) {
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "no-alloc step: U and cfg are required and nsteps must be >= 0");
    return OMHD_BAD_ARG;
  }
  if (cfg->nd != 2 || cfg->kx != 1 || cfg->ix < 4 || cfg->jx < 4 || !(cfg->dx > 0) || !(cfg->dy > 0) ||
      cfg->precision < 0 || cfg->precision > 2 || cfg->flux_type < 0 || cfg->flux_type > 4 || cfg->lm_type < 0 ||
      cfg->lm_type > 4 || (cfg->time_type != 0 && cfg->time_type != 1) || cfg->eta_kind < 0 || cfg->eta_kind > 2) {
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "no-alloc step: configuration is not a valid 2D run");
    return OMHD_BAD_ARG;
  }
  if ((cfg->bc_kind[0] == OMHD_BC_PERIODIC) != (cfg->bc_kind[1] == OMHD_BC_PERIODIC) ||
      (cfg->bc_kind[2] == OMHD_BC_PERIODIC) != (cfg->bc_kind[3] == OMHD_BC_PERIODIC)) {
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "no-alloc step: periodic sides must come in pairs");
    return OMHD_BAD_ARG;
  }
  const bool iso = cfg->dx == cfg->dy;
  if (cfg->eta_kind != OMHD_ETA_NONE && !iso) {
    set_host_error(OMHD_NOT_SUPPORTED, 0, 0, 0, 0.0,
                   "no-alloc step: resistive terms need equal grid spacings (dx == dy)");
    return OMHD_NOT_SUPPORTED;
  }
  const size_t n = (size_t)cfg->ix * cfg->jx;
  const size_t u1_off = align32(kCoordOff + (size_t)cfg->ix + (size_t)cfg->jx);
  const size_t need = u1_off + (size_t)NV * n;
  if (need > OMHD_NOALLOC_SCRATCH_DOUBLES) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "no-alloc step: grid %dx%d needs %zu scratch doubles, the fixed array holds %u "
             "(at most about %u cells)",
             cfg->ix, cfg->jx, need, OMHD_NOALLOC_SCRATCH_DOUBLES,
             (unsigned)((OMHD_NOALLOC_SCRATCH_DOUBLES - kCoordOff) / (NV + 1)));
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, (double)need, msg);
    return OMHD_BAD_ARG;
  }
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, U) != cudaSuccess ||
      (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
    cudaGetLastError();
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "no-alloc step: U must be device memory");
    return OMHD_BAD_ARG;
  }
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) {
    cudaGetLastError();
    set_host_error(OMHD_CUDA_ERR, 0, 0, 0, 0.0, "no-alloc step: no usable current CUDA device");
    return OMHD_CUDA_ERR;
  }
  if (attr.type == cudaMemoryTypeDevice && attr.device != cur) {
    // the scratch array and the kernels belong to the current device
    char msg[160];
    snprintf(msg, sizeof msg, "no-alloc step: U is memory of device %d, but device %d is current", attr.device,
             cur);
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, msg);
    return OMHD_BAD_ARG;
  }
  double* base = nullptr;
  int sms = 0;
  int r = scratch_address(&base, &sms);
  if (r) return r;
  cudaStream_t s = (cudaStream_t)stream;
  StepState* st = reinterpret_cast<StepState*>(base + kRecordOff);
  DevError* err = reinterpret_cast<DevError*>(base + kErrorOff);
  double* xc = base + kCoordOff;
  double* yc = xc + cfg->ix;
  double* U1 = base + u1_off;

  // coordinates by the reference recurrence (2D_basic/model.f90:19-28), only
  // read by the resistive terms; one thread runs the sequential sum in IEEE
  // double, the same values the host recurrence gives
  if (cfg->eta_kind != OMHD_ETA_NONE) {
    k_na_coords<<<1, 1, 0, s>>>(xc, cfg->ix, cfg->x0, cfg->dx, yc, cfg->jx, cfg->y0, cfg->dy);
    r = cuda_status(cudaGetLastError(), "no-alloc coordinates kernel");
    if (r) return r;
  }

  // step record and error word start at zero on every call
  StepState h;
  memset(&h, 0, sizeof h);
  h.t = t0;
  h.tend = (cfg->tend > 0) ? cfg->tend : INFINITY;
  r = cuda_status(cudaMemcpyAsync(st, &h, sizeof h, cudaMemcpyHostToDevice, s), "no-alloc step record");
  if (r) return r;
  r = cuda_status(cudaMemsetAsync(err, 0, sizeof(DevError), s), "no-alloc error word");
  if (r) return r;

  // bc on the incoming state, then the first dt (as omhd_solver_put_state)
  for (int axis = 0; axis < 2; ++axis) {
    const long long line = (axis == 0) ? cfg->jx : cfg->ix;
    k_na_bc_axis<<<ceil_div(line * NV, kTPB), kTPB, 0, s>>>(U, cfg->ix, cfg->jx, axis, cfg->bc_kind[2 * axis],
                                                           cfg->bc_flip[2 * axis], cfg->bc_flip[2 * axis + 1]);
  }
  const double dmin = iso ? cfg->dx : fmin2(cfg->dx, cfg->dy);
  StepConsts sc{cfg->cfl, dmin, cfg->dx, cfg->eta_kind};
  const long long cells = (long long)(cfg->ix - 2) * (cfg->jx - 2);
  int blocks = ceil_div(cells, kTPB);
  if (blocks > sms * 8) blocks = sms * 8;
  k_na_plan<<<blocks, kTPB, 0, s>>>(U, cfg->ix, cfg->jx, cfg->gamma, st, err, sc);
  r = cuda_status(cudaGetLastError(), "no-alloc planning kernel");
  if (r) return r;

  StageArgs a;
  memset(&a, 0, sizeof a);
  a.ix = cfg->ix;
  a.jx = cfg->jx;
  a.kx = 1;
  a.nd = 2;
  a.dx = cfg->dx;
  a.dy = cfg->dy;
  a.dz = cfg->dx;
  a.gamma = cfg->gamma;
  a.lm_type = cfg->lm_type;
  a.flux_type = cfg->flux_type;
  a.time_type = cfg->time_type;
  a.iso = iso ? 1 : 0;
  for (int q = 0; q < 6; ++q) {
    a.bc_kind[q] = cfg->bc_kind[q];
    a.bc_flip[q] = cfg->bc_flip[q];
  }
  a.eta_kind = cfg->eta_kind;
  a.xc = xc;
  a.yc = yc;
  a.zc = xc;
  a.st = st;
  a.err = err;
  a.cfl = cfg->cfl;
  a.dmin = dmin;
  auto launch = cfg->precision == OMHD_PREC_FP64          ? launch_stage2d_fp64
                : cfg->precision == OMHD_PREC_FP64_PARITY ? launch_stage2d_parity
                                                          : launch_stage2d_mixed;
  for (int k = 0; k < nsteps; ++k) {
    for (int stage = 1; stage <= 2; ++stage) {
      a.stage = stage;
      a.Uin = (stage == 1) ? U : U1;
      a.Ubase = U;
      a.U1 = (stage == 2) ? U1 : nullptr;
      a.Uout = (stage == 1) ? U1 : U;
      a.dtx_scale = (stage == 1 && cfg->time_type == OMHD_TIME_RK2) ? 0.5 : 1.0;
      stage_args_derived(a);
      const int e = launch(a, s);
      if (e) return cuda_status((cudaError_t)e, "no-alloc stage kernel");
    }
  }
  StepState out;
  DevError de;
  r = cuda_status(cudaMemcpyAsync(&out, st, sizeof out, cudaMemcpyDeviceToHost, s), "no-alloc record readback");
  if (r) return r;
  r = cuda_status(cudaMemcpyAsync(&de, err, sizeof de, cudaMemcpyDeviceToHost, s), "no-alloc error readback");
  if (r) return r;
  r = cuda_status(cudaStreamSynchronize(s), "no-alloc synchronize");
  if (r) return r;
  if (info) {
    info->t = out.t;
    info->dt = out.last_dt;
    info->ch = out.last_ch;
    info->vmax_next = out.vmax_now;
    info->steps = out.steps;
    info->done = out.done;
    info->status = de.code;
  }
  if (de.code != 0) {
    // the device's failure record, with the 1-based cell, for omhd_last_error()
    char msg[200];
    if (de.code == OMHD_NEG_PRESSURE)
      snprintf(msg, sizeof msg, "negative pressure at %d %d P: %.17g", de.i, de.j, de.value);
    else if (de.code == OMHD_NEG_DENSITY)
      snprintf(msg, sizeof msg, "negative density at %d %d rho: %.17g", de.i, de.j, de.value);
    else if (de.code == OMHD_DT_TOO_SMALL)
      snprintf(msg, sizeof msg, " dt is too small : %.17g < 1e-07", de.value);
    else
      snprintf(msg, sizeof msg, "no-alloc step: device error %d", de.code);
    set_host_error(de.code, de.i, de.j, de.k, de.value, msg);
  }
  return de.code;
}

}  // extern "C"
