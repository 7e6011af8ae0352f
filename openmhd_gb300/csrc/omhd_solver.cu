// omhd_solver.cu -- the fused solver handle: owns (or binds) the state and
// stage buffers, the device step record and the error word; launches two
// fused stage kernels per TVD-RK2 step; optionally replays the launch
// sequence as a CUDA graph.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "omhd_common.cuh"
#include "omhd_fused.h"
#include "omhd_riemann.cuh"
#include "omhd_solver_impl.h"
#include "omhd_step.cuh"

namespace omhd {
namespace {

constexpr int TPB = 256;

__global__ void k_model(double* __restrict__ U, const double* __restrict__ x, const double* __restrict__ y,
                        const double* __restrict__ z, int ix, int jx, int kx, double dx, double dy, double dz,
                        double gamma, omhd_model m);

// Harris-sheet vector potential A_y from a few seeded modes (model helper)
__device__ double harris_ay(const omhd_model& m, double x, double y, double z, double Lx, double Ly) {
  const double two_pi = 8.0 * atan(1.0);
  double s = 0.0;
  for (int a = 1; a <= 4; ++a)
    for (int b = 0; b <= 1; ++b) {
      const uint64_t key = (uint64_t)(a * 8 + b);
      const double c = uniform_pm1(m.seed, 2 * key);
      const double ph = (uniform_pm1(m.seed, 2 * key + 1) + 1.0) * (two_pi / 2.0);
      s = s + c * cos(two_pi * a * x / Lx + two_pi * b * y / Ly + ph);
    }
  return m.amp * exp(-(z * z) / 4.0) * s;
}

// vector-potential profile of the 3D field loop (3D_basic/model.f90:1-6)
__device__ double loop_a3(double xx, double yy, double zz) {
  const double myr = 0.3;
  const double a = 2 * xx + zz;
  const double m2 = fmin2(fmin2((a - 2) * (a - 2), a * a), (a + 2) * (a + 2));
  return fmax2(0.0, myr - sqrt(yy * yy + m2 / 5.0));
}

// Model initial states: Orszag-Tang (2D_basic/model.f90:34-50), KH shear
// layer with a seeded vy perturbation, Harris sheet with a curl(A) perturbation
// (3D_basic/model.f90:61-63 style half-cell differences).
__global__ void k_model(double* __restrict__ U, const double* __restrict__ x, const double* __restrict__ y,
                        const double* __restrict__ z, int ix, int jx, int kx, double dx, double dy, double dz,
                        double gamma, omhd_model m) {
  const size_t n = (size_t)ix * jx * kx;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = (int)(c % ix), j = (int)((c / ix) % jx), k = (int)(c / ((size_t)ix * jx));
  const double f1 = 1.0 / (gamma - 1);
  double ro, pr, vx, vy, vz, bx, by, bz;
  if (m.kind == 0) {
    ro = gamma * gamma;
    pr = gamma;
    vx = -sin(y[j] + m.phase_y);
    vy = sin(x[i] + m.phase_x);
    vz = 0.0;
    bx = m.amp * -sin(y[j] + m.phase_y);
    by = m.amp * sin(2 * (x[i] + m.phase_x));
    bz = 0.0;
  } else if (m.kind == 1) {
    ro = 1.0;
    pr = 0.5;
    vx = m.amp * tanh(y[j]);
    vy = m.pert * exp(-(y[j] * y[j])) * uniform_pm1(m.seed, (uint64_t)c);
    vz = 0.0;
    bx = m.bx0;
    by = 0.0;
    bz = 0.0;
  } else if (m.kind == 2) {
    const double Lx = dx * (ix - 2), Ly = dy * (jx - 2);
    const double chz = cosh(z[k]);
    ro = 1.0 + (1.0 / (chz * chz)) / m.beta;
    pr = 0.5 * m.beta * ro;
    vx = 0.0;
    vy = 0.0;
    vz = 0.0;
    const double dAz =
        (harris_ay(m, x[i], y[j], z[k] + dz / 2, Lx, Ly) - harris_ay(m, x[i], y[j], z[k] - dz / 2, Lx, Ly)) / dz;
    const double dAx =
        (harris_ay(m, x[i] + dx / 2, y[j], z[k], Lx, Ly) - harris_ay(m, x[i] - dx / 2, y[j], z[k], Lx, Ly)) / dx;
    bx = tanh(z[k]) - dAz;
    by = 0.0;
    bz = dAx;
  } else if (m.kind == 3) {
    // 2D reconnection (2D_reconnection/model.f90:37-58): Harris sheet in y
    // with a localised X-point perturbation of amplitude b1 = amp
    const double chy = cosh(fmin2(y[j], 25.0));
    ro = 1.0 + (1.0 / (chy * chy)) / m.beta;
    pr = 0.5 * m.beta * ro;
    vx = 0.0;
    vy = 0.0;
    vz = 0.0;
    const double r2 = x[i] * x[i] + y[j] * y[j];
    bx = tanh(y[j]) - m.amp * y[j] * exp(-r2 / 4.0);
    by = 0.0 + m.amp * x[i] * exp(-r2 / 4.0);
    bz = 0.0;
  } else if (m.kind == 4) {
    // Brio-Wu shock tube along x (1D_basic/model.f90:43-68, the active states)
    const bool left = x[i] < 0.0;
    ro = left ? 1.0 : 0.125;
    pr = left ? 1.0 : 0.1;
    vx = 0.0;
    vy = 0.0;
    vz = 0.0;
    bx = 0.75;
    by = left ? 1.0 : -1.0;
    bz = 0.0;
  } else {
    // 3D field-loop advection (3D_basic/model.f90:1-6, 37-66): B = curl(A)
    // of a cylindrical A-profile by centred half-cell differences, v = (1,1,2)
    ro = 1.0;
    pr = 1.0;
    vx = 1.0;
    vy = 1.0;
    vz = 2.0;
    const double fx = -(m.amp / dx) * (1.0 / sqrt(5.0));
    const double fz = +(m.amp / dx) * (2.0 / sqrt(5.0));
    const double h = dx / 2;
    const double xx = x[i], yy = y[j], zz = z[k];
    bx = fz * (loop_a3(xx, yy + h, zz) - loop_a3(xx, yy - h, zz));
    by = fx * (loop_a3(xx, yy, zz + h) - loop_a3(xx, yy, zz - h)) - fz * (loop_a3(xx + h, yy, zz) - loop_a3(xx - h, yy, zz));
    bz = -fx * (loop_a3(xx, yy + h, zz) - loop_a3(xx, yy - h, zz));
  }
  const double v2 = vx * vx + vy * vy + vz * vz;
  const double B2 = bx * bx + by * by + bz * bz;
  U[RO * n + c] = ro;
  U[MX * n + c] = ro * vx;
  U[MY * n + c] = ro * vy;
  U[MZ * n + c] = ro * vz;
  U[EN * n + c] = 0.5 * (ro * v2 + B2) + f1 * pr;
  U[BX * n + c] = bx;
  U[BY * n + c] = by;
  U[BZ * n + c] = bz;
  U[PS * n + c] = 0.0;
}

// ghost fill of one axis for the whole array (bc.f90 and wall variants)
__global__ void k_bc_axis_s(double* __restrict__ U, int ix, int jx, int kx, int axis, int kind, int flip_lo,
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
  const double lo = U[b + s], hi = U[b + (size_t)(nx - 2) * s];
  if (kind == OMHD_BC_PERIODIC) {
    U[b + (size_t)(nx - 1) * s] = lo;
    U[b] = hi;
  } else {
    U[b] = ((flip_lo >> v) & 1) ? -lo : lo;
    U[b + (size_t)(nx - 1) * s] = ((flip_hi >> v) & 1) ? -hi : hi;
  }
}

// CFL speed of one cell from its conserved variables (set_dt.f90:27-37)
__device__ __forceinline__ double cell_cfl_speed(const double (&u)[NV], double gamma, int nd) {
  const double f1g = gamma - 1;
  const double ro = u[RO];
  const double mx = u[MX], my = u[MY], mz = u[MZ];
  const double vx = mx / ro, vy = my / ro, vz = mz / ro;
  const double rv2 = vx * mx + vy * my + vz * mz;
  const double bx = u[BX], by = u[BY], bz = u[BZ];
  const double B2 = bx * bx + by * by + bz * bz;
  const double pr = f1g * (u[EN] - 0.5 * (rv2 + B2));
  const double f1 = gamma * pr;
  double sp = fmax2(fabs(vx) + fast_speed(f1, B2, bx, ro), fabs(vy) + fast_speed(f1, B2, by, ro));
  if (nd == 3) sp = fmax2(sp, fabs(vz) + fast_speed(f1, B2, bz, ro));
  return sp;
}

// CFL speed of the current state (set_dt.f90:27-52) + device step planning
__global__ void k_init_cfl(const double* __restrict__ U, int ix, int jx, int kx, int nd, double gamma,
                           StepState* st, DevError* err, StepConsts sc) {
  __shared__ double red32[32];
  const int ni = ix - 2, nj = jx - 2, nk = (nd == 3) ? kx - 2 : 1;
  const long long total = (long long)ni * nj * nk;
  const size_t n = (size_t)ix * jx * kx;
  double v = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % ni), j = 1 + (int)((t / ni) % nj), k = (nd == 3 ? 1 : 0) + (int)(t / ((long long)ni * nj));
    const size_t c = (size_t)i + (size_t)ix * ((size_t)j + (size_t)jx * k);
    double u[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) u[q] = U[q * n + c];
    v = fmax2(cell_cfl_speed(u, gamma, nd), v);
  }
  const double bm = block_max_pos(v, red32);
  reduce_and_finalize(st, sc, err, bm, gridDim.x, 0);
}

// put_state for page-locked host input: one pass copies the state from host
// memory (through its device address) into U and computes the CFL speed of
// the interior cells with k_init_cfl's arithmetic, so the upload and the
// first-dt reduction share one read of the host data
__global__ void k_upload_cfl(const double* __restrict__ Uh, double* __restrict__ U, int ix, int jx, int kx, int nd,
                             double gamma, StepState* st, DevError* err, StepConsts sc) {
  __shared__ double red32[32];
  const size_t n = (size_t)ix * jx * kx;
  double v = 0.0;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    double u[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      u[q] = Uh[q * n + c];
      U[q * n + c] = u[q];
    }
    const int i = (int)(c % ix), j = (int)((c / ix) % jx), k = (int)(c / ((size_t)ix * jx));
    const bool interior = i >= 1 && i <= ix - 2 && j >= 1 && j <= jx - 2 && (nd != 3 || (k >= 1 && k <= kx - 2));
    if (interior) v = fmax2(cell_cfl_speed(u, gamma, nd), v);
  }
  const double bm = block_max_pos(v, red32);
  reduce_and_finalize(st, sc, err, bm, gridDim.x, 0);
}

__global__ void k_set_tend(StepState* st, double tend) {
  st->tend = tend;
  st->done = (st->t >= tend) ? 1 : 0;
}

}  // namespace
}  // namespace omhd

using namespace omhd;

namespace omhd {
StageArgs make_stage_args(const omhd_solver* s, int stage) {
  StageArgs a;
  memset(&a, 0, sizeof a);
  const omhd_config& c = s->cfg;
  a.Uin = (stage == 1) ? s->U : s->U1;
  a.Ubase = s->U;
  a.U1 = (stage == 2) ? s->U1 : nullptr;
  a.Uout = (stage == 1) ? s->U1 : s->U;
  a.ix = c.ix;
  a.jx = c.jx;
  a.kx = c.kx;
  a.nd = c.nd;
  a.dx = c.dx;
  a.dy = c.dy;
  a.dz = c.nd == 3 ? c.dz : c.dx;
  a.dtx_scale = (stage == 1 && c.time_type == OMHD_TIME_RK2) ? 0.5 : 1.0;
  a.gamma = c.gamma;
  a.lm_type = c.lm_type;
  a.flux_type = c.flux_type;
  a.time_type = c.time_type;
  a.stage = stage;
  a.iso = s->iso;
  for (int q = 0; q < 6; ++q) {
    a.bc_kind[q] = c.bc_kind[q];
    a.bc_flip[q] = c.bc_flip[q];
  }
  a.eta_kind = c.eta_kind;
  a.xc = s->xc;
  a.yc = s->yc;
  a.zc = s->zc;
  a.st = s->st;
  a.err = s->err;
  a.cfl = c.cfl;
  a.dmin = s->dmin;
  stage_args_derived(a);
  return a;
}
}  // namespace omhd

namespace {

int cerr(omhd_solver* s, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return OMHD_OK;
  if (s) {
    s->last.code = OMHD_CUDA_ERR;
    snprintf(s->last.message, sizeof s->last.message, "CUDA error in %s: %s", where, cudaGetErrorString(e));
  }
  return OMHD_CUDA_ERR;
}

int validate(const omhd_config* c) {
  if (!c) return OMHD_BAD_ARG;
  if (c->nd != 2 && c->nd != 3) return OMHD_BAD_ARG;
  if (c->ix < 4 || c->jx < 4) return OMHD_BAD_ARG;
  if (c->nd == 2 && c->kx != 1) return OMHD_BAD_ARG;
  if (c->nd == 3 && c->kx < 4) return OMHD_BAD_ARG;
  if (!(c->dx > 0) || !(c->dy > 0) || (c->nd == 3 && !(c->dz > 0))) return OMHD_BAD_ARG;
  if (c->lm_type < 0 || c->lm_type > 4 || c->flux_type < 0 || c->flux_type > 4) return OMHD_BAD_ARG;
  if (c->time_type != 0 && c->time_type != 1) return OMHD_BAD_ARG;
  if (c->precision < 0 || c->precision > 2) return OMHD_BAD_ARG;
  for (int a = 0; a < c->nd; ++a)
    if ((c->bc_kind[2 * a] == OMHD_BC_PERIODIC) != (c->bc_kind[2 * a + 1] == OMHD_BC_PERIODIC)) return OMHD_BAD_ARG;
  const bool iso = c->dx == c->dy && (c->nd < 3 || c->dx == c->dz);
  if (c->eta_kind != OMHD_ETA_NONE && !iso) return OMHD_NOT_SUPPORTED;
  if (c->eta_kind < 0 || c->eta_kind > 2) return OMHD_BAD_ARG;
  return OMHD_OK;
}

StepConsts consts_of(const omhd_solver* s) {
  return StepConsts{s->cfg.cfl, s->dmin, s->cfg.dx, s->cfg.eta_kind};
}

// one stage of the current step; Uhost (stage 2 only): the result is also
// written to this device address of page-locked host memory
int launch_stage(omhd_solver* s, int stage, double* Uhost = nullptr) {
  StageArgs a = make_stage_args(s, stage);
  a.Uhost = Uhost;
  const omhd_config& c = s->cfg;
  int e;
  if (c.nd == 2) {
    if (c.precision == OMHD_PREC_FP64)
      e = launch_stage2d_fp64(a, s->stream);
    else if (c.precision == OMHD_PREC_FP64_PARITY)
      e = launch_stage2d_parity(a, s->stream);
    else
      e = launch_stage2d_mixed(a, s->stream);
  } else {
    if (c.precision == OMHD_PREC_FP64)
      e = launch_stage3d_fp64(a, s->stream);
    else if (c.precision == OMHD_PREC_FP64_PARITY)
      e = launch_stage3d_parity(a, s->stream);
    else
      e = launch_stage3d_mixed(a, s->stream);
  }
  return cerr(s, (cudaError_t)e, "stage kernel launch");
}

int apply_bc(omhd_solver* s) {
  const omhd_config& c = s->cfg;
  const int ext[3] = {c.ix, c.jx, c.kx};
  for (int axis = 0; axis < c.nd; ++axis) {
    const long long plane = (long long)ext[(axis + 1) % 3] * ext[(axis + 2) % 3];
    k_bc_axis_s<<<ceil_div(plane * NV, TPB), TPB, 0, s->stream>>>(s->U, c.ix, c.jx, c.kx, axis, c.bc_kind[2 * axis],
                                                                  c.bc_flip[2 * axis], c.bc_flip[2 * axis + 1]);
  }
  return cerr(s, cudaGetLastError(), "bc kernel");
}

// new run from time t: step record and error word reset on the stream
int reset_run(omhd_solver* s, double t) {
  const omhd_config& c = s->cfg;
  StepState h;
  memset(&h, 0, sizeof h);
  h.t = t;
  h.tend = (c.tend > 0) ? c.tend : INFINITY;
  int r = cerr(s, cudaMemcpyAsync(s->st, &h, sizeof h, cudaMemcpyHostToDevice, s->stream), "step record upload");
  if (r) return r;
  r = cerr(s, cudaMemsetAsync(s->err, 0, sizeof(DevError), s->stream), "error reset");
  if (r) return r;
  s->last_status = OMHD_OK;
  memset(&s->last, 0, sizeof s->last);
  return OMHD_OK;
}

int plan_first(omhd_solver* s, double t) {
  const omhd_config& c = s->cfg;
  int r = reset_run(s, t);
  if (r) return r;
  const long long cells = (long long)(c.ix - 2) * (c.jx - 2) * (c.nd == 3 ? c.kx - 2 : 1);
  int blocks = ceil_div(cells, TPB);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_init_cfl<<<blocks, TPB, 0, s->stream>>>(s->U, c.ix, c.jx, c.kx, c.nd, c.gamma, s->st, s->err, consts_of(s));
  return cerr(s, cudaGetLastError(), "cfl kernel");
}

void drop_graph(omhd_solver* s) {
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  s->graph_steps = 0;
}

}  // namespace

namespace omhd {
int validate_config(const omhd_config* c) { return validate(c); }
}  // namespace omhd

extern "C" {

int omhd_solver_create(const omhd_config* cfg, omhd_solver** out) {
  if (!out) return OMHD_BAD_ARG;
  *out = nullptr;
  int v = validate(cfg);
  if (v) return v;
  omhd_solver* s = new omhd_solver();
  s->cfg = *cfg;
  if (s->cfg.nd == 2) s->cfg.kx = 1;
  const omhd_config& c = s->cfg;
  s->n = (size_t)c.ix * c.jx * c.kx;
  s->iso = (c.dx == c.dy && (c.nd < 3 || c.dx == c.dz)) ? 1 : 0;
  s->dmin = s->iso ? c.dx : fmin2(c.dx, c.nd == 3 ? fmin2(c.dy, c.dz) : c.dy);
  // coordinates by the reference recurrence (2D_basic/model.f90:19-28)
  s->hx.resize(c.ix);
  s->hy.resize(c.jx);
  s->hz.resize(c.kx);
  s->hx[0] = c.x0 - c.dx / 2;
  for (int i = 1; i < c.ix; ++i) s->hx[i] = s->hx[i - 1] + c.dx;
  s->hy[0] = c.y0 - c.dy / 2;
  for (int j = 1; j < c.jx; ++j) s->hy[j] = s->hy[j - 1] + c.dy;
  const double dz = c.nd == 3 ? c.dz : c.dx;
  s->hz[0] = c.z0 - dz / 2;
  for (int k = 1; k < c.kx; ++k) s->hz[k] = s->hz[k - 1] + dz;
  int r = OMHD_OK;
  r = r ? r : cerr(s, cudaMalloc(&s->xc, sizeof(double) * c.ix), "coordinate allocation");
  r = r ? r : cerr(s, cudaMalloc(&s->yc, sizeof(double) * c.jx), "coordinate allocation");
  r = r ? r : cerr(s, cudaMalloc(&s->zc, sizeof(double) * c.kx), "coordinate allocation");
  r = r ? r : cerr(s, cudaMalloc(&s->st, sizeof(StepState)), "step record allocation");
  r = r ? r : cerr(s, cudaMalloc(&s->err, sizeof(DevError)), "error word allocation");
  if (!r) {
    cudaMemcpy(s->xc, s->hx.data(), sizeof(double) * c.ix, cudaMemcpyHostToDevice);
    cudaMemcpy(s->yc, s->hy.data(), sizeof(double) * c.jx, cudaMemcpyHostToDevice);
    cudaMemcpy(s->zc, s->hz.data(), sizeof(double) * c.kx, cudaMemcpyHostToDevice);
    cudaMemset(s->st, 0, sizeof(StepState));
    cudaMemset(s->err, 0, sizeof(DevError));
  }
  if (r) {
    omhd_solver_destroy(s);
    return r;
  }
  *out = s;
  return OMHD_OK;
}

int omhd_solver_destroy(omhd_solver* s) {
  if (!s) return OMHD_OK;
  drop_graph(s);
  if (s->own_state) {
    cudaFree(s->U);
    cudaFree(s->U1);
  }
  cudaFree(s->xc);
  cudaFree(s->yc);
  cudaFree(s->zc);
  cudaFree(s->st);
  cudaFree(s->err);
  delete s;
  return OMHD_OK;
}

int omhd_solver_set_stream(omhd_solver* s, void* stream) {
  if (!s) return OMHD_BAD_ARG;
  drop_graph(s);
  s->stream = (cudaStream_t)stream;
  return OMHD_OK;
}

int omhd_solver_bind(omhd_solver* s, double* U_dev, double* U1_dev) {
  if (!s || !U_dev || !U1_dev) return OMHD_BAD_ARG;
  drop_graph(s);
  if (s->own_state) {
    cudaFree(s->U);
    cudaFree(s->U1);
    s->own_state = false;
  }
  s->U = U_dev;
  s->U1 = U1_dev;
  return OMHD_OK;
}

static int ensure_state(omhd_solver* s) {
  if (s->U) return OMHD_OK;
  int r = cerr(s, cudaMalloc(&s->U, sizeof(double) * NV * s->n), "state allocation");
  if (r) return r;
  r = cerr(s, cudaMalloc(&s->U1, sizeof(double) * NV * s->n), "stage buffer allocation");
  if (r) {
    cudaFree(s->U);
    s->U = nullptr;
    return r;
  }
  s->own_state = true;
  return OMHD_OK;
}

int omhd_solver_state_ptr(omhd_solver* s, double** U_dev) {
  if (!s || !U_dev) return OMHD_BAD_ARG;
  int r = ensure_state(s);
  if (r) return r;
  *U_dev = s->U;
  return OMHD_OK;
}

int omhd_solver_put_state(omhd_solver* s, const double* U, double t) {
  if (!s || !U) return OMHD_BAD_ARG;
  int r = ensure_state(s);
  if (r) return r;
  r = cerr(s, cudaMemcpyAsync(s->U, U, sizeof(double) * NV * s->n, cudaMemcpyDefault, s->stream), "state upload");
  if (r) return r;
  r = apply_bc(s);
  if (r) return r;
  return plan_first(s, t);
}

int omhd_solver_get_state(omhd_solver* s, double* U) {
  if (!s || !U || !s->U) return OMHD_BAD_ARG;
  int r = cerr(s, cudaMemcpyAsync(U, s->U, sizeof(double) * NV * s->n, cudaMemcpyDefault, s->stream), "state download");
  if (r) return r;
  return cerr(s, cudaStreamSynchronize(s->stream), "state download sync");
}

int omhd_solver_init_model(omhd_solver* s, const omhd_model* m) {
  if (!s || !m) return OMHD_BAD_ARG;
  int r = ensure_state(s);
  if (r) return r;
  const omhd_config& c = s->cfg;
  k_model<<<ceil_div(s->n, TPB), TPB, 0, s->stream>>>(s->U, s->xc, s->yc, s->zc, c.ix, c.jx, c.kx, c.dx, c.dy,
                                                     c.nd == 3 ? c.dz : c.dx, c.gamma, *m);
  r = cerr(s, cudaGetLastError(), "model kernel");
  if (r) return r;
  r = apply_bc(s);
  if (r) return r;
  return plan_first(s, 0.0);
}

int omhd_solver_coords(omhd_solver* s, double* x, double* y, double* z) {
  if (!s) return OMHD_BAD_ARG;
  if (x) memcpy(x, s->hx.data(), sizeof(double) * s->cfg.ix);
  if (y) memcpy(y, s->hy.data(), sizeof(double) * s->cfg.jx);
  if (z) memcpy(z, s->hz.data(), sizeof(double) * s->cfg.kx);
  return OMHD_OK;
}

int omhd_solver_set_tend(omhd_solver* s, double tend) {
  if (!s) return OMHD_BAD_ARG;
  s->cfg.tend = tend;
  k_set_tend<<<1, 1, 0, s->stream>>>(s->st, tend > 0 ? tend : INFINITY);
  return cerr(s, cudaGetLastError(), "set_tend kernel");
}

int omhd_solver_step(omhd_solver* s, int nsteps) {
  if (!s || nsteps < 0 || !s->U) return OMHD_BAD_ARG;
  for (int k = 0; k < nsteps; ++k) {
    int r = launch_stage(s, 1);
    if (r) return r;
    r = launch_stage(s, 2);
    if (r) return r;
  }
  return OMHD_OK;
}

// device address of page-locked (or registered) host memory, else nullptr
static double* mapped_host(const void* p) {
  cudaPointerAttributes at;
  if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<double*>(at.devicePointer);
}

int omhd_solver_step_host(omhd_solver* s, const double* U_in, double* U_out, double t, int nsteps) {
  if (!s || !U_out || nsteps < 1) return OMHD_BAD_ARG;
  int r = ensure_state(s);
  if (r) return r;
  const omhd_config& c = s->cfg;
  const size_t n = (size_t)c.ix * c.jx * c.kx;
  // input: one fused upload + first-dt pass from page-locked memory, else put_state
  if (U_in) {
    const double* din = mapped_host(U_in);
    if (din) {
      r = reset_run(s, t);
      if (r) return r;
      int blocks = ceil_div((long long)n, TPB);
      if (blocks > 152 * 8) blocks = 152 * 8;
      k_upload_cfl<<<blocks, TPB, 0, s->stream>>>(din, s->U, c.ix, c.jx, c.kx, c.nd, c.gamma, s->st, s->err,
                                                  consts_of(s));
      r = cerr(s, cudaGetLastError(), "upload kernel");
      if (!r) r = apply_bc(s);
    } else {
      r = omhd_solver_put_state(s, U_in, t);
    }
    if (r) return r;
  }
  StepState before;
  r = cerr(s, cudaMemcpyAsync(&before, s->st, sizeof before, cudaMemcpyDeviceToHost, s->stream), "step record read");
  if (!r) r = cerr(s, cudaStreamSynchronize(s->stream), "step record sync");
  if (r) return r;
  // output: the last stage 2 writes the result into page-locked memory as it
  // stores it, else (or if that stage did not run) a copy after the steps
  double* dout = mapped_host(U_out);
  for (int k = 0; k < nsteps; ++k) {
    r = launch_stage(s, 1);
    if (!r) r = launch_stage(s, 2, k == nsteps - 1 ? dout : nullptr);
    if (r) return r;
  }
  StepState after;
  r = cerr(s, cudaMemcpyAsync(&after, s->st, sizeof after, cudaMemcpyDeviceToHost, s->stream), "step record read");
  if (!r) r = cerr(s, cudaStreamSynchronize(s->stream), "step record sync");
  if (r) return r;
  if (!dout || after.steps != before.steps + nsteps) {
    r = cerr(s, cudaMemcpyAsync(U_out, s->U, sizeof(double) * NV * n, cudaMemcpyDefault, s->stream), "state download");
    if (!r) r = cerr(s, cudaStreamSynchronize(s->stream), "state download sync");
    if (r) return r;
  }
  return omhd_solver_sync(s, nullptr);
}

int omhd_solver_step_graph(omhd_solver* s, int nsteps, int replays) {
  if (!s || nsteps <= 0 || replays < 0 || !s->U) return OMHD_BAD_ARG;
  if (!s->stream) return OMHD_NOT_SUPPORTED;  // capture needs a non-default stream
  if (s->graph_steps != nsteps) {
    drop_graph(s);
    cudaGraph_t g;
    int r = cerr(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    if (r) return r;
    int lr = omhd_solver_step(s, nsteps);
    r = cerr(s, cudaStreamEndCapture(s->stream, &g), "graph capture end");
    if (lr) return lr;
    if (r) return r;
    r = cerr(s, cudaGraphInstantiate(&s->graph, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    if (r) return r;
    s->graph_steps = nsteps;
  }
  for (int q = 0; q < replays; ++q) {
    int r = cerr(s, cudaGraphLaunch(s->graph, s->stream), "graph launch");
    if (r) return r;
  }
  return OMHD_OK;
}

int omhd_solver_sync(omhd_solver* s, omhd_step_info* info) {
  if (!s) return OMHD_BAD_ARG;
  int r = cerr(s, cudaStreamSynchronize(s->stream), "solver synchronize");
  if (r) return r;
  StepState h;
  DevError e;
  r = cerr(s, cudaMemcpy(&h, s->st, sizeof h, cudaMemcpyDeviceToHost), "step record download");
  if (r) return r;
  r = cerr(s, cudaMemcpy(&e, s->err, sizeof e, cudaMemcpyDeviceToHost), "error download");
  if (r) return r;
  if (info) {
    info->t = h.t;
    info->dt = h.last_dt;
    info->ch = h.last_ch;
    info->vmax_next = h.vmax_now;
    info->steps = h.steps;
    info->done = h.done;
    info->status = e.code;
  }
  if (e.code != 0 && s->last.code == 0) {
    s->last.code = e.code;
    s->last.i = e.i;
    s->last.j = e.j;
    s->last.k = e.k;
    s->last.instance = e.instance;
    s->last.value = e.value;
    if (e.code == OMHD_NEG_PRESSURE)
      snprintf(s->last.message, sizeof s->last.message, "negative pressure at %d %d %d P: %.17g", e.i, e.j, e.k, e.value);
    else if (e.code == OMHD_NEG_DENSITY)
      snprintf(s->last.message, sizeof s->last.message, "negative density at %d %d %d rho: %.17g", e.i, e.j, e.k, e.value);
    else if (e.code == OMHD_DT_TOO_SMALL)
      snprintf(s->last.message, sizeof s->last.message, " dt is too small : %.17g < 1e-07", e.value);
    else
      snprintf(s->last.message, sizeof s->last.message, "device error %d", e.code);
  }
  return e.code;
}

int omhd_solver_last_error(omhd_solver* s, omhd_error_info* info) {
  if (!s) return OMHD_BAD_ARG;
  omhd_solver_sync(s, nullptr);
  if (info) *info = s->last;
  return s->last.code;
}

int omhd_solver_launches_per_step(omhd_solver* s) { return s ? 2 : 0; }

}  // extern "C"
