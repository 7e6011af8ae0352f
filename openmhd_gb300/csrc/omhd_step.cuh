// omhd_step.cuh -- the device-resident step record of a fused solver and the
// per-step finalisation (set_dt + glm factor + t update) done by the last CTA
// of the second stage kernel.  dt and ch never leave the device inside a run.
#pragma once
#include "omhd_common.cuh"
#include "omhd_riemann.cuh"

namespace omhd {

struct StepState {
  double t;         // simulation time
  double dt;        // dt of the step about to run
  double ch;        // GLM speed of the step about to run (== vmax, set_dt.f90:52)
  double glm_f;     // exp(-0.5*dt*ch/cr), glm_ss2.f90:27
  double tend;      // stop at the first t >= tend (main.f90:73)
  double last_dt;   // dt of the last completed step
  double last_ch;
  double vmax_now;  // vmax of the current state
  unsigned long long vmax_acc;  // ordered-bits max of the next state's wave speeds
  unsigned int counter;         // CTAs of stage 2 that finished
  int done;
  long long steps;
};

struct StepConsts {
  double cfl;
  double dmin;       // dx (isotropic) or min(dx,dy[,dz])
  double dx;         // for the resistive dt limit
  int eta_kind;
};

__device__ __forceinline__ double glm_factor(double dt, double ch) {
  const double cr = 0.2;  // glm_ss2.f90:15
  return exp(-(0.5 * dt * ch / cr));
}

// set_dt (2D_basic/set_dt.f90:52-65) + set_dt_resistive, given the max speed
// of the current state; advances nothing.
__device__ __forceinline__ void plan_next_step(StepState* s, const StepConsts& c, double vmax, DevError* err) {
  const double dt0 = c.cfl * c.dmin / vmax;
  double dt = dt0;
  if (c.eta_kind == OMHD_ETA_RECON2D) {
    const double Rm1 = 60.0;
    dt = fmin2(dt, 0.5 * c.cfl * Rm1 * (c.dx * c.dx));
  } else if (c.eta_kind == OMHD_ETA_HARRIS_XZ) {
    const double eta_max = 1.0e-3 + 1.0 / 60.0;
    dt = fmin2(dt, 0.5 * c.cfl / eta_max * (c.dx * c.dx));
  }
  s->vmax_now = vmax;
  s->ch = vmax;
  s->dt = dt;
  s->glm_f = glm_factor(dt, vmax);
  if (!s->done && dt0 < 1.0e-7) raise_error(err, OMHD_DT_TOO_SMALL, 0, 0, 0, 0, dt0);
}

// Called by exactly one thread after all contributions to vmax_acc landed.
// stage2_done = 1 when a step just completed (t += dt).
__device__ __forceinline__ void finalize_step(StepState* s, const StepConsts& c, DevError* err, int stage2_done) {
  const unsigned long long bits = atomicExch(&s->vmax_acc, 0ull);
  const double vmax = __longlong_as_double((long long)bits);
  s->counter = 0u;
  if (stage2_done) {
    s->last_dt = s->dt;
    s->last_ch = s->ch;
    s->t = s->t + s->dt;
    s->steps = s->steps + 1;
  }
  if (s->t >= s->tend) s->done = 1;
  plan_next_step(s, c, vmax, err);
}

// warp + block max of non-negative doubles; result valid in thread 0.  For
// non-negative doubles the integer order of the bit patterns is the numeric
// order, so the max runs on the integer pipe (a floating-point compare holds
// the FP64 pipe like an FMA, and this reduction runs once per tile); a NaN
// counts as 0.
__device__ __forceinline__ double block_max_pos(double v, double* red32) {
  long long b = __double_as_longlong(v);
  if (b > 0x7ff0000000000000LL) b = 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red32[w] = __longlong_as_double(b);
  __syncthreads();
  if (w == 0) {
    b = (lane < (int)(blockDim.x >> 5)) ? __double_as_longlong(red32[lane]) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  return __longlong_as_double(b);
}

// Last-CTA-done pattern: every CTA publishes its max, the last to arrive
// finalises the step.  No CTA waits on another.
__device__ __forceinline__ void reduce_and_finalize(StepState* s, const StepConsts& c, DevError* err, double block_v,
                                                    unsigned int nblocks, int stage2_done) {
  __shared__ unsigned int is_last;
  if (threadIdx.x == 0) {
    atomic_max_pos_double(&s->vmax_acc, block_v);
    __threadfence();
    const unsigned int prev = atomicAdd(&s->counter, 1u);
    is_last = (prev == nblocks - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    finalize_step(s, c, err, stage2_done);
  }
}

}  // namespace omhd
