// omhd_adjoint.cu -- reverse mode of the fused 2D FP64 TVD-RK2 step, and the
// checkpointed driver that gives dJ/dU_0 of N steps.
//
// One step (2D_basic/main.f90:56-188) maps U^n to U^{n+1} by
//   Ua  = glm(U^n)                      psi *= f        (glm_ss2.f90)
//   U1  = bc(Ua + D(Ua))                                (rk.f90:33-45, bc.f90)
//   U'  = bc(0.5 (Ua + U1 + D(U1)))                     (rk.f90:56-66)
//   U^{n+1} = glm(U')
// where D(U) = dt/dx (F_{i-1/2} - F_{i+1/2}) + dt/dy (G_{j-1/2} - G_{j+1/2}) on
// the interior and F = HLLD(recon(u2v(U))) with the face fixes of bc.f90 at
// the boundaries.  Its adjoint, with lam = dJ/dU^{n+1}, runs six kernels:
//   k_adj_prim  (U1)   primitives of U1; lam: psi *= f, then the bc adjoint
//                      (ghost entries of lam folded into their source cells)
//   k_adj_faces (U1)   per face: g_F = 0.5 dt/dx (lam_{i+1} - lam_i), HLLD
//                      adjoint -> gradients of the two face states
//   k_adj_cells (U1)   per cell: limiter adjoint of the three reconstructions
//                      that read the cell, u2v adjoint -> lam1 = dJ/dU1 (all
//                      cells, ghosts included) + 0.5 lam (interior)
//   k_adj_prim  (Ua)   primitives of Ua; bc adjoint of lam1
//   k_adj_faces (Ua)   g_F = dt/dx (lam1_{i+1} - lam1_i)
//   k_adj_cells (Ua)   lam^n = 0.5 lam + lam1 (interior) + stage adjoint; psi *= f
// The HLLD branches and limiter selections are the forward's: the backward
// pass recomputes each checkpoint segment with the fused stage kernels in
// tape-recording mode (omhd_tape.h) and the adjoint kernels replay those
// decisions, so at a limiter kink the adjoint takes the branch the forward
// took (a fixed subgradient).  dt and ch are the forward's recorded values,
// held fixed.  A full-length tape also drives a frozen-decision forward
// (omhd_adjoint_replay): the smooth map whose derivative the adjoint is.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "omhd_adjoint_face.h"
#include "omhd_common.cuh"
#include "omhd_fused.h"
#include "omhd_riemann.cuh"
#include "omhd_solver_impl.h"
#include "omhd_step.cuh"
#include "omhd_tape.h"

namespace omhd {
namespace {

struct AdjGeo {
  int ix, jx;
  size_t n;
  double gamma;
  double dx, dy;
  int lm;
  int per[2];   // periodic along x, y
  int flip[4];  // mirror sign masks: x-, x+, y-, y+ (bit v: slot v flips)
};

__device__ __forceinline__ double sgn_of(int mask, int v, double x) { return ((mask >> v) & 1) ? -x : x; }

// bc adjoint at interior cell (i, j), slot v: the cell's own value plus every
// ghost that bc.f90 fills from it (x sides first, then y sides over the full
// rows, so a corner ghost carries both sides' sign masks).
__device__ __forceinline__ double ring_gather(const AdjGeo& g, const double* __restrict__ lam, int v, int i, int j) {
  const size_t n = g.n;
  const int ix = g.ix, jx = g.jx;
  double val = lam[v * n + (size_t)j * ix + i];
  int gx = -1, fx = 0, gy = -1, fy = 0;
  if (g.per[0]) {
    gx = (i == 1) ? ix - 1 : ((i == ix - 2) ? 0 : -1);
  } else if (i == 1) {
    gx = 0;
    fx = g.flip[0];
  } else if (i == ix - 2) {
    gx = ix - 1;
    fx = g.flip[1];
  }
  if (g.per[1]) {
    gy = (j == 1) ? jx - 1 : ((j == jx - 2) ? 0 : -1);
  } else if (j == 1) {
    gy = 0;
    fy = g.flip[2];
  } else if (j == jx - 2) {
    gy = jx - 1;
    fy = g.flip[3];
  }
  if (gx >= 0) val += sgn_of(fx, v, lam[v * n + (size_t)j * ix + gx]);
  if (gy >= 0) val += sgn_of(fy, v, lam[v * n + (size_t)gy * ix + i]);
  if (gx >= 0 && gy >= 0) val += sgn_of(fx ^ fy, v, lam[v * n + (size_t)gy * ix + gx]);
  return val;
}

// Primitive face variables w = (vx vy vz p rho Bx By Bz psi) of a stage input
// (the same u2v as the forward stage kernel); in the same pass, the bc
// adjoint of lam on the interior (in place: only interior entries are
// written and only ghost entries are read across cells).
__global__ void __launch_bounds__(256) k_adj_prim(AdjGeo g, const double* __restrict__ U, const double* __restrict__ lg,
                                                  int state_glm, double* __restrict__ W, double* lam, int lam_glm) {
  const size_t n = g.n;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = (int)(c % g.ix), j = (int)(c / g.ix);
  if (U) {
    const double ro = U[RO * n + c];
    const double mx = U[MX * n + c], my = U[MY * n + c], mz = U[MZ * n + c];
    const double rr = rcp_nr(ro);
    const double vx = mx * rr, vy = my * rr, vz = mz * rr;  // u2v.f90:24
    const double rv2 = vx * mx + vy * my + vz * mz;
    const double bx = U[BX * n + c], by = U[BY * n + c], bz = U[BZ * n + c];
    const double B2 = bx * bx + by * by + bz * bz;
    const double pr = (g.gamma - 1) * (U[EN * n + c] - 0.5 * (rv2 + B2));  // u2v.f90:27
    double ps = U[PS * n + c];
    if (state_glm) ps = lg[2] * ps;
    W[VX * n + c] = vx;
    W[VY * n + c] = vy;
    W[VZ * n + c] = vz;
    W[PR * n + c] = pr;
    W[RO * n + c] = ro;
    W[BX * n + c] = bx;
    W[BY * n + c] = by;
    W[BZ * n + c] = bz;
    W[PS * n + c] = ps;
  }
  if (lam && i >= 1 && i <= g.ix - 2 && j >= 1 && j <= g.jx - 2) {
    const bool ring = i == 1 || i == g.ix - 2 || j == 1 || j == g.jx - 2;
    if (ring) {
      double r[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) r[v] = ring_gather(g, lam, v, i, j);
#pragma unroll
      for (int v = 0; v < NV; ++v) lam[v * n + c] = r[v];
    }
    if (lam_glm) lam[PS * n + c] *= lg[2];
  }
}

// Adjoint of one face's flux: the face between cells f and f+1 along DIR in
// row/column q.  Writes the gradients of the two face states: gUp(cell f) =
// upper state of cell f, gLo(cell f+1) = lower state of cell f+1, with the
// face fixes of bc.f90 folded in (periodic: the face at the last cell pairs
// with the first cell; mirror: the ghost-side state is the signed copy of
// the interior one).
// With a tape (tlim, tface non-null) the limiter selections and the HLLD
// branches are the recorded ones, else they are recomputed from W.
template <int DIR, int MODE>
__device__ __forceinline__ void face_vjp(const AdjGeo& g, const double* __restrict__ W, const double* __restrict__ lam,
                                         double gscale, double ch, int q, int f, const unsigned char* __restrict__ tlim,
                                         const unsigned short* __restrict__ tface, double* __restrict__ gUp,
                                         double* __restrict__ gLo) {
  constexpr int A = DIR - 1;
  const int nx = (DIR == 1) ? g.ix : g.jx;
  const size_t s = (DIR == 1) ? 1 : (size_t)g.ix;
  const size_t base = (DIR == 1) ? (size_t)q * g.ix : (size_t)q;
  const size_t n = g.n;
  const bool per = g.per[A] != 0;
  if (per && f == 0) return;  // same face as f = nx-2
  const bool lo_wall = (f == 0);
  const int mr = (f == nx - 2) ? (per ? 1 : -1) : f + 1;  // cell whose lower state is R
  double L[NV], R[NV];
  const unsigned char* tl = (MODE == tape::kReplay) ? tlim + (size_t)A * NV * n : nullptr;
  if (!lo_wall) {
    const size_t c0 = base + (size_t)f * s;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double up, lo;
      unsigned char k = (MODE == tape::kReplay) ? tl[v * n + c0] : 0;
      reconstruct_fp64<true, MODE>(g.lm, W[v * n + c0 - s], W[v * n + c0], W[v * n + c0 + s], up, lo, &k);
      L[v] = up;
    }
  }
  if (mr >= 0) {
    const size_t c0 = base + (size_t)mr * s;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double up, lo;
      unsigned char k = (MODE == tape::kReplay) ? tl[v * n + c0] : 0;
      reconstruct_fp64<true, MODE>(g.lm, W[v * n + c0 - s], W[v * n + c0], W[v * n + c0 + s], up, lo, &k);
      R[v] = lo;
    }
  }
  if (lo_wall) {
#pragma unroll
    for (int v = 0; v < NV; ++v) L[v] = sgn_of(g.flip[2 * A], v, R[v]);
  }
  if (mr < 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) R[v] = sgn_of(g.flip[2 * A + 1], v, L[v]);
  }
  double gF[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double lr = (mr >= 0) ? lam[v * n + base + (size_t)mr * s] : 0.0;
    const double ll = lo_wall ? 0.0 : lam[v * n + base + (size_t)f * s];
    gF[v] = gscale * (lr - ll);
  }
  double gL[NV], gR[NV];
  unsigned hk = (MODE == tape::kReplay) ? tface[(size_t)A * n + base + (size_t)f * s] : 0u;
  adj::hlld_vjp<DIR, MODE>(L, R, ch, g.gamma, gF, gL, gR, &hk);
  const size_t up_off = (size_t)A * NV * n, lo_off = up_off;
  if (lo_wall) {
    const size_t c1 = base + s;
#pragma unroll
    for (int v = 0; v < NV; ++v) gLo[lo_off + v * n + c1] = gR[v] + sgn_of(g.flip[2 * A], v, gL[v]);
    return;
  }
  const size_t cf = base + (size_t)f * s;
  if (mr < 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) gUp[up_off + v * n + cf] = gL[v] + sgn_of(g.flip[2 * A + 1], v, gR[v]);
    return;
  }
  const size_t cr = base + (size_t)mr * s;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    gUp[up_off + v * n + cf] = gL[v];
    gLo[lo_off + v * n + cr] = gR[v];
  }
}

// x faces (rows 1..jx-2, faces 0..ix-2) in the first nbx blocks, y faces
// (columns 1..ix-2, faces 0..jx-2) in the rest; consecutive threads take
// consecutive cells along x in both.
template <int MODE>
__global__ void __launch_bounds__(128) k_adj_faces(AdjGeo g, const double* __restrict__ W,
                                                   const double* __restrict__ lam, const double* __restrict__ lg,
                                                   double lscale, int nbx, const unsigned char* __restrict__ tlim,
                                                   const unsigned short* __restrict__ tface,
                                                   double* __restrict__ gUp, double* __restrict__ gLo) {
  const double dt = lg[0], ch = lg[1];
  if ((int)blockIdx.x < nbx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nf = g.ix - 1;
    if (t >= (long long)nf * (g.jx - 2)) return;
    face_vjp<1, MODE>(g, W, lam, lscale * (dt / g.dx), ch, 1 + (int)(t / nf), (int)(t % nf), tlim, tface, gUp, gLo);
  } else {
    const long long t = (long long)(blockIdx.x - nbx) * blockDim.x + threadIdx.x;
    const int nq = g.ix - 2;
    if (t >= (long long)nq * (g.jx - 1)) return;
    face_vjp<2, MODE>(g, W, lam, lscale * (dt / g.dy), ch, 1 + (int)(t % nq), (int)(t / nq), tlim, tface, gUp, gLo);
  }
}

// Per cell: adjoint of the (up to) three reconstructions per direction that
// read the cell, then of u2v; adds a1*A + B on the interior (the RK
// pass-through terms) and the GLM factor on psi when asked.
__global__ void __launch_bounds__(256) k_adj_cells(AdjGeo g, const double* __restrict__ U,
                                                   const double* __restrict__ W, const double* __restrict__ gUp,
                                                   const double* __restrict__ gLo, const double* __restrict__ Ain,
                                                   double a1, const double* __restrict__ Bin,
                                                   const double* __restrict__ lg, int out_glm,
                                                   const unsigned char* __restrict__ tlim,
                                                   double* __restrict__ out) {
  const size_t n = g.n;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int ix = g.ix, jx = g.jx;
  const int i = (int)(c % ix), j = (int)(c / ix);
  double gw[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) gw[v] = 0.0;
#pragma unroll
  for (int A = 0; A < 2; ++A) {
    const int pos = A == 0 ? i : j;
    const int nx = A == 0 ? ix : jx;
    const bool row_ok = A == 0 ? (j >= 1 && j <= jx - 2) : (i >= 1 && i <= ix - 2);
    if (!row_ok) continue;
    const size_t s = A == 0 ? 1 : (size_t)ix;
#pragma unroll
    for (int d = -1; d <= 1; ++d) {  // this cell is at offset d from the reconstructed cell m
      const int m = pos - d;
      if (m < 1 || m > nx - 2) continue;
      const size_t cm = (d == -1) ? c + s : ((d == 1) ? c - s : c);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double gm = 0.0, g0 = 0.0, gp = 0.0;
        const unsigned char k = tlim ? tlim[(A * NV + v) * n + cm]
                                     : adj::recon_code(g.lm, W[v * n + cm - s], W[v * n + cm], W[v * n + cm + s]);
        adj::recon_vjp_code(g.lm, k, gUp[(A * NV + v) * n + cm], gLo[(A * NV + v) * n + cm], gm, g0, gp);
        gw[v] += (d == -1) ? gm : ((d == 0) ? g0 : gp);
      }
    }
  }
  double Uc[NV], gU[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    Uc[v] = U[v * n + c];
    gU[v] = 0.0;
  }
  adj::u2v_vjp(Uc, g.gamma, gw, gU);
  const bool interior = i >= 1 && i <= ix - 2 && j >= 1 && j <= jx - 2;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double val = gU[v];
    if (interior) {
      val += a1 * Ain[v * n + c];
      if (Bin) val += Bin[v * n + c];
    }
    if (v == PS && out_glm) val *= lg[2];
    out[v * n + c] = val;
  }
}

// bc adjoint of the initial fill: interior gets the ring gather, ghosts 0.
__global__ void __launch_bounds__(256) k_adj_final(AdjGeo g, const double* __restrict__ lam, double* __restrict__ out) {
  const size_t n = g.n;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = (int)(c % g.ix), j = (int)(c / g.ix);
  const bool interior = i >= 1 && i <= g.ix - 2 && j >= 1 && j <= g.jx - 2;
#pragma unroll
  for (int v = 0; v < NV; ++v) out[v * n + c] = interior ? ring_gather(g, lam, v, i, j) : 0.0;
}

// {dt, ch, glm factor} of the step about to run
__global__ void k_log_step(const StepState* __restrict__ st, double* __restrict__ out) {
  out[0] = st->dt;
  out[1] = st->ch;
  out[2] = st->glm_f;
}

// the step about to run takes a recorded {dt, ch, glm factor}
__global__ void k_force_step(StepState* __restrict__ st, const double* __restrict__ in) {
  st->dt = in[0];
  st->ch = in[1];
  st->glm_f = in[2];
}

}  // namespace
}  // namespace omhd

using namespace omhd;

struct omhd_adjoint {
  omhd_config cfg;
  omhd_solver* s = nullptr;  // forward stepping with the fused FP64 kernels
  AdjGeo geo;
  int nsteps = 0, every = 1, nck = 0;
  size_t n = 0;
  cudaStream_t stream = nullptr;
  double* ck = nullptr;      // nck states
  StepState* ckst = nullptr; // nck step records
  double* segU = nullptr;    // every states U^k of the segment being reversed
  double* segU1 = nullptr;   // every stage-1 results U1^k
  unsigned char* segTl = nullptr;   // decision tape of the segment: every x 2 stages
  unsigned short* segTf = nullptr;
  unsigned char* fullTl = nullptr;  // decision tape of a whole recorded run (nsteps x 2 stages)
  unsigned short* fullTf = nullptr;
  double* Uw = nullptr;      // working state of the forward runs
  double* U1w = nullptr;     // stage buffer of the plain forward run
  double* logd = nullptr;    // 3 * nsteps: {dt, ch, glm factor} of the last forward run
  double* tlog = nullptr;    // 3 * nsteps: the same, of the recorded run (replay takes these)
  double* W = nullptr;       // primitives of the current stage input
  double* gUp = nullptr;     // 2 * NV planes
  double* gLo = nullptr;     // 2 * NV planes
  double* lam[3] = {nullptr, nullptr, nullptr};
  size_t bytes = 0;
  bool have_forward = false, have_tape = false;
  bool last_seg_live = false;  // the plain forward left the last segment's stage inputs and tape in place
  omhd_error_info last = {};
};

namespace {

int acerr(omhd_adjoint* a, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return OMHD_OK;
  if (a) {
    a->last.code = OMHD_CUDA_ERR;
    snprintf(a->last.message, sizeof a->last.message, "CUDA error in %s: %s", where, cudaGetErrorString(e));
  }
  return OMHD_CUDA_ERR;
}

template <class P>
int amalloc(omhd_adjoint* a, P** p, size_t count, const char* what) {
  const int r = acerr(a, cudaMalloc(p, sizeof(P) * count), what);
  if (!r) a->bytes += sizeof(P) * count;
  return r;
}

// decision-tape slots of one stage
size_t tl_stride(const omhd_adjoint* a) { return (size_t)2 * NV * a->n; }
size_t tf_stride(const omhd_adjoint* a) { return (size_t)2 * a->n; }

// One fused step of the solver's bound state with its stages' decisions
// recorded in (or replayed from) the tape slots tl[0..1], tf[0..1].
int taped_step(omhd_adjoint* a, int mode, unsigned char* tl, unsigned short* tf) {
  for (int stage = 1; stage <= 2; ++stage) {
    StageArgs sa = make_stage_args(a->s, stage);
    sa.tlim = tl + (size_t)(stage - 1) * tl_stride(a);
    sa.tface = tf + (size_t)(stage - 1) * tf_stride(a);
    const int e = launch_stage2d_fp64_tape(sa, mode, a->stream);
    if (e) return acerr(a, (cudaError_t)e, "taped stage kernel launch");
  }
  return OMHD_OK;
}

int launch_step_vjp(omhd_adjoint* a, const double* Un, const double* U1, const double* lg, double* lam_in,
                    double* lam1, double* lam_out, const unsigned char* tl, const unsigned short* tf) {
  const AdjGeo& g = a->geo;
  const int TPB = 256, FPB = 128;
  const int cb = ceil_div((long long)g.n, TPB);
  const int nbx = ceil_div((long long)(g.ix - 1) * (g.jx - 2), FPB);
  const int nby = ceil_div((long long)(g.ix - 2) * (g.jx - 1), FPB);
  cudaStream_t st = a->stream;
  const unsigned char* tl1 = tl;
  const unsigned char* tl2 = tl ? tl + tl_stride(a) : nullptr;
  const unsigned short* tf1 = tf;
  const unsigned short* tf2 = tf ? tf + tf_stride(a) : nullptr;
  // stage 2: U' = 0.5 (Ua + U1 + D(U1)), then bc and the second GLM half
  k_adj_prim<<<cb, TPB, 0, st>>>(g, U1, lg, 0, a->W, lam_in, 1);
  if (tl)
    k_adj_faces<tape::kReplay><<<nbx + nby, FPB, 0, st>>>(g, a->W, lam_in, lg, 0.5, nbx, tl2, tf2, a->gUp, a->gLo);
  else
    k_adj_faces<tape::kNone><<<nbx + nby, FPB, 0, st>>>(g, a->W, lam_in, lg, 0.5, nbx, nullptr, nullptr, a->gUp,
                                                         a->gLo);
  k_adj_cells<<<cb, TPB, 0, st>>>(g, U1, a->W, a->gUp, a->gLo, lam_in, 0.5, nullptr, lg, 0, tl2, lam1);
  // stage 1: U1 = bc(Ua + D(Ua)), Ua = first GLM half of U^n
  k_adj_prim<<<cb, TPB, 0, st>>>(g, Un, lg, 1, a->W, lam1, 0);
  if (tl)
    k_adj_faces<tape::kReplay><<<nbx + nby, FPB, 0, st>>>(g, a->W, lam1, lg, 1.0, nbx, tl1, tf1, a->gUp, a->gLo);
  else
    k_adj_faces<tape::kNone><<<nbx + nby, FPB, 0, st>>>(g, a->W, lam1, lg, 1.0, nbx, nullptr, nullptr, a->gUp,
                                                         a->gLo);
  k_adj_cells<<<cb, TPB, 0, st>>>(g, Un, a->W, a->gUp, a->gLo, lam_in, 0.5, lam1, lg, 1, tl1, lam_out);
  return acerr(a, cudaGetLastError(), "adjoint step kernels");
}

int validate_adjoint(const omhd_config* c) {
  if (!c) return OMHD_BAD_ARG;
  if (c->nd != 2) return OMHD_NOT_SUPPORTED;
  if (c->flux_type != OMHD_FLUX_HLLD) return OMHD_NOT_SUPPORTED;
  if (c->lm_type != OMHD_LM_MINMOD && c->lm_type != OMHD_LM_MC) return OMHD_NOT_SUPPORTED;
  if (c->time_type != OMHD_TIME_TVDRK2) return OMHD_NOT_SUPPORTED;
  if (c->eta_kind != OMHD_ETA_NONE) return OMHD_NOT_SUPPORTED;
  return OMHD_OK;
}

// Forward run from U0 (copied, bc applied): checkpoints and the step log,
// optionally the full decision tape (mode tape::kRecord) or, with
// tape::kReplay, every decision and every {dt, ch, glm factor} taken from a
// recorded run.
int run_forward(omhd_adjoint* a, const double* U0, double* UN, int mode) {
  omhd_solver* s = a->s;
  const size_t S = NV * a->n;
  int r = omhd_solver_bind(s, a->Uw, a->U1w);
  r = r ? r : omhd_solver_put_state(s, U0, 0.0);  // copy, bc, plan the first dt
  for (int k = 0; k < a->nsteps && !r; ++k) {
    if (mode != tape::kReplay && k % a->every == 0) {
      const int q = k / a->every;
      r = acerr(a, cudaMemcpyAsync(a->ck + S * q, a->Uw, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream),
                "checkpoint copy");
      r = r ? r
            : acerr(a, cudaMemcpyAsync(a->ckst + q, s->st, sizeof(StepState), cudaMemcpyDeviceToDevice, a->stream),
                    "checkpoint record copy");
    }
    if (r) break;
    if (mode == tape::kReplay)
      k_force_step<<<1, 1, 0, a->stream>>>(s->st, a->tlog + 3 * (size_t)k);
    else
      k_log_step<<<1, 1, 0, a->stream>>>(s->st, a->logd + 3 * (size_t)k);
    r = acerr(a, cudaGetLastError(), "step record kernel");
    if (r) break;
    const int klast = (a->nck - 1) * a->every;  // first step of the last segment
    if (mode == tape::kNone && k >= klast) {
      // the last segment is reversed first: keep its stage inputs and decisions
      // now, so the backward pass need not recompute it
      const int j = k - klast;
      r = acerr(a, cudaMemcpyAsync(a->segU + S * j, a->Uw, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream),
                "segment copy");
      r = r ? r : omhd_solver_bind(s, a->Uw, a->segU1 + S * j);
      r = r ? r : taped_step(a, tape::kRecord, a->segTl + 2 * tl_stride(a) * j, a->segTf + 2 * tf_stride(a) * j);
    } else if (mode == tape::kNone) {
      r = omhd_solver_step(s, 1);
    } else {
      r = taped_step(a, mode, a->fullTl + 2 * tl_stride(a) * k, a->fullTf + 2 * tf_stride(a) * k);
    }
  }
  const int rb = omhd_solver_bind(s, a->Uw, a->U1w);
  r = r ? r : rb;
  if (!r && UN)
    r = acerr(a, cudaMemcpyAsync(UN, a->Uw, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream), "state copy");
  return r;
}

}  // namespace

extern "C" {

int omhd_adjoint_create(const omhd_config* cfg, int nsteps, int checkpoint_every, omhd_adjoint** out) {
  if (!out || nsteps < 1 || checkpoint_every < 1) return OMHD_BAD_ARG;
  *out = nullptr;
  int r = validate_adjoint(cfg);
  if (r) return r;
  omhd_config c = *cfg;
  c.kx = 1;
  c.precision = OMHD_PREC_FP64;
  c.tend = 0.0;
  omhd_adjoint* a = new omhd_adjoint();
  a->cfg = c;
  r = omhd_solver_create(&c, &a->s);
  if (r) {
    delete a;
    return r;
  }
  a->nsteps = nsteps;
  a->every = checkpoint_every < nsteps ? checkpoint_every : nsteps;
  a->nck = (nsteps + a->every - 1) / a->every;
  a->n = (size_t)c.ix * c.jx;
  AdjGeo& g = a->geo;
  g.ix = c.ix;
  g.jx = c.jx;
  g.n = a->n;
  g.gamma = c.gamma;
  g.dx = c.dx;
  g.dy = c.dy;
  g.lm = c.lm_type;
  g.per[0] = c.bc_kind[0] == OMHD_BC_PERIODIC;
  g.per[1] = c.bc_kind[2] == OMHD_BC_PERIODIC;
  for (int q = 0; q < 4; ++q) g.flip[q] = c.bc_flip[q];
  const size_t S = NV * a->n;
  r = r ? r : amalloc(a, &a->ck, S * a->nck, "checkpoint allocation");
  r = r ? r : amalloc(a, &a->segU, S * a->every, "segment allocation");
  r = r ? r : amalloc(a, &a->segU1, S * a->every, "segment allocation");
  r = r ? r : amalloc(a, &a->segTl, 2 * tl_stride(a) * a->every, "segment tape allocation");
  r = r ? r : amalloc(a, &a->segTf, 2 * tf_stride(a) * a->every, "segment tape allocation");
  r = r ? r : amalloc(a, &a->Uw, S, "work state allocation");
  r = r ? r : amalloc(a, &a->U1w, S, "work state allocation");
  r = r ? r : amalloc(a, &a->logd, 3 * (size_t)nsteps, "step log allocation");
  r = r ? r : amalloc(a, &a->W, S, "adjoint work allocation");
  r = r ? r : amalloc(a, &a->gUp, 2 * S, "adjoint work allocation");
  r = r ? r : amalloc(a, &a->gLo, 2 * S, "adjoint work allocation");
  for (int q = 0; q < 3; ++q) r = r ? r : amalloc(a, &a->lam[q], S, "adjoint work allocation");
  r = r ? r : amalloc(a, &a->ckst, (size_t)a->nck, "checkpoint record allocation");
  if (!r) {  // tape entries of cells no stage records (ghosts) stay defined
    r = acerr(a, cudaMemset(a->segTl, 0, 2 * tl_stride(a) * a->every), "tape clear");
    r = r ? r : acerr(a, cudaMemset(a->segTf, 0, sizeof(unsigned short) * 2 * tf_stride(a) * a->every), "tape clear");
  }
  if (!r) r = omhd_solver_bind(a->s, a->Uw, a->U1w);
  if (r) {
    omhd_adjoint_destroy(a);
    return r;
  }
  *out = a;
  return OMHD_OK;
}

int omhd_adjoint_destroy(omhd_adjoint* a) {
  if (!a) return OMHD_OK;
  if (a->s) omhd_solver_destroy(a->s);
  void* bufs[] = {a->ck,   a->segU, a->segU1, a->segTl,  a->segTf,  a->fullTl, a->fullTf, a->Uw,  a->U1w,
                  a->logd, a->tlog, a->W,    a->gUp,    a->gLo,    a->lam[0], a->lam[1], a->lam[2], a->ckst};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete a;
  return OMHD_OK;
}

int omhd_adjoint_set_stream(omhd_adjoint* a, void* stream) {
  if (!a) return OMHD_BAD_ARG;
  a->stream = (cudaStream_t)stream;
  return omhd_solver_set_stream(a->s, stream);
}

int omhd_adjoint_forward(omhd_adjoint* a, const double* U0, double* UN) {
  if (!a || !U0) return OMHD_BAD_ARG;
  a->have_forward = a->last_seg_live = false;
  const int r = run_forward(a, U0, UN, tape::kNone);
  if (!r) a->have_forward = a->last_seg_live = true;
  return r;
}

int omhd_adjoint_record(omhd_adjoint* a, const double* U0, double* UN) {
  if (!a || !U0) return OMHD_BAD_ARG;
  int r = OMHD_OK;
  if (!a->fullTl) {
    r = amalloc(a, &a->fullTl, 2 * tl_stride(a) * a->nsteps, "tape allocation");
    r = r ? r : amalloc(a, &a->fullTf, 2 * tf_stride(a) * a->nsteps, "tape allocation");
    r = r ? r : amalloc(a, &a->tlog, 3 * (size_t)a->nsteps, "tape log allocation");
    r = r ? r : acerr(a, cudaMemsetAsync(a->fullTl, 0, 2 * tl_stride(a) * a->nsteps, a->stream), "tape clear");
    r = r ? r
          : acerr(a, cudaMemsetAsync(a->fullTf, 0, sizeof(unsigned short) * 2 * tf_stride(a) * a->nsteps, a->stream),
                  "tape clear");
    if (r) return r;
  }
  a->have_forward = a->have_tape = a->last_seg_live = false;
  r = run_forward(a, U0, UN, tape::kRecord);
  r = r ? r
        : acerr(a, cudaMemcpyAsync(a->tlog, a->logd, sizeof(double) * 3 * a->nsteps, cudaMemcpyDeviceToDevice,
                                   a->stream),
                "tape log copy");
  if (!r) a->have_forward = a->have_tape = true;
  return r;
}

int omhd_adjoint_replay(omhd_adjoint* a, const double* U0, double* UN) {
  if (!a || !U0) return OMHD_BAD_ARG;
  if (!a->have_tape) return OMHD_BAD_ARG;
  return run_forward(a, U0, UN, tape::kReplay);
}

int omhd_adjoint_step_vjp(omhd_adjoint* a, const double* Un, const double* U1, const double* log3, double* lam_in,
                          double* lam_out) {
  if (!a || !Un || !U1 || !log3 || !lam_in || !lam_out || lam_in == lam_out) return OMHD_BAD_ARG;
  return launch_step_vjp(a, Un, U1, log3, lam_in, a->lam[2], lam_out, nullptr, nullptr);
}

int omhd_adjoint_backward(omhd_adjoint* a, const double* gUN, double* gU0) {
  if (!a || !gUN || !gU0) return OMHD_BAD_ARG;
  if (!a->have_forward) return OMHD_BAD_ARG;
  omhd_solver* s = a->s;
  const size_t S = NV * a->n;
  double* lcur = a->lam[0];
  double* lnext = a->lam[1];
  int r = acerr(a, cudaMemcpyAsync(lcur, gUN, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream), "gradient copy");
  for (int q = a->nck - 1; q >= 0 && !r; --q) {
    const int k0 = q * a->every;
    const int k1 = (k0 + a->every < a->nsteps) ? k0 + a->every : a->nsteps;
    // recompute the segment from its checkpoint, keeping each step's stage
    // inputs and recording its decisions (the last segment is still in place
    // after a plain forward run)
    const bool live = (q == a->nck - 1) && a->last_seg_live;
    if (!live) {
      r = acerr(a, cudaMemcpyAsync(a->Uw, a->ck + S * q, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream),
                "checkpoint restore");
      r = r ? r
            : acerr(a, cudaMemcpyAsync(s->st, a->ckst + q, sizeof(StepState), cudaMemcpyDeviceToDevice, a->stream),
                    "checkpoint record restore");
    }
    for (int k = k0; k < k1 && !r && !live; ++k) {
      const int j = k - k0;
      double* Uk = a->segU + S * j;
      r = acerr(a, cudaMemcpyAsync(Uk, a->Uw, sizeof(double) * S, cudaMemcpyDeviceToDevice, a->stream), "segment copy");
      r = r ? r : omhd_solver_bind(s, a->Uw, a->segU1 + S * j);
      r = r ? r : taped_step(a, tape::kRecord, a->segTl + 2 * tl_stride(a) * j, a->segTf + 2 * tf_stride(a) * j);
    }
    // reverse the segment
    for (int k = k1 - 1; k >= k0 && !r; --k) {
      const int j = k - k0;
      r = launch_step_vjp(a, a->segU + S * j, a->segU1 + S * j, a->logd + 3 * (size_t)k, lcur, a->lam[2], lnext,
                          a->segTl + 2 * tl_stride(a) * j, a->segTf + 2 * tf_stride(a) * j);
      double* t = lcur;
      lcur = lnext;
      lnext = t;
    }
  }
  if (!r) {
    k_adj_final<<<ceil_div((long long)a->n, 256), 256, 0, a->stream>>>(a->geo, lcur, gU0);
    r = acerr(a, cudaGetLastError(), "adjoint final kernel");
  }
  if (a->nck > 1) a->last_seg_live = false;  // earlier segments now occupy the buffers
  const int rb = omhd_solver_bind(s, a->Uw, a->U1w);
  return r ? r : rb;
}

int omhd_adjoint_sync(omhd_adjoint* a) {
  if (!a) return OMHD_BAD_ARG;
  int r = acerr(a, cudaStreamSynchronize(a->stream), "adjoint synchronize");
  if (r) return r;
  return omhd_solver_sync(a->s, nullptr);
}

int omhd_adjoint_step_log(omhd_adjoint* a, double* log3) {
  if (!a || !log3) return OMHD_BAD_ARG;
  int r = acerr(a, cudaStreamSynchronize(a->stream), "adjoint synchronize");
  if (r) return r;
  return acerr(a, cudaMemcpy(log3, a->logd, sizeof(double) * 3 * a->nsteps, cudaMemcpyDeviceToHost), "step log copy");
}

int omhd_adjoint_memory(omhd_adjoint* a, size_t* bytes) {
  if (!a || !bytes) return OMHD_BAD_ARG;
  *bytes = a->bytes;
  return OMHD_OK;
}

}  // extern "C"
