/*
 * openmhd_gb300.h -- C ABI of the GB300-native OpenMHD step (sm_103a).
 *
 * Two layers:
 *
 *  1. Routine-level entry points with the reference's argument lists and array
 *     layout.  Arrays are Fortran column-major double arrays U(ix,jx[,kx],var)
 *     (i fastest, variable slowest, one ghost cell per side), variable slots
 *     as in param.h:6-15.  Pointers may be host or device memory (detected
 *     with cudaPointerGetAttributes); host arrays go through a cached device
 *     mirror and the call returns with the results in host memory, device
 *     arrays are processed in place on the library's current stream.
 *       - omhd_<routine>_2d / _3d : C calling convention, scalars by value,
 *         returns an omhd_status_t.
 *       - <routine>_ : gfortran link-level drop-ins for the 2D drivers (every
 *         argument by reference, lowercase name + trailing underscore, void).
 *         Failures are recorded for omhd_last_error() and, unless
 *         omhd_set_abort_on_error(0) was called, end the process with the
 *         reference's message, as the reference's `stop` does.
 *
 *  2. A fused solver handle (omhd_solver) that advances a whole grid by full
 *     TVD-RK2 steps with two fused stage kernels per step, keeps dt/ch on the
 *     device and never synchronises inside a step.
 *
 * Errors never trap the GPU: kernels record the first failure in a device
 * error word that the host reads.
 *
 * Threads: like the reference's single-threaded drivers, the routine-level
 * entry points share library-global state (stream, error record, host-array
 * mirrors) and must be called from one thread at a time; so do the calls that
 * use them internally (omhd_fileio_output with V = NULL, omhd_solver_write)
 * and omhd_step2d_noalloc, which also keeps its scratch in one static device
 * array, so that its calls must not overlap on the GPU either.  Solver,
 * ensemble and adjoint handles are otherwise independent of each other; one
 * handle must not be used from two threads at once.
 */
#ifndef OPENMHD_GB300_H
#define OPENMHD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OMHD_ABI_VERSION 1

typedef enum {
  OMHD_OK = 0,
  OMHD_NEG_PRESSURE = 1,   /* u2v.f90:34-38 "negative pressure" */
  OMHD_NEG_DENSITY = 2,    /* u2v.f90:39-43 "negative density" */
  OMHD_DT_TOO_SMALL = 3,   /* set_dt.f90:55-65 "dt is too small" */
  OMHD_BAD_ARG = 4,        /* invalid size, direction or type */
  OMHD_TIMEOUT = 5,        /* a bounded device wait gave up */
  OMHD_CUDA_ERR = 6,       /* CUDA runtime failure */
  OMHD_NOT_SUPPORTED = 7,  /* option combination not built */
  OMHD_IO_ERR = 8          /* snapshot file error (fileio.f90:77-82) */
} omhd_status_t;

typedef struct {
  int code;        /* omhd_status_t */
  int i, j, k;     /* 1-based Fortran location of the offending cell, 0 if none */
  int instance;    /* ensemble member (batched runs), else 0 */
  double value;    /* offending value (pressure, density or dt) */
  char message[160];
} omhd_error_info;

/* ---- scheme switches (2D_basic/main.f90:16-21) ---- */
enum { OMHD_LM_FLAT = 0, OMHD_LM_MINMOD = 1, OMHD_LM_MC = 2, OMHD_LM_VANLEER = 3, OMHD_LM_KOREN = 4 };
enum { OMHD_FLUX_LLF = 0, OMHD_FLUX_HLL = 1, OMHD_FLUX_HLLC = 2, OMHD_FLUX_HLLD = 3, OMHD_FLUX_LHLLD = 4 };
enum { OMHD_TIME_TVDRK2 = 0, OMHD_TIME_RK2 = 1 };

/* ---- boundaries ---- side order: west, east, south, north, down, up */
enum { OMHD_BC_PERIODIC = 0, OMHD_BC_MIRROR = 1 };
/* flip masks (bit = variable slot) for the reference's wall conditions */
#define OMHD_FLIP(slot) (1 << ((slot) - 1)) /* slot is the 1-based param.h index */

/* ---- resistivity models ---- */
enum {
  OMHD_ETA_NONE = 0,
  OMHD_ETA_RECON2D = 1,   /* 2D_reconnection/flux_resistive.f90:1-16 */
  OMHD_ETA_HARRIS_XZ = 2  /* 1e-3 + (1/60) exp(-(x^2+z^2)/4) */
};

/* ---- arithmetic of the fused step ---- */
enum {
  OMHD_PREC_FP64 = 0,        /* FP64 throughout, multiply-add contraction on */
  OMHD_PREC_FP64_PARITY = 1, /* FP64, no contraction: the reference's IEEE op sequence */
  OMHD_PREC_MIXED = 2        /* FP32 reconstruction, Riemann solver and resistive face terms; FP64 state,
                                update and dt; u2v in FP32 except where E < rho v^2 + B^2 (low beta) */
};

/* ======================================================================
 * Routine-level entry points, C convention (0 = OMHD_OK)
 * ==================================================================== */

/* u2v: 2D_basic/u2v.f90:1-46 ; 3D_basic/u2v.f90:1-48 */
int omhd_u2v_2d(const double* U, double* V, int ix, int jx);
int omhd_u2v_3d(const double* U, double* V, int ix, int jx, int kx);

/* limiter: 2D_basic/limiter.f90:1-318 ; 3D_basic/limiter.f90:1-419 */
int omhd_limiter_2d(const double* wk, double* wL, double* wR, int ix, int jx, int dir, int type);
int omhd_limiter_3d(const double* wk, double* wL, double* wR, int ix, int jx, int kx, int dir, int type);

/* flux_solver: 2D_basic/flux_solver.f90:1-795 ; 3D_basic/flux_solver.f90:1-811 */
int omhd_flux_solver_2d(double* F, const double* VL, const double* VR, double ch, int ix, int jx,
                        int dir, int type);
int omhd_flux_solver_3d(double* F, const double* VL, const double* VR, double ch, int ix, int jx,
                        int kx, int dir, int type);

/* rk_tvd21/22, rk_std21/22: 2D_basic/rk.f90:9-131 ; 3D_basic/rk.f90:9-147 (dx == dy == dz) */
int omhd_rk_tvd21_2d(const double* U, double* U1, const double* F, const double* G, double dt,
                     double dx, int ix, int jx);
int omhd_rk_tvd22_2d(double* U, const double* U1, const double* F, const double* G, double dt,
                     double dx, int ix, int jx);
int omhd_rk_std21_2d(const double* U, double* U1, const double* F, const double* G, double dt,
                     double dx, int ix, int jx);
int omhd_rk_std22_2d(double* U, const double* F, const double* G, double dt, double dx, int ix, int jx);
int omhd_rk_tvd21_3d(const double* U, double* U1, const double* F, const double* G, const double* H,
                     double dt, double dx, int ix, int jx, int kx);
int omhd_rk_tvd22_3d(double* U, const double* U1, const double* F, const double* G, const double* H,
                     double dt, double dx, int ix, int jx, int kx);
int omhd_rk_std21_3d(const double* U, double* U1, const double* F, const double* G, const double* H,
                     double dt, double dx, int ix, int jx, int kx);
int omhd_rk_std22_3d(double* U, const double* F, const double* G, const double* H, double dt,
                     double dx, int ix, int jx, int kx);

/* glm_ss2: 2D_basic/glm_ss2.f90:1-39 (whole array incl. ghosts) ; 3D_basic/glm_ss2.f90 */
int omhd_glm_ss2_2d(double* U, double ch, double dt, int ix, int jx);
int omhd_glm_ss2_3d(double* U, double ch, double dt, int ix, int jx, int kx);

/* set_dt: 2D_basic/set_dt.f90:1-68 ; 3D_basic/set_dt.f90:1-74.  vmax (== ch) and dt out. */
int omhd_set_dt_2d(const double* U, const double* V, double* vmax, double* dt, double dx, double cfl,
                   int ix, int jx);
int omhd_set_dt_3d(const double* U, const double* V, double* vmax, double* dt, double dx, double cfl,
                   int ix, int jx, int kx);

/* set_dt_resistive: 2D_reconnection/flux_resistive.f90:18-25 (host scalar routine) */
int omhd_set_dt_resistive(double* dt, double dx, double cfl, int eta_kind);

/* bc: 2D_basic/bc.f90:1-16, 3D_basic/bc.f90 (all periodic) and the wall variants
 * 2D_KH/bc.f90:6-38, 2D_reconnection/bc.f90:6-50, 3D_reconnection_gpu/bc.cuf:7-98,
 * expressed as a kind and a sign-flip mask per side. */
int omhd_bc_2d(double* U, int ix, int jx, const int kind[4], const int flip[4]);
int omhd_bc_3d(double* U, int ix, int jx, int kx, const int kind[6], const int flip[6]);

/* face-state fix at the domain edges: main.f90:101-102,119-120 (periodic);
 * bc_for_F/G 2D_KH/bc.f90:42-83, 2D_reconnection/bc.f90:136-197;
 * bc_for_F/G/H 3D_reconnection_gpu/bc.cuf:103-218 */
int omhd_facefix_2d(double* VL, double* VR, int ix, int jx, int dir, int kind_lo, int flip_lo,
                    int kind_hi, int flip_hi);
int omhd_facefix_3d(double* VL, double* VR, int ix, int jx, int kx, int dir, int kind_lo,
                    int flip_lo, int kind_hi, int flip_hi);

/* flux_resistive: 2D_reconnection/flux_resistive.f90:27-115 ;
 * 3D_reconnection_gpu/flux_resistive.cuf:11-140 (x, y, z: cell-centre coordinates) */
int omhd_flux_resistive_2d(double* F, const double* U, const double* x, const double* y, double dx,
                           int ix, int jx, int dir, int eta_kind);
int omhd_flux_resistive_3d(double* F, const double* U, const double* x, const double* y,
                           const double* z, double dx, int ix, int jx, int kx, int dir, int eta_kind);

/* ======================================================================
 * gfortran link-level drop-ins for the 2D reference drivers
 * (2D_basic/main.f90 calls these names with these argument lists)
 * ==================================================================== */
void u2v_(const double* U, double* V, const int* ix, const int* jx);
void limiter_(const double* wk, double* wL, double* wR, const int* ix, const int* jx, const int* dir,
              const int* type);
void flux_solver_(double* F, const double* VL, const double* VR, const double* ch, const int* ix,
                  const int* jx, const int* dir, const int* type);
void rk_tvd21_(const double* U, double* U1, const double* F, const double* G, const double* dt,
               const double* dx, const int* ix, const int* jx);
void rk_tvd22_(double* U, const double* U1, const double* F, const double* G, const double* dt,
               const double* dx, const int* ix, const int* jx);
void rk_std21_(const double* U, double* U1, const double* F, const double* G, const double* dt,
               const double* dx, const int* ix, const int* jx);
void rk_std22_(double* U, const double* F, const double* G, const double* dt, const double* dx,
               const int* ix, const int* jx);
void glm_ss2_(double* U, const double* ch, const double* dt, const int* ix, const int* jx);
void set_dt_(const double* U, const double* V, double* vmax, double* dt, const double* dx,
             const double* cfl, const int* ix, const int* jx);
void bc_(double* U, const int* ix, const int* jx);
void flux_resistive_(double* F, const double* U, const double* x, const double* y, const double* dx,
                     const int* ix, const int* jx, const int* dir);
void set_dt_resistive_(double* dt, const double* dx, const double* cfl);

/* ======================================================================
 * Library control
 * ==================================================================== */
int omhd_abi_version(void);
/* stream used by the routine-level entry points (NULL = legacy default stream) */
int omhd_set_stream(void* cuda_stream);
/* reference semantics for the `_` drop-ins: 1 = print and exit(1) on failure (default) */
void omhd_set_abort_on_error(int on);
/* last failure of a routine-level call (synchronises the stream) */
int omhd_last_error(omhd_error_info* info);
void omhd_clear_error(void);
/* frees the cached device mirrors used for host-pointer calls */
void omhd_release_host_mirrors(void);
/* measured FP64 FMA throughput of the current GPU in GFLOP/s (roofline denominator;
 * no counterpart in the reference) */
int omhd_probe_fp64_peak(double* gflops);
/* TMA staging of halo tiles in the FP64 pipelined 2D stage kernel (no
 * counterpart in the reference): on by default; 0 makes the kernel load its
 * tiles with ordinary loads (same arithmetic, same results), for comparisons.
 * Library-global: set it before stepping, from one thread. */
void omhd_set_tma_staging(int enable);
/* The warp-specialised FP64 3D stage kernel (HLLD with minmod or MC; no
 * counterpart in the reference): off by default, where the one-role 3D kernel
 * runs (three CTA barriers per plane; the faster of the two on GB300); 1
 * selects the warp-specialised kernel (same scheme; results agree to
 * rounding).  Library-global: set it before stepping, from one thread. */
void omhd_set_3d_pipeline(int enable);
/* The warp-specialised FP64 2D stage kernel (HLLD with minmod or MC, no
 * resistivity; no counterpart in the reference): on by default; 0 selects the
 * one-role 2D kernel (same scheme; results agree to rounding), for
 * comparisons.  Library-global: set it before stepping, from one thread. */
void omhd_set_2d_pipeline(int enable);
/* measured FP32 FMA throughput of the current GPU in GFLOP/s (the FP32 roofline
 * denominator of the mixed-precision kernels; no counterpart in the reference) */
int omhd_probe_fp32_peak(double* gflops);
/* accuracy probe of the fast FP64 arithmetic of the performance kernels (no
 * counterpart in the reference): for n device doubles x, writes 5*n device
 * doubles to out, planes rcp_nr(x), 1.0/x, rsqrt_nr(x), sqrt_nr(x), sqrt(x)
 * (the second and last by the device's IEEE division and square root);
 * synchronous, on the default stream */
int omhd_probe_fastmath(const double* x_dev, long long n, double* out_dev);
/* probe of the integer-pipe binary32 <-> binary64 conversions of the
 * FP32-mixed kernels (no counterpart in the reference): for n device values,
 * nd_dev[i] = narrow(xd_dev[i]) and wf_dev[i] = widen(xf_dev[i]); synchronous,
 * on the default stream */
int omhd_probe_convert(const double* xd_dev, float* nd_dev, const float* xf_dev, double* wf_dev, long long n);

/* ======================================================================
 * Fused solver handle
 * ==================================================================== */
typedef struct omhd_solver omhd_solver;

typedef struct {
  int nd;              /* 2 or 3 */
  int ix, jx, kx;      /* array extents incl. one ghost per side (kx = 1 in 2D) */
  double dx, dy, dz;   /* spacings (the reference uses dx = dy = dz) */
  double x0, y0, z0;   /* lower domain corner: x(1) = x0 - dx/2 (2D_basic/model.f90:19-28) */
  double cfl;          /* CFL number (main.f90:15) */
  double gamma;        /* ratio of specific heats (param.h:3) */
  int lm_type;         /* OMHD_LM_* */
  int flux_type;       /* OMHD_FLUX_* */
  int time_type;       /* OMHD_TIME_* */
  int eta_kind;        /* OMHD_ETA_*: resistive fluxes + set_dt_resistive when != NONE */
  int bc_kind[6];      /* OMHD_BC_* per side */
  int bc_flip[6];      /* sign-flip masks per side (mirror sides) */
  int precision;       /* OMHD_PREC_* */
  double tend;         /* end time: steps stop at the first t >= tend (main.f90:73); <= 0: none */
} omhd_config;

typedef struct {
  double t;            /* simulation time */
  double dt;           /* last step's dt */
  double ch;           /* last step's GLM speed (== vmax) */
  double vmax_next;    /* fastest wave speed of the current state (next step's ch) */
  long long steps;     /* completed steps */
  int done;            /* 1 once t >= tend */
  int status;          /* first failure (omhd_status_t) */
} omhd_step_info;

/* model initial states (reference-style problem setups) */
typedef struct {
  int kind;            /* 0 Orszag-Tang (2D_basic/model.f90), 1 KH shear layer, 2 Harris sheet (3D),
                          3 2D reconnection (2D_reconnection/model.f90), 4 Brio-Wu (1D_basic/model.f90),
                          5 3D field loop (3D_basic/model.f90) */
  double amp;          /* OT: B amplitude scale (1); KH: shear speed; Harris: A_y amplitude;
                          reconnection: X-point perturbation b1; field loop: A amplitude */
  double bx0;          /* KH: uniform Bx */
  double phase_x, phase_y;  /* OT phase shifts (0, 0) */
  double beta;         /* Harris plasma beta */
  double pert;         /* KH: vy perturbation amplitude */
  uint64_t seed;       /* seeded deviates (SplitMix64) */
} omhd_model;

int omhd_solver_create(const omhd_config* cfg, omhd_solver** out);
int omhd_solver_destroy(omhd_solver* s);
/* stream for all work of this handle (NULL = the legacy default stream) */
int omhd_solver_set_stream(omhd_solver* s, void* cuda_stream);
/* Bind caller-owned device arrays (ix*jx*kx*9 doubles each) for the state U
 * and the stage buffer U1.  Unbound handles allocate their own. */
int omhd_solver_bind(omhd_solver* s, double* U_dev, double* U1_dev);
/* device pointer of the state array */
int omhd_solver_state_ptr(omhd_solver* s, double** U_dev);
/* copy a full state (ghosts included) in / out; host or device pointer.
 * put_state applies the boundary conditions and computes the first dt. */
int omhd_solver_put_state(omhd_solver* s, const double* U, double t);
int omhd_solver_get_state(omhd_solver* s, double* U);
/* One call for a driver whose state lives in host memory, the way the
 * reference's main loop (2D_basic/main.f90:56-188) holds U: put_state(U_in, t)
 * (U_in == NULL: continue from the state on the device), nsteps steps, and
 * get_state(U_out), returning the device error code like omhd_solver_sync.
 * With page-locked host buffers (cudaHostAlloc / cudaHostRegister) the upload
 * and the first-dt reduction are one pass over the host data, and the last
 * step writes its result into U_out as it stores it, so no separate copy
 * follows the steps; other buffers take the put_state / get_state copies.
 * U_in and U_out may be the same buffer.  Results are those of
 * put_state + step + get_state, bit for bit. */
int omhd_solver_step_host(omhd_solver* s, const double* U_in, double* U_out, double t, int nsteps);
/* fill the state with a model (2D_basic/model.f90 style), apply bc, compute dt */
int omhd_solver_init_model(omhd_solver* s, const omhd_model* m);
/* cell-centre coordinates (reference recurrence x(i) = x(i-1) + dx), host arrays */
int omhd_solver_coords(omhd_solver* s, double* x, double* y, double* z);
/* end time (main.f90:73): steps stop on the device at the first t >= tend; <= 0: none */
int omhd_solver_set_tend(omhd_solver* s, double tend);
/* enqueue n full steps (asynchronous: returns before the GPU finishes) */
int omhd_solver_step(omhd_solver* s, int nsteps);
/* capture n steps once into a CUDA graph and replay it `replays` times */
int omhd_solver_step_graph(omhd_solver* s, int nsteps, int replays);
/* wait for the GPU and read the step record; returns the first failure */
int omhd_solver_sync(omhd_solver* s, omhd_step_info* info);
int omhd_solver_last_error(omhd_solver* s, omhd_error_info* info);
/* kernels launched by the last omhd_solver_step call per step (for accounting) */
int omhd_solver_launches_per_step(omhd_solver* s);

/* ======================================================================
 * Ensembles of independent 2D problems (no counterpart in the reference,
 * which runs one problem per program): every member keeps its own grid size,
 * boundaries, model and dt; all members advance together with one persistent
 * batched kernel per RK stage.  Members must share nd = 2, the flux type
 * (HLLD) and the precision (OMHD_PREC_MIXED or OMHD_PREC_FP64).
 * ==================================================================== */
typedef struct omhd_ensemble omhd_ensemble;
int omhd_ensemble_create(const omhd_config* cfgs, int n, omhd_ensemble** out);
int omhd_ensemble_destroy(omhd_ensemble* e);
int omhd_ensemble_size(omhd_ensemble* e);
int omhd_ensemble_set_stream(omhd_ensemble* e, void* cuda_stream);
/* member i as a solver handle (state pointer, put/get state, coordinates) */
int omhd_ensemble_member(omhd_ensemble* e, int i, omhd_solver** s);
int omhd_ensemble_init_models(omhd_ensemble* e, const omhd_model* models);
/* tile_kind 0: 32x8, 1: 32x4, 2: 16x16, 3: 64x4, 4: 16x8 cells per CTA; CTAs = ctas_per_sm x SMs */
int omhd_ensemble_set_tiling(omhd_ensemble* e, int tile_kind, int ctas_per_sm);
/* time `steps` real steps per candidate tiling, each from the same ensemble
 * state (saved and restored: tuning leaves the states, times and step counts
 * unchanged; it allocates a copy of the ensemble's state pool meanwhile), and
 * keep the fastest */
int omhd_ensemble_autotune(omhd_ensemble* e, int steps, int* tile_kind, int* ctas_per_sm, double* ms_per_step);
int omhd_ensemble_step(omhd_ensemble* e, int nsteps);
int omhd_ensemble_step_graph(omhd_ensemble* e, int nsteps, int replays);
/* waits; infos (n entries, may be NULL) get every member's step record */
int omhd_ensemble_sync(omhd_ensemble* e, omhd_step_info* infos);

/* ======================================================================
 * Fused 2D step without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- drivers inside an
 * application whose framework owns the whole device memory pool, or jobs
 * that must reserve all device memory when the program loads.  The stage
 * buffer, step record, error word and coordinates live in one static device
 * array of omhd_step2d_noalloc_max_doubles() doubles (32 MiB) that every GPU
 * loading the library holds until exit; grids needing more scratch than that
 * (9*ix*jx + ix + jx + 64 doubles, about 419k cells) are rejected with
 * OMHD_BAD_ARG and a message in omhd_last_error().  U must be device memory
 * of the current device (ix*jx*9 doubles, reference layout; memory of another
 * device is refused with OMHD_BAD_ARG); bc is applied to it, then nsteps
 * steps run from time t0 on `stream`.  The call is synchronous: it reads the
 * step record back and waits for the stream before it returns, and a failure
 * the kernels record (negative pressure or density, dt too small) is returned
 * with its cell and value in omhd_last_error().  Every call reuses the same
 * array: calls that overlap on the GPU race.  Because every call copies the
 * step record to host memory and waits for its stream, no call may be made
 * while its stream is being captured into a CUDA graph.
 * ==================================================================== */
int omhd_step2d_noalloc(double* U_dev, const omhd_config* cfg, double t0, int nsteps, void* stream,
                        omhd_step_info* info);
size_t omhd_step2d_noalloc_max_doubles(void);

/* ======================================================================
 * Snapshot files (2D_basic/fileio.f90:16-115, 3D_basic/fileio.f90:16-122):
 * the reference's stream layout, native byte order:
 *   t | ix, jx[, kx] (int32) | x, y[, z] | U: 9 planes (mx..ps) | V: vx vy vz pr
 * Arrays may be host or device memory.  V may be NULL: it is then computed
 * from U on the GPU (u2v.f90), and a failing u2v (negative pressure or
 * density) is returned without writing.  fileio_input reads t, x, y[, z] and
 * U and rejects a file whose sizes differ (fileio.f90:77-82) with
 * OMHD_BAD_ARG; a missing or short file gives OMHD_IO_ERR, and the output
 * arrays may then hold part of the file (omhd_solver_read reads into its own
 * buffers first, so a failed restart leaves the solver as it was).  The
 * reference's readers read these files unchanged.
 * ==================================================================== */
int omhd_fileio_output(const char* path, int nd, int ix, int jx, int kx, double t, const double* x,
                       const double* y, const double* z, const double* U, const double* V);
int omhd_fileio_input(const char* path, int nd, int ix, int jx, int kx, double* t, double* x, double* y,
                      double* z, double* U);
/* a solver's state, primitives, coordinates and time to a snapshot file, and
 * restart from one (put_state with the file's t) */
int omhd_solver_write(omhd_solver* s, const char* path);
int omhd_solver_read(omhd_solver* s, const char* path);

/* ======================================================================
 * Reverse mode through time (no counterpart in the reference).  The
 * gradient of a scalar functional J(U_N) with respect to the initial state
 * U_0 of `nsteps` fused FP64 TVD-RK2 steps (2D, HLLD, minmod or MC, GLM,
 * periodic or mirror boundaries).  Hand-written adjoint kernels per RK stage
 * replay each face's HLLD branch and each limiter selection as the forward
 * took them (a fixed subgradient at limiter kinks); dt and ch of every step
 * are recorded by the forward run and held fixed.  States are kept every
 * `checkpoint_every` steps; the backward pass recomputes one segment of
 * steps at a time with the fused kernels, recording that segment's decision
 * tape (sqrt(N) checkpointing when checkpoint_every ~ sqrt(N)).
 * Arrays are device memory in the reference layout (9 planes of ix*jx).
 * ==================================================================== */
typedef struct omhd_adjoint omhd_adjoint;
/* cfg: nd = 2, flux HLLD, limiter minmod or MC, TVD-RK2, no resistivity;
 * the precision field is ignored (the forward runs the fp64 kernels). */
int omhd_adjoint_create(const omhd_config* cfg, int nsteps, int checkpoint_every, omhd_adjoint** out);
int omhd_adjoint_destroy(omhd_adjoint* a);
int omhd_adjoint_set_stream(omhd_adjoint* a, void* cuda_stream);
/* bc is applied to a copy of U0 (U0 is not modified); U_N goes to UN (may be NULL) */
int omhd_adjoint_forward(omhd_adjoint* a, const double* U0_dev, double* UN_dev);
/* gU0 = (dU_N/dU_0)^T gUN, zero at ghost cells; needs a preceding forward */
int omhd_adjoint_backward(omhd_adjoint* a, const double* gUN_dev, double* gU0_dev);
/* forward run that also records every step's decision tape (limiter
 * selections and HLLD branches; about 44 bytes per cell per step), then
 * replayed by omhd_adjoint_replay: the same steps from another U0 with every
 * decision and every {dt, ch, glm factor} frozen to the recorded run's -- the
 * smooth map whose derivative omhd_adjoint_backward computes (finite
 * differences of it straddle no limiter or branch kink). */
int omhd_adjoint_record(omhd_adjoint* a, const double* U0_dev, double* UN_dev);
int omhd_adjoint_replay(omhd_adjoint* a, const double* U0_dev, double* UN_dev);
/* adjoint of one step given its stage inputs Un (before the first GLM half)
 * and U1 (after bc); log3_dev = {dt, ch, glm factor} on the device; the
 * decisions are recomputed from Un and U1.  lam_in is dJ/dU_{n+1}; it is
 * overwritten (its boundary ring folds in the ghosts). */
int omhd_adjoint_step_vjp(omhd_adjoint* a, const double* Un_dev, const double* U1_dev, const double* log3_dev,
                          double* lam_in_dev, double* lam_out_dev);
/* waits; returns the first device-reported failure of the forward steps */
int omhd_adjoint_sync(omhd_adjoint* a);
/* {dt, ch, glm factor} of each step of the last forward run (3*nsteps doubles) */
int omhd_adjoint_step_log(omhd_adjoint* a, double* log3_host);
/* device bytes held by the handle (checkpoints, segment and work buffers) */
int omhd_adjoint_memory(omhd_adjoint* a, size_t* bytes);

#ifdef __cplusplus
}
#endif
#endif /* OPENMHD_GB300_H */
