/*
 * omhd_oracle.h -- CPU restatement of OpenMHD's finite-volume MHD step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (openmhd_gb300/) links,
 * loads or calls this code; only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py use it, to check results against.
 *
 * Parity status: PINNED.  The reference (zenitani/OpenMHD) is Fortran 90 and
 * ships no tests, fixtures or golden vectors, and no Fortran compiler exists
 * where this project is built.  oracle/ref.py therefore translates the
 * reference's own source files (the routines, model.f90 and main.f90 of
 * 2D_basic, 2D_KH, 2D_reconnection and 3D_basic) mechanically into C
 * (oracle/f90sub.py) and builds them into oracle/_ref/; tests/
 * test_ref_translation.py runs those reference drivers and routines and
 * requires this restatement to give the same bits (every limiter, flux and
 * time integrator, the HLLD branches, walls, resistivity, 2D and 3D), and
 * tests/test_ref_golden.py checks it against fixtures recorded from them.
 * This file follows the reference routine by routine, in the reference's
 * operation order (every function cites the file:line it restates), and is
 * compiled with -ffp-contract=off so that each Fortran expression maps to the
 * same sequence of IEEE-754 double operations.
 *
 * Array layout is the reference's: Fortran column-major U(ix,jx[,kx],var) with
 * i fastest and the variable index slowest.  2D arrays are 3D arrays with
 * kx == 1.  Indices in this API are 0-based (reference index minus one).
 */
#ifndef OMHD_ORACLE_H
#define OMHD_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* variable slots, param.h:6-15 (0-based) */
enum { OMO_MX = 0, OMO_MY, OMO_MZ, OMO_EN, OMO_RO, OMO_BX, OMO_BY, OMO_BZ, OMO_PS };
enum { OMO_VX = 0, OMO_VY, OMO_VZ, OMO_PR };

/* status codes (shared numbering with the product's omhd_status_t) */
enum {
  OMO_OK = 0,
  OMO_NEG_PRESSURE = 1,
  OMO_NEG_DENSITY = 2,
  OMO_DT_TOO_SMALL = 3,
  OMO_BAD_ARG = 4
};

/* boundary side kinds */
enum { OMO_BC_PERIODIC = 0, OMO_BC_MIRROR = 1 };

typedef struct {
  /* side order: west(x-), east(x+), south(y-), north(y+), down(z-), up(z+) */
  int kind[6];
  /* bit v set => variable slot v changes sign in the mirrored ghost / face state */
  int flip[6];
} omo_bcspec;

typedef struct {
  int code;       /* OMO_* */
  int i, j, k;    /* 0-based location of the offending cell (minloc / maxloc) */
  double value;   /* offending value */
} omo_err;

/* eta (resistivity) kinds */
enum { OMO_ETA_NONE = 0, OMO_ETA_RECON2D = 1, OMO_ETA_HARRIS_XZ = 2 };

typedef struct {
  int ix, jx, kx, nd;     /* array extents incl. one ghost per side; nd = 2 or 3 */
  double dx, dy, dz;      /* cell spacings */
  double cfl;
  double gamma;
  int lm_type;            /* 0 flat, 1 minmod, 2 MC, 3 van Leer, 4 Koren */
  int flux_type;          /* 0 LLF, 1 HLL, 2 HLLC, 3 HLLD, 4 LHLLD */
  int time_type;          /* 0 TVD-RK2, 1 standard RK2 */
  int eta_kind;           /* OMO_ETA_* ; resistive fluxes when != NONE */
  omo_bcspec bc;
} omo_cfg;

void omo_set_gamma(double gamma);
double omo_get_gamma(void);

/* routine-level restatements (reference routine names) */
int omo_u2v(const double* U, double* V, int ix, int jx, int kx, omo_err* err);
void omo_limiter(const double* wk, double* wL, double* wR, int ix, int jx, int kx, int dir, int type);
void omo_flux_solver(double* F, const double* VL, const double* VR, double ch,
                     int ix, int jx, int kx, int dir, int type);
void omo_rk_tvd21(const double* U, double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd);
void omo_rk_tvd22(double* U, const double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd);
void omo_rk_std21(const double* U, double* U1, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd);
void omo_rk_std22(double* U, const double* F, const double* G, const double* H,
                  double dt, double dx, double dy, double dz, int ix, int jx, int kx, int nd);
void omo_glm_ss2(double* U, double ch, double dt, int ix, int jx, int kx);
int omo_set_dt(const double* U, const double* V, double* vmax, double* dt, double dx, double dy,
               double dz, double cfl, int ix, int jx, int kx, int nd, omo_err* err);
void omo_set_dt_resistive(double* dt, double dx, double cfl, int eta_kind);
void omo_bc(double* U, int ix, int jx, int kx, int nd, const omo_bcspec* bc);
void omo_facefix(double* VL, double* VR, int ix, int jx, int kx, int dir, const omo_bcspec* bc);
double omo_eta(int eta_kind, double x, double y, double z);
/* HLLD branch histogram of the serial build (FL, FR, HLLC-G L/R, L*, R*, L**, R**) */
void omo_branch_counts(long long out[8], int reset);
void omo_flux_resistive(double* F, const double* U, const double* x, const double* y,
                        const double* z, double dx, int ix, int jx, int kx, int nd, int dir,
                        int eta_kind);

/* One full step of the reference driver loop body (2D_basic/main.f90:56-188,
 * 3D_basic/main.f90 time loop).  U is advanced in place; *t += dt.  ws must
 * hold omo_workspace_doubles(cfg) = 6*9*n + 4*n doubles, n = ix*jx*kx
 * (U1, VL, VR, F, G, H, V).
 * x, y, z are cell-centre coordinates (used by resistive runs only).
* Returns OMO_OK or the first failure; *dt_out and *ch_out get dt and ch. */
int omo_step(const omo_cfg* cfg, double* U, double* ws, const double* x, const double* y,
             const double* z, double* t, double* dt_out, double* ch_out, omo_err* err);
size_t omo_workspace_doubles(const omo_cfg* cfg);

/* Counter-based uniform deviate in [-1, 1): SplitMix64 (Steele, Lea & Flood
 * 2014) finaliser applied twice to (seed, n).  Identical on host and device. */
double omo_uniform_pm1(uint64_t seed, uint64_t n);

/* models: fill x,y,z and U (all cells incl. ghosts), then the caller applies bc. */
typedef struct {
  int kind;            /* 0 Orszag-Tang, 1 KH shear layer (zero-gradient y), 2 Harris sheet 3D,
                          3 2D reconnection, 4 Brio-Wu, 5 3D field loop */
  double amp;          /* OT: B amplitude scale; KH: shear speed; Harris: perturbation amplitude */
  double bx0;          /* KH: guide Bx */
  double phase_x, phase_y;  /* OT phase shifts */
  double beta;         /* Harris beta */
  double pert;         /* KH perturbation amplitude */
  uint64_t seed;
  double x0, y0, z0;   /* domain lower corner */
} omo_model;

void omo_grid(double* x, int n, double x0, double d);
void omo_model_fill(const omo_model* m, double* U, const double* x, const double* y,
                    const double* z, int ix, int jx, int kx, double dx, double dy, double dz);

#ifdef __cplusplus
}
#endif
#endif
