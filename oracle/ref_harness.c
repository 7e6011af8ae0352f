/*
 * ref_harness.c -- snapshot recorder linked into the C translation of a
 * reference problem directory (oracle/ref.py, oracle/f90sub.py).
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the product links or loads it.
 *
 * The reference's driver (main.f90) writes a field file at the top of each
 * loop iteration whose time has reached the next output time
 * (2D_basic/main.f90:62-70).  The translation turns that call,
 * fileio_output(filename,ix,jx,[kx,]t,x,y,[z,]U,V), into a call of
 * ref_snapshot_2d / ref_snapshot_3d with the same arrays plus dx, dt and ch,
 * and this file keeps a copy of each snapshot in memory for the tests.
 */
#include <stdlib.h>
#include <string.h>

typedef struct {
  int ix, jx, kx;
  double t, dx, dt, ch;
  double *x, *y, *z, *U;
} ref_snap;

static ref_snap* g_snaps = NULL;
static int g_count = 0, g_cap = 0;

static double* dup(const double* a, long n) {
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  if (p) memcpy(p, a, sizeof(double) * (size_t)n);
  return p;
}

static void record(int ix, int jx, int kx, const double* t, const double* x, const double* y, const double* z,
                   const double* U, const double* dx, const double* dt, const double* ch) {
  if (g_count == g_cap) {
    int cap = g_cap ? 2 * g_cap : 16;
    ref_snap* p = (ref_snap*)realloc(g_snaps, sizeof(ref_snap) * (size_t)cap);
    if (!p) return;
    g_snaps = p;
    g_cap = cap;
  }
  ref_snap* s = &g_snaps[g_count++];
  s->ix = ix;
  s->jx = jx;
  s->kx = kx;
  s->t = *t;
  s->dx = *dx;
  s->dt = *dt;
  s->ch = *ch;
  s->x = dup(x, ix);
  s->y = dup(y, jx);
  s->z = z ? dup(z, kx) : NULL;
  s->U = dup(U, 9L * ix * jx * kx);
}

void ref_snapshot_2d(int* ix, int* jx, double* t, double* x, double* y, double* U, double* V, double* dx,
                     double* dt, double* ch) {
  (void)V;
  record(*ix, *jx, 1, t, x, y, NULL, U, dx, dt, ch);
}

void ref_snapshot_3d(int* ix, int* jx, int* kx, double* t, double* x, double* y, double* z, double* U, double* V,
                     double* dx, double* dt, double* ch) {
  (void)V;
  record(*ix, *jx, *kx, t, x, y, z, U, dx, dt, ch);
}

/* Initial state injected into a 2D driver in place of its model (the
 * benchmark runs the reference's driver from the configuration's own initial
 * state): set by ref_set_initial_2d, consumed by the translated driver's call
 * of model(U,V,x,y,dx,ix,jx), which REF_MODEL_HOOK routes here. */
#ifdef REF_MODEL_HOOK_2D
void f90_model(double*, double*, double*, double*, double*, int*, int*);
void f90_u2v(double*, double*, int*, int*);
static double *g_init_U = NULL, *g_init_x = NULL, *g_init_y = NULL, g_init_dx = 0.0;
static int g_init_ix = 0, g_init_jx = 0;

int ref_set_initial_2d(const double* U, const double* x, const double* y, double dx, int ix, int jx) {
  free(g_init_U);
  free(g_init_x);
  free(g_init_y);
  g_init_U = g_init_x = g_init_y = NULL;
  if (!U) return 0; /* clear: the driver's own model again */
  g_init_U = dup(U, 9L * ix * jx);
  g_init_x = dup(x, ix);
  g_init_y = dup(y, jx);
  g_init_dx = dx;
  g_init_ix = ix;
  g_init_jx = jx;
  return (g_init_U && g_init_x && g_init_y) ? 0 : 1;
}

void ref_model_2d(double* U, double* V, double* x, double* y, double* dx, int* ix, int* jx) {
  if (!g_init_U || *ix != g_init_ix || *jx != g_init_jx) {
    f90_model(U, V, x, y, dx, ix, jx);
    return;
  }
  memcpy(U, g_init_U, sizeof(double) * 9UL * (size_t)(*ix) * (size_t)(*jx));
  memcpy(x, g_init_x, sizeof(double) * (size_t)(*ix));
  memcpy(y, g_init_y, sizeof(double) * (size_t)(*jx));
  *dx = g_init_dx;
  f90_u2v(U, V, ix, jx); /* the primitives the driver's first set_dt reads */
}
#endif

int ref_snap_count(void) { return g_count; }

/* dims = {ix, jx, kx}; vals = {t, dx, dt, ch} */
int ref_snap_info(int k, int* dims, double* vals) {
  if (k < 0 || k >= g_count) return 1;
  const ref_snap* s = &g_snaps[k];
  dims[0] = s->ix;
  dims[1] = s->jx;
  dims[2] = s->kx;
  vals[0] = s->t;
  vals[1] = s->dx;
  vals[2] = s->dt;
  vals[3] = s->ch;
  return 0;
}

/* U: 9*ix*jx*kx doubles; x, y, z: the coordinate arrays (z may be NULL) */
int ref_snap_copy(int k, double* U, double* x, double* y, double* z) {
  if (k < 0 || k >= g_count) return 1;
  const ref_snap* s = &g_snaps[k];
  memcpy(U, s->U, sizeof(double) * 9UL * (size_t)s->ix * (size_t)s->jx * (size_t)s->kx);
  if (x) memcpy(x, s->x, sizeof(double) * (size_t)s->ix);
  if (y) memcpy(y, s->y, sizeof(double) * (size_t)s->jx);
  if (z && s->z) memcpy(z, s->z, sizeof(double) * (size_t)s->kx);
  return 0;
}

void ref_snap_clear(void) {
  for (int k = 0; k < g_count; ++k) {
    free(g_snaps[k].x);
    free(g_snaps[k].y);
    free(g_snaps[k].z);
    free(g_snaps[k].U);
  }
  g_count = 0;
}
