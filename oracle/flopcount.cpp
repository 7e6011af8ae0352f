// flopcount.cpp -- flop-counting build of the CPU oracle (test/measurement
// infrastructure only).  The oracle source is compiled with `double` replaced
// by a counting type, so every arithmetic operation of the reference's step on
// a real state is tallied:
//   add, sub, mul, div, sqrt, exp, cosh, tanh, sin, cos = 1 flop;
//   negation, abs, sign (copysign), min, max, compare = 0 flops.
// The face reconstruction and flux work of a step (limiters, face fixes,
// Riemann solver, resistive face terms: the part the FP32-mixed kernels run in
// FP32) is tallied apart from the rest (u2v, CFL, GLM, RK update, bc: the FP64
// residual of the mixed kernels), and within the rest the conserved-to-
// primitive recoveries (u2v), which the mixed kernels run in FP32 where the
// internal energy is at least the kinetic plus magnetic energy.
// Usage: flopcount <nx> <ny> <steps> [kh|ot]
//        flopcount <nx> <ny> <nz> <steps> harris   (3D resistive Harris sheet)
// (prints flops per cell-update, total and split)
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

static unsigned long long g_count[3] = {0, 0, 0};
static int g_region = 0;  // 1 inside the face-flux part of a step, 2 inside u2v
#define g_flops g_count[g_region]

struct cd {
  double v;
  cd() = default;
  constexpr cd(double x) : v(x) {}
};
static_assert(sizeof(cd) == sizeof(double), "counting type must be layout compatible");

inline cd operator+(cd a, cd b) { ++g_flops; return cd(a.v + b.v); }
inline cd operator-(cd a, cd b) { ++g_flops; return cd(a.v - b.v); }
inline cd operator*(cd a, cd b) { ++g_flops; return cd(a.v * b.v); }
inline cd operator/(cd a, cd b) { ++g_flops; return cd(a.v / b.v); }
inline cd operator-(cd a) { return cd(-a.v); }
inline cd operator+(cd a) { return a; }
inline cd& operator+=(cd& a, cd b) { ++g_flops; a.v += b.v; return a; }
inline bool operator<(cd a, cd b) { return a.v < b.v; }
inline bool operator>(cd a, cd b) { return a.v > b.v; }
inline bool operator<=(cd a, cd b) { return a.v <= b.v; }
inline bool operator>=(cd a, cd b) { return a.v >= b.v; }
inline bool operator==(cd a, cd b) { return a.v == b.v; }
inline bool operator!=(cd a, cd b) { return a.v != b.v; }
inline cd sqrt(cd a) { ++g_flops; return cd(std::sqrt(a.v)); }
inline cd exp(cd a) { ++g_flops; return cd(std::exp(a.v)); }
inline cd cosh(cd a) { ++g_flops; return cd(std::cosh(a.v)); }
inline cd tanh(cd a) { ++g_flops; return cd(std::tanh(a.v)); }
inline cd sin(cd a) { ++g_flops; return cd(std::sin(a.v)); }
inline cd cos(cd a) { ++g_flops; return cd(std::cos(a.v)); }
inline cd atan(cd a) { ++g_flops; return cd(std::atan(a.v)); }
inline cd fabs(cd a) { return cd(std::fabs(a.v)); }
inline cd copysign(cd a, cd b) { return cd(std::copysign(a.v, b.v)); }

#define OMO_FLUX_REGION(on) (g_region = (on))
#define OMO_U2V_REGION(on) (g_region = (on) ? 2 : 0)
#define double cd
#include "omhd_oracle.c"
#undef double
#undef g_flops

static void report(const char* what, int nx, int ny, int nz, int steps) {
  const double cells = (double)nx * ny * nz * steps;
  const unsigned long long tot = g_count[0] + g_count[1] + g_count[2];
  printf("workload: %s %dx%dx%d, %d steps\n", what, nx, ny, nz, steps);
  printf("total_flops: %llu\n", tot);
  printf("flops_per_cell_update: %.1f\n", (double)tot / cells);
  printf("face_flux_flops_per_cell_update: %.1f\n", (double)g_count[1] / cells);
  printf("rest_flops_per_cell_update: %.1f\n", (double)(g_count[0] + g_count[2]) / cells);
  printf("u2v_flops_per_cell_update: %.1f\n", (double)g_count[2] / cells);
}

static int harris(int nx, int ny, int nz, int steps) {
  omo_cfg c;
  memset(&c, 0, sizeof c);
  c.ix = nx + 2;
  c.jx = ny + 2;
  c.kx = nz + 2;
  c.nd = 3;
  c.dx = cd(200.0 / nx);
  c.dy = (200.0 / nx == 100.0 / ny) ? c.dx : cd(100.0 / ny);
  c.dz = (200.0 / nx == 200.0 / nz) ? c.dx : cd(200.0 / nz);
  c.cfl = cd(0.4);
  c.gamma = cd(5.0 / 3.0);
  c.lm_type = 2;
  c.flux_type = 3;
  c.eta_kind = OMO_ETA_HARRIS_XZ;
  c.bc.kind[4] = c.bc.kind[5] = OMO_BC_MIRROR;  // conducting z walls: mz and Bz change sign
  c.bc.flip[4] = c.bc.flip[5] = (1 << OMO_MZ) | (1 << OMO_BZ);
  omo_model m;
  memset(&m, 0, sizeof m);
  m.kind = 2;
  m.beta = cd(0.2);
  m.amp = cd(2.0e-3);
  m.seed = 0;
  m.x0 = cd(-100.0);
  m.y0 = cd(-50.0);
  m.z0 = cd(-100.0);
  const size_t n = (size_t)c.ix * c.jx * c.kx;
  std::vector<cd> U(9 * n), ws(omo_workspace_doubles(&c)), x(c.ix), y(c.jx), z(c.kx);
  omo_grid(x.data(), c.ix, cd(-100.0), c.dx);
  omo_grid(y.data(), c.jx, cd(-50.0), c.dy);
  omo_grid(z.data(), c.kx, cd(-100.0), c.dz);
  omo_model_fill(&m, U.data(), x.data(), y.data(), z.data(), c.ix, c.jx, c.kx, c.dx, c.dy, c.dz);
  omo_bc(U.data(), c.ix, c.jx, c.kx, 3, &c.bc);
  cd t(0.0), dt(0.0), ch(0.0);
  omo_err e;
  g_count[0] = g_count[1] = g_count[2] = 0;
  g_region = 0;
  for (int s = 0; s < steps; ++s) {
    if (omo_step(&c, U.data(), ws.data(), x.data(), y.data(), z.data(), &t, &dt, &ch, &e)) {
      fprintf(stderr, "step failed\n");
      return 1;
    }
  }
  report("harris-sheet-3d", nx, ny, nz, steps);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 5 && strcmp(argv[5], "harris") == 0) return harris(atoi(argv[1]), atoi(argv[2]), atoi(argv[3]), atoi(argv[4]));
  const int nx = argc > 1 ? atoi(argv[1]) : 4096;
  const int ny = argc > 2 ? atoi(argv[2]) : 2048;
  const int steps = argc > 3 ? atoi(argv[3]) : 2;
  const bool ot = argc > 4 && strcmp(argv[4], "ot") == 0;
  omo_cfg c;
  memset(&c, 0, sizeof c);
  c.ix = nx + 2;
  c.jx = ny + 2;
  c.kx = 1;
  c.nd = 2;
  c.cfl = cd(0.4);
  c.gamma = cd(5.0 / 3.0);
  c.flux_type = 3;
  c.time_type = 0;
  c.eta_kind = 0;
  omo_model m;
  memset(&m, 0, sizeof m);
  double x0, y0;
  if (ot) {  // Orszag-Tang, MC limiter, periodic
    const double two_pi = 8.0 * std::atan(1.0);
    c.dx = cd(two_pi / nx);
    c.dy = (nx == ny) ? c.dx : cd(two_pi / ny);
    c.lm_type = 2;
    for (int q = 0; q < 6; ++q) c.bc.kind[q] = OMO_BC_PERIODIC;
    m.kind = 0;
    m.amp = cd(1.0);
    x0 = 0.0;
    y0 = 0.0;
  } else {  // KH shear layer, minmod, zero-gradient y walls
    c.dx = cd(40.0 / nx);
    c.dy = (nx == ny) ? c.dx : cd(40.0 / ny);
    c.lm_type = 1;
    c.bc.kind[2] = c.bc.kind[3] = OMO_BC_MIRROR;
    m.kind = 1;
    m.amp = cd(0.5);
    m.bx0 = cd(0.2);
    m.pert = cd(0.01);
    m.seed = 0;
    x0 = 0.0;
    y0 = -20.0;
  }
  c.dz = c.dx;
  const size_t n = (size_t)c.ix * c.jx;
  std::vector<cd> U(9 * n), ws(omo_workspace_doubles(&c)), x(c.ix), y(c.jx), z(1);
  omo_grid(x.data(), c.ix, cd(x0), c.dx);
  omo_grid(y.data(), c.jx, cd(y0), c.dy);
  z[0] = cd(0.0);
  omo_model_fill(&m, U.data(), x.data(), y.data(), z.data(), c.ix, c.jx, 1, c.dx, c.dy, c.dz);
  omo_bc(U.data(), c.ix, c.jx, 1, 2, &c.bc);
  cd t(0.0), dt(0.0), ch(0.0);
  omo_err e;
  g_count[0] = g_count[1] = g_count[2] = 0;
  g_region = 0;
  for (int s = 0; s < steps; ++s) {
    if (omo_step(&c, U.data(), ws.data(), x.data(), y.data(), z.data(), &t, &dt, &ch, &e)) {
      fprintf(stderr, "step failed\n");
      return 1;
    }
  }
  report(ot ? "orszag-tang" : "kelvin-helmholtz", nx, ny, 1, steps);
  return 0;
}
