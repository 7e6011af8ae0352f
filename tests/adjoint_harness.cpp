// Test harness: exposes the adjoint face derivatives of
// openmhd_gb300/csrc/omhd_adjoint_face.h to Python (ctypes) for checks
// against finite differences of the oracle's fluxes.  Built by the tests with g++.
#include "../openmhd_gb300/csrc/omhd_adjoint_face.h"

using namespace omhd::adj;

extern "C" {
void h_hlld_vjp(int dir, const double* L, const double* R, double ch, double gamma, const double* gF, double* gL,
                double* gR) {
  if (dir == 1) hlld_vjp<1>(L, R, ch, gamma, gF, gL, gR);
  if (dir == 2) hlld_vjp<2>(L, R, ch, gamma, gF, gL, gR);
  if (dir == 3) hlld_vjp<3>(L, R, ch, gamma, gF, gL, gR);
}
void h_recon_vjp(int type, double wm, double w0, double wp, double gl, double gr, double* g3) {
  recon_vjp(type, wm, w0, wp, gl, gr, g3[0], g3[1], g3[2]);
}
void h_u2v_vjp(const double* U, double gamma, const double* gw, double* gU) { u2v_vjp(U, gamma, gw, gU); }
}
