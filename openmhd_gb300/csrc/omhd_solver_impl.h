// omhd_solver_impl.h -- internal layout of the fused solver handle, shared by
// the translation units that build on it (the ensemble driver).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/openmhd_gb300.h"
#include "omhd_fused.h"

namespace omhd {
struct StepState;
struct DevError;
}  // namespace omhd

struct omhd_solver {
  omhd_config cfg;
  size_t n = 0;  // cells per variable plane
  double* U = nullptr;
  double* U1 = nullptr;
  bool own_state = false;
  double* xc = nullptr;  // device coordinates
  double* yc = nullptr;
  double* zc = nullptr;
  std::vector<double> hx, hy, hz;
  omhd::StepState* st = nullptr;
  omhd::DevError* err = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int iso = 1;
  double dmin = 0;
  int last_status = OMHD_OK;
  omhd_error_info last = {};
};

namespace omhd {
// argument block of stage 1 or 2 of a solver's current step
StageArgs make_stage_args(const omhd_solver* s, int stage);
// the checks omhd_solver_create makes before any GPU work: OMHD_OK,
// OMHD_BAD_ARG or OMHD_NOT_SUPPORTED
int validate_config(const omhd_config* c);
}  // namespace omhd
