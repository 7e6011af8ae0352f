// omhd_fused.h -- host-visible argument blocks and launchers of the fused
// stage kernels.  Each arithmetic variant lives in its own translation unit
// (compiled with its own floating-point flags) and exports one launcher.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

namespace omhd {

struct StepState;
struct DevError;

struct StageArgs {
  const double* Uin;    // state the fluxes are built from (stage 1: U, stage 2: U1)
  const double* Ubase;  // state the update starts from (U; its psi gets the GLM factor)
  const double* U1;     // stage 2 (TVD): the stage-1 result, else nullptr
  double* Uout;         // stage 1: U1 ; stage 2: U (in place)
  int ix, jx, kx;       // extents incl. ghosts (kx = 1 in 2D)
  int nd;
  double dx, dy, dz;
  double dtx_scale;     // 1.0, or 0.5 for the first stage of standard RK2 (rk.f90:76)
  double gamma;
  int lm_type, flux_type, time_type, stage, iso;
  int bc_kind[6], bc_flip[6];
  int eta_kind;
  const double* xc;     // cell-centre coordinates (resistive runs)
  const double* yc;
  const double* zc;
  StepState* st;
  DevError* err;
  double cfl, dmin;     // for the end-of-step dt planning
  // decision tape of this stage (taped FP64 HLLD launches only; see omhd_tape.h):
  // limiter codes [2 directions][NV][cells], HLLD codes [2 directions][cells]
  // indexed by the face's lower cell
  unsigned char* tlim;
  unsigned short* tface;
  // stage 2 of the last step of omhd_solver_step_host: the result is also
  // written here (the device address of page-locked host memory), else nullptr
  double* Uhost;
  // derived on the host by stage_args_derived (the stage kernels read them
  // instead of dividing in every CTA): dtx_scale/dx, /dy, /dz;
  // 1/(gamma-1), gamma/(gamma-1) (flux_solver.f90:38-39) in FP64 and, with
  // gamma, rounded to binary32 for the FP32 face arithmetic
  double sdx, sdy, sdz;
  double gm1, r1, r2;  // gamma - 1 (u2v.f90:11), 1/(gamma-1), gamma/(gamma-1)
  float gamma_f, gm1_f, r1_f, r2_f;
};

// fills the derived fields of a once dx, dy, dtx_scale and gamma are set
inline void stage_args_derived(StageArgs& a) {
  a.sdx = a.dtx_scale / a.dx;
  a.sdy = a.dtx_scale / a.dy;
  a.sdz = a.dtx_scale / a.dz;
  a.gm1 = a.gamma - 1.0;
  a.r1 = 1.0 / (a.gamma - 1.0);
  a.r2 = a.gamma / (a.gamma - 1.0);
  a.gamma_f = (float)a.gamma;
  a.gm1_f = (float)a.gm1;
  a.r1_f = (float)a.r1;
  a.r2_f = (float)a.r2;
}

// launchers: return 0 or a CUDA error code
int launch_stage2d_fp64(const StageArgs& a, cudaStream_t s);
int launch_stage2d_parity(const StageArgs& a, cudaStream_t s);
int launch_stage2d_mixed(const StageArgs& a, cudaStream_t s);
// fp64 HLLD stage with a decision tape: mode tape::kRecord or tape::kReplay
int launch_stage2d_fp64_tape(const StageArgs& a, int mode, cudaStream_t s);
// ensemble launchers: tile_kind 0: 32x8, 1: 32x4, 2: 16x16, 3: 64x4, 4: 16x8 cells per CTA
int launch_batch2d_fp64(int flux, int tile_kind, const StageArgs* args_dev, int* tile_start_dev, int ngrids,
                        int total_tiles, int ctas, cudaStream_t s);
int launch_batch2d_mixed(int flux, int tile_kind, const StageArgs* args_dev, int* tile_start_dev, int ngrids,
                         int total_tiles, int ctas, cudaStream_t s);
constexpr int kBatchTileKinds = 5;
inline void batch_tile_dims(int kind, int* tx, int* ty) {
  static const int d[kBatchTileKinds][2] = {{32, 8}, {32, 4}, {16, 16}, {64, 4}, {16, 8}};
  const int k = (kind >= 0 && kind < kBatchTileKinds) ? kind : 0;
  *tx = d[k][0];
  *ty = d[k][1];
}
// the most CTAs per SM a batched kernel of this tile kind is built for
// (FP32-mixed: 160-thread tiles four, 288-thread tiles two; FP64: two)
inline int batch_max_ctas(int kind, bool mixed) { return (mixed && (kind == 1 || kind == 4)) ? 4 : 2; }
// Kernels with more than 48 KB of dynamic shared memory need the attribute
// set on every device that launches them: once per (kernel, device), tracked
// in the caller's bit mask (devices 0..63; beyond that, every launch sets it).
template <class K>
inline int set_smem_attr_once(K kernel, size_t bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ULL << dev) : 0ULL;
  if (bit && (done.load(std::memory_order_relaxed) & bit)) return 0;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return (int)e;
  done.fetch_or(bit, std::memory_order_relaxed);
  return 0;
}

int launch_stage3d_fp64(const StageArgs& a, cudaStream_t s);
int launch_stage3d_parity(const StageArgs& a, cudaStream_t s);
int launch_stage3d_mixed(const StageArgs& a, cudaStream_t s);

}  // namespace omhd
