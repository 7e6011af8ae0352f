// omhd_fused2d_fp64.cu -- 2D fused stage kernels, arithmetic variant "fp64"
// (face arithmetic in double).
#define OMHD_VARIANT v_fp64
#define OMHD_FAST true
#include "omhd_fused2d.cuh"

namespace omhd {
// HLLD with minmod or MC runs the tape-recording instantiation with recording
// switched off (null tape pointers): one machine code for the plain and the
// recording step, so a recorded run reproduces a plain run bit for bit.
int launch_stage2d_fp64(const StageArgs& a, cudaStream_t s) {
  if (a.flux_type == FX_HLLD && (a.lm_type == LM_MINMOD || a.lm_type == LM_MC)) {
    StageArgs b = a;
    b.tlim = nullptr;
    b.tface = nullptr;
    if (a.eta_kind == OMHD_ETA_NONE && pipe2d_enabled())
      return v_fp64::launch_pipe<FX_HLLD, tape::kRecord>(b, s);
    return v_fp64::launch_one<double, FX_HLLD, tape::kRecord>(b, s);
  }
  return v_fp64::launch_variant<double>(a, s);
}
int launch_stage2d_fp64_tape(const StageArgs& a, int mode, cudaStream_t s) {
  if (a.flux_type != FX_HLLD || a.nd != 2 || !a.tlim || !a.tface) return (int)cudaErrorInvalidValue;
  if (a.lm_type != LM_MINMOD && a.lm_type != LM_MC) return (int)cudaErrorInvalidValue;
  if (mode == tape::kRecord) {
    if (a.eta_kind == OMHD_ETA_NONE) return v_fp64::launch_pipe<FX_HLLD, tape::kRecord>(a, s);
    return v_fp64::launch_one<double, FX_HLLD, tape::kRecord>(a, s);
  }
  if (mode == tape::kReplay) return v_fp64::launch_one<double, FX_HLLD, tape::kReplay>(a, s);
  return (int)cudaErrorInvalidValue;
}
}  // namespace omhd

namespace omhd {
int launch_batch2d_fp64(int flux, int tile_kind, const StageArgs* args_dev, int* tile_start_dev, int ngrids,
                      int total_tiles, int ctas, cudaStream_t s) {
  return v_fp64::launch_batch_variant<double>(flux, tile_kind, args_dev, tile_start_dev, ngrids, total_tiles, ctas, s);
}
}  // namespace omhd
