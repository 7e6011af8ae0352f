// omhd_fused3d_fp64.cu -- 3D fused stage kernels, arithmetic variant "fp64"
// (face arithmetic in double).
#define OMHD_VARIANT v_fp64
#define OMHD_FAST true
#include "omhd_fused3d.cuh"
#include "omhd_fused3d_pipe.cuh"
#include "omhd_tma.h"

namespace omhd {
// HLLD with minmod or MC: the warp-specialised kernel; the other schemes: the
// one-role kernel
int launch_stage3d_fp64(const StageArgs& a, cudaStream_t s) {
  if (a.flux_type == FX_HLLD && (a.lm_type == LM_MINMOD || a.lm_type == LM_MC) && pipe3d_enabled())
    return v_fp64::d3p::launch_pipe3d<FX_HLLD>(a, s);
  return v_fp64::d3::launch_variant3d<double>(a, s);
}
}  // namespace omhd
