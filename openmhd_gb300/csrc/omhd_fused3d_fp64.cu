// omhd_fused3d_fp64.cu -- 3D fused stage kernels, arithmetic variant "fp64"
// (face arithmetic in double).
#define OMHD_VARIANT v_fp64
#define OMHD_FAST true
#include "omhd_fused3d.cuh"

namespace omhd {
int launch_stage3d_fp64(const StageArgs& a, cudaStream_t s) { return v_fp64::d3::launch_variant3d<double>(a, s); }
}  // namespace omhd
