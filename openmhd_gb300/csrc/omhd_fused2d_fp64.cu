// omhd_fused2d_fp64.cu -- 2D fused stage kernels, arithmetic variant "fp64"
// (face arithmetic in double).
#define OMHD_VARIANT v_fp64
#define OMHD_FAST true
#include "omhd_fused2d.cuh"

namespace omhd {
int launch_stage2d_fp64(const StageArgs& a, cudaStream_t s) { return v_fp64::launch_variant<double>(a, s); }
}  // namespace omhd
