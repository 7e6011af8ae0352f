// omhd_fused2d_mixed.cu -- 2D fused stage kernels, arithmetic variant "mixed"
// (face arithmetic in float).
#define OMHD_VARIANT v_mixed
#define OMHD_FAST true
#include "omhd_fused2d.cuh"

namespace omhd {
int launch_stage2d_mixed(const StageArgs& a, cudaStream_t s) { return v_mixed::launch_variant<float>(a, s); }
}  // namespace omhd
