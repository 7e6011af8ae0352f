// omhd_fused3d_mixed.cu -- 3D fused stage kernels, arithmetic variant "mixed"
// (face arithmetic in float).
#define OMHD_VARIANT v_mixed
#define OMHD_FAST true
#include "omhd_fused3d.cuh"

namespace omhd {
int launch_stage3d_mixed(const StageArgs& a, cudaStream_t s) { return v_mixed::d3::launch_variant3d<float>(a, s); }
}  // namespace omhd
