// omhd_fused3d_parity.cu -- 3D fused stage kernels, arithmetic variant "parity"
// (face arithmetic in double; built with --fmad=false so the op sequence is the reference's).
#define OMHD_VARIANT v_parity
#define OMHD_FAST false
#include "omhd_fused3d.cuh"

namespace omhd {
int launch_stage3d_parity(const StageArgs& a, cudaStream_t s) { return v_parity::d3::launch_variant3d<double>(a, s); }
}  // namespace omhd
