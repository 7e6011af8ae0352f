// omhd_fused2d_parity.cu -- 2D fused stage kernels, arithmetic variant "parity"
// (face arithmetic in double; built with --fmad=false so the op sequence is the reference's).
#define OMHD_VARIANT v_parity
#define OMHD_FAST false
#include "omhd_fused2d.cuh"

namespace omhd {
int launch_stage2d_parity(const StageArgs& a, cudaStream_t s) { return v_parity::launch_variant<double>(a, s); }
}  // namespace omhd
