// placeholder launchers for 3D
#include "omhd_fused.h"
#include "../../include/openmhd_gb300.h"
namespace omhd {
int launch_stage3d_fp64(const StageArgs&, cudaStream_t) { return 801; }
int launch_stage3d_parity(const StageArgs&, cudaStream_t) { return 801; }
int launch_stage3d_mixed(const StageArgs&, cudaStream_t) { return 801; }
}
