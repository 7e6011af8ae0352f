// omhd_fused2d_mixed.cu -- 2D fused stage kernels, arithmetic variant "mixed"
// (face arithmetic in float).
#define OMHD_VARIANT v_mixed
#define OMHD_FAST true
#include "omhd_fused2d.cuh"

namespace omhd {
int launch_stage2d_mixed(const StageArgs& a, cudaStream_t s) { return v_mixed::launch_variant<float>(a, s); }
}  // namespace omhd

namespace omhd {
int launch_batch2d_mixed(int flux, int tile_kind, const StageArgs* args_dev, int* tile_start_dev, int ngrids,
                      int total_tiles, int ctas, cudaStream_t s) {
  return v_mixed::launch_batch_variant<float>(flux, tile_kind, args_dev, tile_start_dev, ngrids, total_tiles, ctas, s);
}
}  // namespace omhd
