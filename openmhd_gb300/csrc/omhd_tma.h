// omhd_tma.h -- tensor-memory-accelerator (TMA) staging of halo tiles:
// mbarrier and cp.async.bulk.tensor wrappers (inline PTX, sm_90+ forms that
// sm_103a keeps) and the host-side tensor-map encoder.
//
// A stage kernel stages the conserved state of a halo tile, all nine planes,
// with one 3D tiled TMA load: the tensor map views U (column-major, i fastest,
// variable slowest) as a 3D tensor {ix, jx, 9} and the box is
// {box_x, box_y, 9}.  Rules kept here (a violation faults, nothing checks them
// before the copy runs):
//   - the innermost coordinate times 8 bytes is a multiple of 16 (x even), and
//     box_x * 8 is a multiple of 16;
//   - the row pitch ix * 8 is a multiple of 16 (ix even) and the base address
//     is 16-byte aligned (checked by the encoder, which refuses otherwise);
//   - the shared-memory destination is 128-byte aligned.
// Loads only: no TMA store or reduce is issued, and no multicast form is used.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace omhd {

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  // make the initialised barrier visible to the async (TMA) proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// the generic-proxy accesses of shared memory ordered before the next async-proxy write
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// true once the barrier's phase `parity` has completed; bounded: gives up
// after max_tries polls (each poll may suspend the thread briefly)
__device__ __forceinline__ bool mbar_wait_parity(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t k = 0; k < max_tries; ++k) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 3D tiled TMA load of the box at coordinates (x, y, z) into shared memory,
// completing `bytes` transaction bytes on `bar`
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
#endif

// Host: encode the tensor map of a state array U (nv planes of ix*jx doubles)
// for boxes of box_x * box_y cells of every plane.  Returns 0, or a nonzero
// code when TMA cannot be used for this array (odd ix, unaligned base, driver
// entry point missing) -- the caller then uses ordinary loads.
int tma_encode_state_map(CUtensorMap* map, const double* U, int ix, int jx, int nv, int box_x, int box_y);

// Library-wide switch of TMA staging (on by default); tests compare the
// staged and the ordinary-load paths bit for bit.
bool tma_staging_enabled();

// Library-wide switch of the warp-specialised FP64 3D stage kernel (on by
// default; off: the one-role kernel), for comparisons in tests.
bool pipe3d_enabled();
bool pipe2d_enabled();

}  // namespace omhd
