// omhd_common.cuh -- shared constants, layout and device helpers.
//
// State layout in HBM is the reference's: column-major U(ix,jx[,kx],var) with
// i fastest and the variable slowest (param.h:6-15), so each of the nine
// variables is one contiguous plane and every 32-thread row segment is a
// coalesced load.  Ghost width is one cell per side, as in the reference.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/openmhd_gb300.h"

namespace omhd {

constexpr int NV = 9;
// conserved slots (param.h:6-15, 0-based)
constexpr int MX = 0, MY = 1, MZ = 2, EN = 3, RO = 4, BX = 5, BY = 6, BZ = 7, PS = 8;
// primitive slots reuse 0..3 (param.h:7-10)
constexpr int VX = 0, VY = 1, VZ = 2, PR = 3;

// Fortran sign(a,b) == copysign(|a|,b) with signed zero honoured.
template <class T>
__host__ __device__ __forceinline__ T fsign(T a, T b) {
  return copysign(fabs(a), b);
}
// Fortran min/max on ordered (non-NaN) operands: first operand wins ties.
template <class T>
__host__ __device__ __forceinline__ T fmin2(T a, T b) {
  return (b < a) ? b : a;
}
template <class T>
__host__ __device__ __forceinline__ T fmax2(T a, T b) {
  return (b > a) ? b : a;
}

// Ordered-bits max for non-negative doubles: integer order of the bit pattern
// equals numeric order, so atomicMax on the bits is a max on the values.
__device__ __forceinline__ void atomic_max_pos_double(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Device error record: the first failure wins (atomicCAS on code), the
// offending cell and value are recorded for the host.  Kernels never trap.
struct DevError {
  int code;
  int i, j, k;
  int instance;
  int pad;
  double value;
};

__device__ __forceinline__ void raise_error(DevError* e, int code, int i, int j, int k, int inst,
                                            double value) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->i = i;
    e->j = j;
    e->k = k;
    e->instance = inst;
    e->value = value;
  }
}

// SplitMix64 (Steele, Lea & Flood 2014) applied twice to (seed, n) -> [-1,1).
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ double uniform_pm1(uint64_t seed, uint64_t n) {
  const uint64_t h = splitmix64(splitmix64(seed) ^ n);
  return (double)(h >> 11) * 0x1.0p-52 - 1.0;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace omhd
