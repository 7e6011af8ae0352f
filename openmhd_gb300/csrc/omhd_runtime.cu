// omhd_runtime.cu -- library stream, error record and host-pointer mirrors for
// the routine-level entry points of libopenmhd_gb300.so.
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "omhd_common.cuh"
#include "omhd_fastmath.h"
#include "omhd_runtime.h"
#include "omhd_tma.h"

namespace omhd {

namespace {
cudaStream_t g_stream = nullptr;
DevError* g_dev_error = nullptr;
unsigned long long* g_dev_accum = nullptr;
bool g_abort = true;
omhd_error_info g_last = {};

struct PoolSlot {
  double* dev = nullptr;
  size_t cap = 0;
};
PoolSlot g_pool[8];
}  // namespace

cudaStream_t lib_stream() { return g_stream; }

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return OMHD_OK;
  char msg[160];
  snprintf(msg, sizeof msg, "CUDA error in %s: %s", where, cudaGetErrorString(e));
  set_host_error(OMHD_CUDA_ERR, 0, 0, 0, 0.0, msg);
  return OMHD_CUDA_ERR;
}

DevError* lib_dev_error() {
  if (!g_dev_error) {
    if (cudaMalloc(&g_dev_error, sizeof(DevError)) != cudaSuccess) return nullptr;
    cudaMemsetAsync(g_dev_error, 0, sizeof(DevError), g_stream);
  }
  return g_dev_error;
}

unsigned long long* lib_dev_accum() {
  if (!g_dev_accum) {
    if (cudaMalloc(&g_dev_accum, sizeof(unsigned long long)) != cudaSuccess) return nullptr;
  }
  return g_dev_accum;
}

void set_host_error(int code, int i, int j, int k, double value, const char* msg) {
  if (g_last.code != OMHD_OK) return;  // keep the first failure
  g_last.code = code;
  g_last.i = i;
  g_last.j = j;
  g_last.k = k;
  g_last.instance = 0;
  g_last.value = value;
  snprintf(g_last.message, sizeof g_last.message, "%s", msg ? msg : "");
}

bool abort_on_error() { return g_abort; }

int finish_status(int code) {
  if (code != OMHD_OK && g_abort) {
    fprintf(stdout, " %s\n", g_last.message);
    fflush(stdout);
    exit(1);
  }
  return code;
}

ArgSet::~ArgSet() {}

double* ArgSet::add(const double* p, size_t count, bool copy_in, bool copy_out) {
  if (status_) return nullptr;
  if (!p) {
    status_ = OMHD_BAD_ARG;
    return nullptr;
  }
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
    return const_cast<double*>(p);
  }
  if (n_ >= 8) {
    status_ = OMHD_BAD_ARG;
    return nullptr;
  }
  PoolSlot& ps = g_pool[n_];
  if (ps.cap < count) {
    if (ps.dev) cudaFree(ps.dev);
    ps.dev = nullptr;
    ps.cap = 0;
    if (cuda_status(cudaMalloc(&ps.dev, count * sizeof(double)), "host mirror allocation")) {
      status_ = OMHD_CUDA_ERR;
      return nullptr;
    }
    ps.cap = count;
  }
  if (copy_in) {
    if (cuda_status(cudaMemcpyAsync(ps.dev, p, count * sizeof(double), cudaMemcpyHostToDevice, g_stream),
                    "host mirror copy-in")) {
      status_ = OMHD_CUDA_ERR;
      return nullptr;
    }
  }
  slots_[n_] = Slot{const_cast<double*>(p), ps.dev, count, copy_out};
  ++n_;
  any_host_ = true;
  return ps.dev;
}

int ArgSet::finish() {
  if (status_) return status_;
  for (int s = 0; s < n_; ++s) {
    if (!slots_[s].out) continue;
    if (cuda_status(cudaMemcpyAsync(slots_[s].host, slots_[s].dev, slots_[s].count * sizeof(double),
                                    cudaMemcpyDeviceToHost, g_stream),
                    "host mirror copy-out"))
      return OMHD_CUDA_ERR;
  }
  if (any_host_) {
    if (cuda_status(cudaStreamSynchronize(g_stream), "stream synchronize")) return OMHD_CUDA_ERR;
  }
  return cuda_status(cudaGetLastError(), "kernel launch");
}

// FP64 fused multiply-add throughput probe: 8 independent DFMA chains per
// thread, 2 flops per DFMA.  Used as the FP64 roofline denominator.
// DFMA throughput probe: 8 independent FMA chains per thread whose operands
// all live in registers (a constant-bank operand lowers the issue rate of
// DFMA on this part), 8 CTAs of 256 threads per SM.
__global__ void k_dfma_probe(double* out, double seed, int iters, int flag) {
  const double b = seed * 1.0000001 + threadIdx.x * 1e-9;
  const double c = 0.999999 + blockIdx.x * 1e-12;
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + k * 1e-3 + threadIdx.x * 1e-7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) sum += a[k];
  if (flag) out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

// FP32 FMA throughput probe, the same shape as the FP64 one: the FP32
// roofline denominator of the mixed-precision kernels.
__global__ void k_ffma_probe(float* out, float seed, int iters, int flag) {
  const float b = seed * 1.0000001f + threadIdx.x * 1e-9f;
  const float c = 0.999999f + blockIdx.x * 1e-12f;
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0f + k * 1e-3f + threadIdx.x * 1e-7f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
  }
  float sum = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) sum += a[k];
  if (flag) out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

// The fast FP64 reciprocal, reciprocal square root and square root of the
// performance kernels beside the device's IEEE division and square root, for
// accuracy tests: out holds five planes of n values each,
// rcp_nr(x), 1.0/x, rsqrt_nr(x), sqrt_nr(x), sqrt(x).
__global__ void k_fastmath_probe(const double* __restrict__ x, long long n, double* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    out[i] = rcp_nr(v);
    out[n + i] = 1.0 / v;
    out[2 * n + i] = rsqrt_nr(v);
    out[3 * n + i] = sqrt_nr(v);
    out[4 * n + i] = sqrt(v);
  }
}

__global__ void k_convert_probe(const double* __restrict__ xd, float* __restrict__ nd, const float* __restrict__ xf,
                                double* __restrict__ wf, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    nd[i] = narrow_f64(xd[i]);
    wf[i] = widen_f32(xf[i]);
  }
}

static std::atomic<int> g_tma_on{1};
bool tma_staging_enabled() { return g_tma_on.load(std::memory_order_relaxed) != 0; }
static std::atomic<int> g_pipe3d_on{0};
bool pipe3d_enabled() { return g_pipe3d_on.load(std::memory_order_relaxed) != 0; }
static std::atomic<int> g_pipe2d_on{1};
bool pipe2d_enabled() { return g_pipe2d_on.load(std::memory_order_relaxed) != 0; }

int tma_encode_state_map(CUtensorMap* map, const double* U, int ix, int jx, int nv, int box_x, int box_y) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    else
      cudaGetLastError();
  });
  if (!encode || !map || !U) return 1;
  // row pitch and base must be 16-byte aligned; the box's inner extent too
  if ((ix & 1) || (reinterpret_cast<uintptr_t>(U) & 15) || ((box_x * 8) & 15)) return 2;
  if (box_x > 256 || box_y > 256 || nv > 256 || box_x > ix || box_y > jx) return 3;
  const cuuint64_t dims[3] = {(cuuint64_t)ix, (cuuint64_t)jx, (cuuint64_t)nv};
  const cuuint64_t strides[2] = {(cuuint64_t)ix * 8, (cuuint64_t)ix * (cuuint64_t)jx * 8};
  const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, (cuuint32_t)nv};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(U), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : 4;
}

}  // namespace omhd

using namespace omhd;

extern "C" {

void omhd_set_tma_staging(int enable) { g_tma_on.store(enable ? 1 : 0, std::memory_order_relaxed); }
void omhd_set_3d_pipeline(int enable) { g_pipe3d_on.store(enable ? 1 : 0, std::memory_order_relaxed); }
void omhd_set_2d_pipeline(int enable) { g_pipe2d_on.store(enable ? 1 : 0, std::memory_order_relaxed); }

int omhd_probe_fastmath(const double* x, long long n, double* out) {
  if (!x || !out || n < 0) return OMHD_BAD_ARG;
  if (n == 0) return OMHD_OK;
  cudaPointerAttributes ax, ao;
  if (cudaPointerGetAttributes(&ax, x) != cudaSuccess || cudaPointerGetAttributes(&ao, out) != cudaSuccess ||
      ax.type != cudaMemoryTypeDevice || ao.type != cudaMemoryTypeDevice) {
    cudaGetLastError();
    set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "fast-math probe: x and out must be device memory");
    return OMHD_BAD_ARG;
  }
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_fastmath_probe<<<(unsigned)blocks, 256>>>(x, n, out);
  if (cuda_status(cudaGetLastError(), "fast-math probe launch")) return OMHD_CUDA_ERR;
  return cuda_status(cudaDeviceSynchronize(), "fast-math probe");
}

int omhd_probe_convert(const double* xd, float* nd, const float* xf, double* wf, long long n) {
  if (!xd || !nd || !xf || !wf || n < 0) return OMHD_BAD_ARG;
  if (n == 0) return OMHD_OK;
  const void* ptrs[4] = {xd, nd, xf, wf};
  for (const void* p : ptrs) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      set_host_error(OMHD_BAD_ARG, 0, 0, 0, 0.0, "conversion probe: all four arrays must be device memory");
      return OMHD_BAD_ARG;
    }
  }
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_convert_probe<<<(unsigned)blocks, 256>>>(xd, nd, xf, wf, n);
  if (cuda_status(cudaGetLastError(), "conversion probe launch")) return OMHD_CUDA_ERR;
  return cuda_status(cudaDeviceSynchronize(), "conversion probe");
}

int omhd_probe_fp64_peak(double* gflops) {
  if (!gflops) return OMHD_BAD_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return OMHD_CUDA_ERR;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 2048;
  double* out = nullptr;
  if (cuda_status(cudaMalloc(&out, sizeof(double) * blocks * threads), "probe allocation")) return OMHD_CUDA_ERR;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_probe<<<blocks, threads>>>(out, 1.0, iters, 0);  // warm-up
  double best = 0.0;
  for (int r = 0; r < 5; ++r) {  // best of five launches (burst rate)
    cudaEventRecord(e0);
    k_dfma_probe<<<blocks, threads>>>(out, 1.0, iters, 0);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = (double)blocks * threads * (double)iters * 8 * 2;
    if (ms > 0 && flops / (ms * 1e6) > best) best = flops / (ms * 1e6);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = best;
  return cuda_status(cudaGetLastError(), "probe kernel");
}

int omhd_probe_fp32_peak(double* gflops) {
  if (!gflops) return OMHD_BAD_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return OMHD_CUDA_ERR;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 16384;
  float* out = nullptr;
  if (cuda_status(cudaMalloc(&out, sizeof(float) * blocks * threads), "probe allocation")) return OMHD_CUDA_ERR;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_ffma_probe<<<blocks, threads>>>(out, 1.0f, iters, 0);  // warm-up
  double best = 0.0;
  for (int r = 0; r < 5; ++r) {  // best of five launches (burst rate)
    cudaEventRecord(e0);
    k_ffma_probe<<<blocks, threads>>>(out, 1.0f, iters, 0);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = (double)blocks * threads * (double)iters * 8 * 2;
    if (ms > 0 && flops / (ms * 1e6) > best) best = flops / (ms * 1e6);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *gflops = best;
  return cuda_status(cudaGetLastError(), "probe kernel");
}

int omhd_abi_version(void) { return OMHD_ABI_VERSION; }

int omhd_set_stream(void* s) {
  g_stream = (cudaStream_t)s;
  return OMHD_OK;
}

void omhd_set_abort_on_error(int on) { g_abort = on != 0; }

int omhd_last_error(omhd_error_info* info) {
  if (g_stream || g_dev_error) cudaStreamSynchronize(g_stream);
  if (info) *info = g_last;
  return g_last.code;
}

void omhd_clear_error(void) {
  memset(&g_last, 0, sizeof g_last);
  if (g_dev_error) {
    cudaMemsetAsync(g_dev_error, 0, sizeof(DevError), g_stream);
    cudaStreamSynchronize(g_stream);
  }
}

void omhd_release_host_mirrors(void) {
  for (auto& ps : g_pool) {
    if (ps.dev) cudaFree(ps.dev);
    ps.dev = nullptr;
    ps.cap = 0;
  }
}

}  // extern "C"
