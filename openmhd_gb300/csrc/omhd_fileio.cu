// omhd_fileio.cu -- snapshot files in the reference's format, and restart.
//
// The layout is the stream file of fileio_output / fileio_input
// (2D_basic/fileio.f90:16-115, 3D_basic/fileio.f90:16-122), native byte order,
// no record markers (access='stream'):
//   t (f64) | ix, jx [, kx] (int32) | x(ix), y(jx) [, z(kx)] (f64) |
//   U: mx my mz en ro bx by bz ps (one plane each, i fastest) |
//   V: vx vy vz pr (one plane each)
// U and V planes are the in-memory layout of the state, so each block is one
// contiguous write.  The reference's readers (fileio_input, the plotting
// scripts' data_read) read these files unchanged.
#include <cstdio>
#include <cstring>
#include <vector>

#include "omhd_common.cuh"
#include "omhd_solver_impl.h"

namespace {
using omhd::NV;

bool is_device_ptr(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// count doubles of `src` (host or device) written to `f`, in chunks
bool write_doubles(FILE* f, const double* src, size_t count) {
  if (!is_device_ptr(src)) return fwrite(src, sizeof(double), count, f) == count;
  const size_t chunk = (size_t)1 << 24;  // 128 MiB staging
  std::vector<double> buf(count < chunk ? count : chunk);
  for (size_t off = 0; off < count; off += buf.size()) {
    const size_t n = (count - off < buf.size()) ? count - off : buf.size();
    if (cudaMemcpy(buf.data(), src + off, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    if (fwrite(buf.data(), sizeof(double), n, f) != n) return false;
  }
  return true;
}

bool read_doubles(FILE* f, double* dst, size_t count) {
  if (!is_device_ptr(dst)) return fread(dst, sizeof(double), count, f) == count;
  const size_t chunk = (size_t)1 << 24;
  std::vector<double> buf(count < chunk ? count : chunk);
  for (size_t off = 0; off < count; off += buf.size()) {
    const size_t n = (count - off < buf.size()) ? count - off : buf.size();
    if (fread(buf.data(), sizeof(double), n, f) != n) return false;
    if (cudaMemcpy(dst + off, buf.data(), n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return false;
  }
  return true;
}

}  // namespace

extern "C" {

int omhd_fileio_output(const char* path, int nd, int ix, int jx, int kx, double t, const double* x, const double* y,
                       const double* z, const double* U, const double* V) {
  if (!path || !x || !y || !U || (nd != 2 && nd != 3) || ix < 1 || jx < 1) return OMHD_BAD_ARG;
  if (nd == 3 && (!z || kx < 1)) return OMHD_BAD_ARG;
  if (nd == 2) kx = 1;
  const size_t n = (size_t)ix * jx * kx;
  // primitives: the caller's, or u2v of U on the GPU (u2v.f90)
  double* Vown = nullptr;
  std::vector<double> Vhost;
  if (!V) {
    const bool dev = is_device_ptr(U);
    if (dev) {
      if (cudaMalloc(&Vown, sizeof(double) * 4 * n) != cudaSuccess) return OMHD_CUDA_ERR;
    } else {
      Vhost.resize(4 * n);
    }
    double* Vt = dev ? Vown : Vhost.data();
    const int st = (nd == 2) ? omhd_u2v_2d(U, Vt, ix, jx) : omhd_u2v_3d(U, Vt, ix, jx, kx);
    if (st != OMHD_OK) {
      if (Vown) cudaFree(Vown);
      return st;
    }
    if (dev && cudaDeviceSynchronize() != cudaSuccess) {
      cudaFree(Vown);
      return OMHD_CUDA_ERR;
    }
    V = Vt;
  }
  FILE* f = fopen(path, "wb");
  if (!f) {
    if (Vown) cudaFree(Vown);
    return OMHD_IO_ERR;
  }
  const int32_t dims[3] = {ix, jx, kx};
  bool ok = fwrite(&t, sizeof t, 1, f) == 1 && fwrite(dims, sizeof(int32_t), nd, f) == (size_t)nd;
  ok = ok && write_doubles(f, x, ix) && write_doubles(f, y, jx) && (nd == 2 || write_doubles(f, z, kx));
  ok = ok && write_doubles(f, U, NV * n) && write_doubles(f, V, 4 * n);
  ok = (fclose(f) == 0) && ok;
  if (Vown) cudaFree(Vown);
  return ok ? OMHD_OK : OMHD_IO_ERR;
}

int omhd_fileio_input(const char* path, int nd, int ix, int jx, int kx, double* t, double* x, double* y, double* z,
                      double* U) {
  if (!path || !t || !x || !y || !U || (nd != 2 && nd != 3) || ix < 1 || jx < 1) return OMHD_BAD_ARG;
  if (nd == 3 && (!z || kx < 1)) return OMHD_BAD_ARG;
  if (nd == 2) kx = 1;
  FILE* f = fopen(path, "rb");
  if (!f) return OMHD_IO_ERR;
  int32_t dims[3] = {0, 0, 1};
  bool ok = fread(t, sizeof *t, 1, f) == 1 && fread(dims, sizeof(int32_t), nd, f) == (size_t)nd;
  if (ok && (dims[0] != ix || dims[1] != jx || (nd == 3 && dims[2] != kx))) {  // fileio.f90:77-82
    fclose(f);
    return OMHD_BAD_ARG;
  }
  const size_t n = (size_t)ix * jx * kx;
  ok = ok && read_doubles(f, x, ix) && read_doubles(f, y, jx) && (nd == 2 || read_doubles(f, z, kx));
  ok = ok && read_doubles(f, U, NV * n);
  fclose(f);
  return ok ? OMHD_OK : OMHD_IO_ERR;
}

int omhd_solver_write(omhd_solver* s, const char* path) {
  if (!s || !path || !s->U) return OMHD_BAD_ARG;
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return OMHD_CUDA_ERR;
  double t = 0.0;
  {
    omhd_step_info info;
    const int st = omhd_solver_sync(s, &info);
    if (st) return st;
    t = info.t;
  }
  const omhd_config& c = s->cfg;
  return omhd_fileio_output(path, c.nd, c.ix, c.jx, c.kx, t, s->hx.data(), s->hy.data(), s->hz.data(), s->U,
                            nullptr);
}

int omhd_solver_read(omhd_solver* s, const char* path) {
  if (!s || !path) return OMHD_BAD_ARG;
  const omhd_config& c = s->cfg;
  std::vector<double> U((size_t)NV * s->n), x(c.ix), y(c.jx), z(c.kx);
  double t = 0.0;
  const int r = omhd_fileio_input(path, c.nd, c.ix, c.jx, c.kx, &t, x.data(), y.data(), z.data(), U.data());
  if (r) return r;
  const int p = omhd_solver_put_state(s, U.data(), t);
  if (p) return p;
  return (cudaStreamSynchronize(s->stream) == cudaSuccess) ? OMHD_OK : OMHD_CUDA_ERR;
}

}  // extern "C"
