// omhd_runtime.h -- host-side runtime shared by the translation units of
// libopenmhd_gb300.so: the library stream, the error record, the device
// mirrors used when a routine-level entry point receives host pointers.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>

#include "../../include/openmhd_gb300.h"

namespace omhd {

struct DevError;

// library-wide state for the routine-level entry points
cudaStream_t lib_stream();
DevError* lib_dev_error();           // device error word (lazily allocated)
unsigned long long* lib_dev_accum(); // device scalar accumulator for reductions
void set_host_error(int code, int i, int j, int k, double value, const char* msg);
int finish_status(int code);         // records + honours abort-on-error for '_' wrappers
bool abort_on_error();

// Resolve one array argument: device pointers pass through, host pointers get
// a device mirror (copied in when `copy_in`, copied back by release()).
class ArgSet {
 public:
  ArgSet() = default;
  ~ArgSet();
  // returns a device pointer usable by kernels, or nullptr on failure
  double* add(const double* p, size_t count, bool copy_in, bool copy_out);
  // copy results back to host arrays; synchronise when any host array was used
  int finish();
  bool any_host() const { return any_host_; }
  int status() const { return status_; }

 private:
  struct Slot {
    double* host;
    double* dev;
    size_t count;
    bool out;
  };
  Slot slots_[8];
  int n_ = 0;
  bool any_host_ = false;
  int status_ = 0;
};

int cuda_status(cudaError_t e, const char* where);

}  // namespace omhd
