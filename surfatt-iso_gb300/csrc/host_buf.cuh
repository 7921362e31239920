// host_buf.cuh -- host-side helpers shared by the C-ABI translation units:
// a CUDA-call check that returns SURFATT_CUDA_ERROR, and a grow-only device
// buffer.
#pragma once
#include <cstdio>

#include <cuda_runtime.h>

#include "../../include/surfatt_gb300.h"

namespace sgb {

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      std::fprintf(stderr, "surfatt_gb300: %s failed: %s (%s:%d)\n", #call,       \
                   cudaGetErrorString(e_), __FILE__, __LINE__);                  \
      return SURFATT_CUDA_ERROR;                                                 \
    }                                                                            \
  } while (0)

// Grow-only device buffer.
struct DBuf {
  void* p = nullptr;
  size_t cap = 0;
  size_t* counter = nullptr;  // engine allocation counter (budget), may be null
  int ensure(size_t bytes) {
    if (bytes <= cap) return SURFATT_OK;
    release();
    size_t want = bytes < 256 ? 256 : bytes;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      p = nullptr;
      cap = 0;
      cudaGetLastError();
      return SURFATT_OOM;
    }
    cap = want;
    if (counter) *counter += cap;
    return SURFATT_OK;
  }
  void release() {
    if (p) {
      cudaFree(p);
      if (counter) *counter -= cap;
    }
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// Status bookkeeping of the drop-in symbols (surfatt_last_status /
// surfatt_last_iterations) and the `stop` switch (surfatt_set_exit_on_boundary),
// defined in capi.cu.
int host_record(int status, int iters);
bool host_exit_on_stop();

}  // namespace sgb
