// peaks.cu -- FP64 / FP32 FMA issue-rate measurement used as the roofline
// denominators of the sweep kernels (the pool's measured-peaks file carries
// only HBM bandwidth and bf16 tensor throughput).  Eight independent FMA
// chains per thread, 8 blocks of 256 threads per SM, timed with CUDA events.
#include <cuda_runtime.h>

#include "../../include/surfatt_gb300.h"

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double run(int blocks, int iters) {
  T* d = nullptr;
  if (cudaMalloc(&d, (size_t)blocks * 256 * sizeof(T)) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, 256>>>(d, iters / 10, (T)0.999, (T)1e-3);  // warm-up
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, 256>>>(d, iters, (T)0.999, (T)1e-3);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (cudaGetLastError() != cudaSuccess || ms <= 0) return -1;
  const double fma = (double)blocks * 256 * iters * 64;
  return 2.0 * fma / (ms * 1e-3) / 1e12;  // TFLOP/s, an FMA counted as 2 flops
}

}  // namespace

extern "C" surfatt_status_t surfatt_measure_peaks(int device, double* fp64_tflops,
                                                  double* fp32_tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return SURFATT_CUDA_ERROR;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return SURFATT_CUDA_ERROR;
  const double f64 = run<double>(nsm * 8, 1000);
  const double f32 = run<float>(nsm * 8, 20000);
  if (f64 <= 0 || f32 <= 0) return SURFATT_CUDA_ERROR;
  if (fp64_tflops) *fp64_tflops = f64;
  if (fp32_tflops) *fp32_tflops = f32;
  return SURFATT_OK;
}
