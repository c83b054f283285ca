// FMA throughput probe used for the compute roof of the FP64 and FP32 kernels:
// independent FMA chains in registers, no memory traffic.
#include <cuda_runtime.h>

#include "wumingpic_gb300.h"

namespace {

template <typename T>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
int run(int iters, double* gflops) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const dim3 grid(nsm * 16), block(256);
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * grid.x * block.x) != cudaSuccess) return WPIC_CUDA_ERROR;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T><<<grid, block>>>(out, iters / 10, (T)0.999, (T)0.001);
  cudaEventRecord(e0);
  k_fma_chain<T><<<grid, block>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return WPIC_CUDA_ERROR;
  *gflops = 2.0 * 8.0 * (double)iters * grid.x * block.x / (ms * 1e6);
  return WPIC_OK;
}

}  // namespace

extern "C" int wpic_measure_fma_peak(int fp64, double* gflops) {
  if (!gflops) return WPIC_BAD_ARGUMENT;
  return fp64 ? run<double>(2000, gflops) : run<float>(20000, gflops);
}
