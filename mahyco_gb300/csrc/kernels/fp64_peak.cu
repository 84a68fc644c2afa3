// Measured FP64 throughput of the device: a chain of independent DFMAs per
// thread, timed with CUDA events.  It is the denominator of the FP64
// roofline the benchmark reports next to the HBM one (the hydro kernels are
// FP64-instruction bound on GB300).
#include <cuda_runtime.h>

#include "../internal.h"

namespace hydro {
namespace {
__global__ void k_dfma_chain(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
  double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
  for (int k = 0; k < iters; ++k) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (r == 1234.5) out[0] = r;  // keeps the chain live
}
}  // namespace

int measure_fp64_peak(int device, double* tflops) {
  cudaSetDevice(device);
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, device);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return fail(-50, "fp64 peak: cudaMalloc");
  const int threads = 256, blocks = prop.multiProcessorCount * 8, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_chain<<<blocks, threads>>>(d, 64, 0.999999, 1e-9);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_dfma_chain<<<blocks, threads>>>(d, iters, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return fail(-51, std::string("fp64 peak: ") + cudaGetErrorString(err));
  const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return 0;
}

}  // namespace hydro
