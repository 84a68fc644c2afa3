// Device checks of the integer-pipe binary64 operations (softfp.cuh): each
// element computed by the fast path and by the FP64 instruction on the GPU,
// and the throughput of both forms (dependent chains per thread, CUDA
// events).  Diagnostics, no counterpart in the reference.
#include <cuda_runtime.h>

#include "../host/runtime.h"
#include "scheme_math.cuh"

namespace hydro {
namespace {

__global__ void k_softfp_check(int op, const double* a, const double* b, double* soft,
                               double* hw, unsigned char* fast, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = a[i], y = b[i];
  unsigned long long r = 0;
  bool f = false;
  double h = 0.;
  switch (op) {
    case 0: f = sfp::mul_fast(ubits(x), ubits(y), r); h = x * y; break;
    case 1: f = sfp::add_fast(ubits(x), ubits(y), r); h = x + y; break;
    case 2: f = sfp::div_fast(ubits(x), ubits(y), r); h = x / y; break;
    case 3: f = sfp::sqrt_fast(ubits(x), r); h = sqrt(x); break;
    case 4: f = sfp::add_fast(ubits(x), ubits(y) ^ 0x8000000000000000ull, r); h = x - y; break;
    default: break;
  }
  soft[i] = from_bits(r);
  hw[i] = h;
  fast[i] = f ? 1 : 0;
}

// 8 independent chains per thread of one operation, native (soft = 0) or
// through the *_ip wrappers (soft = 1); the operands keep every chain
// normal.
template <int OP, int SOFT>
__global__ void k_softfp_rate(double* out, int iters, double c) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 1.0 + (threadIdx.x * 8 + k) * 1e-7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (OP == 0) x[k] = SOFT ? mul_ip(x[k], c) : x[k] * c;
      if (OP == 1) x[k] = SOFT ? add_ip(x[k], c) : x[k] + c;
      if (OP == 2) x[k] = SOFT ? div_ip(x[k], c) : x[k] / c;
      if (OP == 3) x[k] = SOFT ? sqrt_ip(x[k]) : sqrt(x[k]);
    }
  }
  double r = 0.;
#pragma unroll
  for (int k = 0; k < 8; ++k) r += x[k];
  if (r == 1234.5) out[0] = r;  // keeps the chains live
}

template <int OP, int SOFT>
float time_rate(double* d, int blocks, int threads, int iters, double c) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_softfp_rate<OP, SOFT><<<blocks, threads>>>(d, 16, c);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0);
    k_softfp_rate<OP, SOFT><<<blocks, threads>>>(d, iters, c);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace
}  // namespace hydro

using namespace hydro;

extern "C" {

int hydro_softfp_check(int op, const double* a, const double* b, double* soft, double* hw,
                       unsigned char* fast, long long n, void* stream) {
  if (op < 0 || op > 4 || n < 0 || (n > 0 && (!a || !b || !soft || !hw || !fast)))
    return fail(-1, "hydro_softfp_check: bad argument");
  if (n == 0) return 0;
  const int threads = 256;
  const long long blocks = (n + threads - 1) / threads;
  k_softfp_check<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(op, a, b, soft, hw,
                                                                         fast, n);
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// Operations per second of mul, add, div, sqrt: rates[2 k] native,
// rates[2 k + 1] through the integer-pipe wrappers.
int hydro_softfp_rates(int device, double* rates) {
  if (!rates) return fail(-1, "hydro_softfp_rates: null argument");
  CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop{};
  CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  double* d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(double)));
  const int threads = 256, blocks = prop.multiProcessorCount * 8;
  const int it_native = 256, it_soft = 256;
  float ms[8];
  ms[0] = time_rate<0, 0>(d, blocks, threads, it_native, 0.9999999);
  ms[1] = time_rate<0, 1>(d, blocks, threads, it_soft, 0.9999999);
  ms[2] = time_rate<1, 0>(d, blocks, threads, it_native, 1e-9);
  ms[3] = time_rate<1, 1>(d, blocks, threads, it_soft, 1e-9);
  ms[4] = time_rate<2, 0>(d, blocks, threads, it_native, 1.0000001);
  ms[5] = time_rate<2, 1>(d, blocks, threads, it_soft, 1.0000001);
  ms[6] = time_rate<3, 0>(d, blocks, threads, it_native, 0.);
  ms[7] = time_rate<3, 1>(d, blocks, threads, it_soft, 0.);
  const cudaError_t err = cudaGetLastError();
  cudaFree(d);
  if (err != cudaSuccess) return fail(-51, std::string("softfp rates: ") + cudaGetErrorString(err));
  const double ops = 8.0 * (double)threads * blocks;
  for (int k = 0; k < 8; ++k)
    rates[k] = ops * (k & 1 ? it_soft : it_native) / (ms[k] * 1e-3);
  return 0;
}

}  // extern "C"
