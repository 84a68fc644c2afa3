// CFL time step of a VNR state that lives in the caller's device memory,
// computed without allocating anything.
//
// Who needs it: code that owns every byte of device memory through its own
// pool (a serving process, a host solver that embeds one hydro step in its
// own time loop) or that runs while another library holds the device
// allocator, and therefore may not call cudaMalloc / cudaFree.  Those
// callers pass their own buffers for the inputs and the output; the only
// other memory the computation needs -- one partial minimum per thread
// block -- is the file-scope device array below, reserved when the library
// is loaded.
//
// The value is the one a run computes at the start of its next cycle
// (Vnr::computeDeltaT, vnr_remap/VnrRemap.cc:14-50, with the remap on:
// cfl 0.05, dt <= 1.05 * dt_n): min over cells of
// 0.05*sqrt(sum of the cell's initial sub-volumes) / (sum_p 0.25*|u_p| + c).
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../internal.h"
#include "scheme_math.cuh"

namespace hydro {

// Largest state accepted: kDtMaxBlocks blocks of kDtBlock cells.
constexpr int kDtBlock = 256;
constexpr int kDtMaxBlocks = 4096;  // 32 KiB of scratch: 1,048,576 cells

// One ordered-int partial minimum per block.  Every call overwrites the
// slots of the blocks it launches before the final pass reads them, so
// nothing has to be cleared between calls; two calls that overlap on the GPU
// (different streams, or the same scratch in flight) race on these slots.
static __device__ __align__(256) unsigned long long g_dt_scratch[kDtMaxBlocks];

namespace {

// Initial sub-volume sum of one cell (Vnr::initCellPos + initSubVol,
// vnr_remap/Init.cc:400-429, 495-511) from the Cartesian node coordinates
// dx*j, dy*i, with the reference's operation order.
__device__ double initial_volume_sum(int i, int j, double dx, double dy) {
  double X[4][2] = {{dx * (double)j, dy * (double)i},
                    {dx * (double)(j + 1), dy * (double)i},
                    {dx * (double)(j + 1), dy * (double)(i + 1)},
                    {dx * (double)j, dy * (double)(i + 1)}};
  double xc0 = 0.0, xc1 = 0.0;
  for (int k = 0; k < 4; ++k) {
    xc0 = xc0 + X[k][0];
    xc1 = xc1 + X[k][1];
  }
  xc0 = 0.25 * xc0;
  xc1 = 0.25 * xc1;
  double r = 0.0;
  for (int k = 0; k < 4; ++k) {
    const int km = (k + 3) & 3, kp = (k + 1) & 3;
    const double x2a = 0.5 * (X[km][0] + X[k][0]), x2b = 0.5 * (X[km][1] + X[k][1]);
    const double x4a = 0.5 * (X[kp][0] + X[k][0]), x4b = 0.5 * (X[kp][1] + X[k][1]);
    const double c12 = xc0 * x2b - xc1 * x2a;
    const double c23 = x2a * X[k][1] - x2b * X[k][0];
    const double c34 = X[k][0] * x4b - X[k][1] * x4a;
    const double c41 = x4a * xc1 - x4b * xc0;
    r = r + 0.5 * (c12 + c23 + c34 + c41);
  }
  return r;
}

__global__ void __launch_bounds__(kDtBlock)
k_dt_partial(int nx, int ny, double dx, double dy, const double* u,
             const double* v, const double* c, unsigned long long* scratch) {
  const long long cell = (long long)blockIdx.x * kDtBlock + threadIdx.x;
  unsigned long long best = ~0ull;
  if (cell < (long long)nx * ny) {
    const int i = (int)(cell / nx), j = (int)(cell - (long long)i * nx);
    const long long n0 = (long long)i * (nx + 1) + j;
    const long long nd[4] = {n0, n0 + 1, n0 + nx + 2, n0 + nx + 1};
    double uc = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double a = u[nd[k]], b = v[nd[k]];
      uc += sqrt(a * a + b * b) * 0.25;
    }
    const double cflsq = 0.05 * sqrt(initial_volume_sum(i, j, dx, dy));
    const double d = cflsq / (uc + c[cell]);
    if (d == d) best = ord_bits(d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, best, o);
    best = t < best ? t : best;
  }
  __shared__ unsigned long long warp_min[kDtBlock / 32];
  if ((threadIdx.x & 31) == 0) warp_min[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = warp_min[0];
    for (int w = 1; w < kDtBlock / 32; ++w) m = warp_min[w] < m ? warp_min[w] : m;
    scratch[blockIdx.x] = m;
  }
}

__global__ void __launch_bounds__(kDtBlock)
k_dt_final(int nblocks, double dt_n, const unsigned long long* scratch,
           double* dt_out) {
  unsigned long long best = ~0ull;
  for (int b = threadIdx.x; b < nblocks; b += kDtBlock)
    best = scratch[b] < best ? scratch[b] : best;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, best, o);
    best = t < best ? t : best;
  }
  __shared__ unsigned long long warp_min[kDtBlock / 32];
  if ((threadIdx.x & 31) == 0) warp_min[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = warp_min[0];
    for (int w = 1; w < kDtBlock / 32; ++w) m = warp_min[w] < m ? warp_min[w] : m;
    // no valid candidate: the reference's reduction starts at DBL_MAX
    const double red = (m == ~0ull) ? 1.7976931348623157e308 : from_ord(m);
    *dt_out = smin(red, 1.05 * dt_n);
  }
}

// Device address of g_dt_scratch, looked up once per device (with that
// device current) on the first call made on it, in the device's primary
// context (the CUDA runtime's); it stays valid until that context is reset,
// after which the function must not be called (documented in the header).
constexpr int kMaxDevices = 64;
unsigned long long* g_scratch_ptr[kMaxDevices];
std::mutex g_scratch_mu;

}  // namespace

}  // namespace hydro

using namespace hydro;

extern "C" int hydro_vnr_dt_noalloc(int nx, int ny, double dx, double dy,
                                    const double* d_u, const double* d_v,
                                    const double* d_c, double dt_n,
                                    double* d_dt_out, void* stream) {
  if (!d_u || !d_v || !d_c || !d_dt_out)
    return fail(-1, "hydro_vnr_dt_noalloc: null device pointer");
  if (nx < 2 || ny < 2) return fail(-2, "hydro_vnr_dt_noalloc: nx and ny must be >= 2");
  const long long ncells = (long long)nx * ny;
  const long long nblocks = (ncells + kDtBlock - 1) / kDtBlock;
  if (nblocks > kDtMaxBlocks)
    return fail(-3, "hydro_vnr_dt_noalloc: " + std::to_string(ncells) +
                        " cells exceed the fixed scratch limit of " +
                        std::to_string((long long)kDtMaxBlocks * kDtBlock) +
                        " cells");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(-4, "hydro_vnr_dt_noalloc: no usable current device");
  unsigned long long* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_dt_scratch);
      if (e != cudaSuccess)
        return fail(-5, std::string("hydro_vnr_dt_noalloc: cudaGetSymbolAddress: ") +
                            cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_dt_partial<<<(unsigned)nblocks, kDtBlock, 0, s>>>(nx, ny, dx, dy, d_u, d_v,
                                                      d_c, scratch);
  k_dt_final<<<1, kDtBlock, 0, s>>>((int)nblocks, dt_n, scratch, d_dt_out);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(-6, std::string("hydro_vnr_dt_noalloc: launch: ") + cudaGetErrorString(e));
  return 0;
}
