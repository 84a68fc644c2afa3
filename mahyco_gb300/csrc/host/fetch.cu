// Device -> caller copies of run fields (hydro_run_fetch and the output
// planes of the drop-in driver).
//
// A field is K device planes (K = 1 for a cell or node scalar, 2 for a
// velocity, 3 for the per-material "_env" fields, whose planes beyond the
// run's materials read as zeros) interleaved into the caller's buffer as
// dst[i * K + k].  The copy runs through a few pinned staging chunks: a pack
// kernel reads the planes from HBM and writes chunk j, already in the
// caller's layout, straight into mapped pinned host memory, while host
// threads copy chunk j - 1 from pinned memory into the caller's (pageable)
// buffer.  A pageable cudaMemcpy stages through the driver's bounce buffers
// on one thread, and the interleave of a multi-plane field was a host loop
// on top of it; here the interleave costs nothing and the host side of the
// copy runs on several cores, overlapped with the device side.
#include <thread>

#include "copy_pool.h"
#include "fetch.h"

namespace hydro {

namespace {

// out[e] = plane[(e0 + e) % K][(e0 + e) / K], a zero for a missing plane
template <int K>
__global__ void __launch_bounds__(256) k_fetch_pack(FetchPlanes g, long long e0, long long ne,
                                                    double* __restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
    const long long q = e0 + e;
    const long long i = q / K;
    const int k = (int)(q - i * K);
    const double* pl = (k == 0) ? g.p[0] : ((k == 1) ? g.p[1] : g.p[2]);
    out[e] = pl ? __ldg(pl + i) : 0.0;
  }
}

}  // namespace

struct FetchStage {
  static constexpr int kBufs = 3;
  static constexpr size_t kChunkBytes = 8u << 20;
  double* host[kBufs] = {nullptr, nullptr, nullptr};
  double* dev[kBufs] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev[kBufs] = {nullptr, nullptr, nullptr};
  int grid = 0;
  CopyPool* pool = nullptr;
  std::mutex mu;  // one fetch at a time per context
};

void destroy_fetch_stage(FetchStage* st) {
  if (!st) return;
  delete st->pool;
  for (int k = 0; k < FetchStage::kBufs; ++k) {
    if (st->ev[k]) cudaEventDestroy(st->ev[k]);
    if (st->host[k]) cudaFreeHost(st->host[k]);
  }
  delete st;
}

int create_fetch_stage(int num_sms, FetchStage** out) {
  auto* st = new FetchStage();
  for (int k = 0; k < FetchStage::kBufs; ++k) {
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&st->host[k]),
                                  FetchStage::kChunkBytes, cudaHostAllocMapped);
    if (e == cudaSuccess)
      e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&st->dev[k]), st->host[k], 0);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&st->ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      destroy_fetch_stage(st);
      return fail(-100, std::string("fetch staging: ") + cudaGetErrorString(e));
    }
  }
  st->grid = (num_sms > 0 ? num_sms : 152) * 8;
  const unsigned hw = std::thread::hardware_concurrency();
  const int workers = (int)std::min(7u, hw > 1 ? hw - 1 : 0u);
  st->pool = new CopyPool(workers);
  *out = st;
  return 0;
}

int fetch_planes(hydro_ctx* ctx, const FetchPlanes& g, long long count, double* dst,
                 long long* launches) {
  if (g.k < 1 || g.k > 3) return fail(-1, "fetch_planes: bad plane count");
  if (count <= 0) return 0;
  if (!ctx->fetch)
    if (int rc = create_fetch_stage(ctx->num_sms, &ctx->fetch)) return rc;
  FetchStage& st = *ctx->fetch;
  std::lock_guard<std::mutex> lock(st.mu);
  cudaStream_t s = ctx->stream;
  const long long total = count * g.k;
  const long long per = (long long)(FetchStage::kChunkBytes / sizeof(double));
  const long long nchunks = (total + per - 1) / per;
  long long issued = 0;
  auto issue = [&]() -> cudaError_t {
    const int b = (int)(issued % FetchStage::kBufs);
    const long long e0 = issued * per, ne = std::min(per, total - e0);
    const int grid = (int)std::min<long long>(st.grid, (ne + 255) / 256);
    switch (g.k) {
      case 1: k_fetch_pack<1><<<grid, 256, 0, s>>>(g, e0, ne, st.dev[b]); break;
      case 2: k_fetch_pack<2><<<grid, 256, 0, s>>>(g, e0, ne, st.dev[b]); break;
      default: k_fetch_pack<3><<<grid, 256, 0, s>>>(g, e0, ne, st.dev[b]); break;
    }
    if (launches) *launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(st.ev[b], s);
    ++issued;
    return e;
  };
  // every buffer filled ahead; a buffer is refilled once its chunk is out
  while (issued < std::min<long long>(nchunks, FetchStage::kBufs)) CUDA_TRY(issue());
  for (long long j = 0; j < nchunks; ++j) {
    const int b = (int)(j % FetchStage::kBufs);
    const long long e0 = j * per, ne = std::min(per, total - e0);
    CUDA_TRY(cudaEventSynchronize(st.ev[b]));
    st.pool->copy(dst + e0, st.host[b], (size_t)ne * sizeof(double));
    if (issued < nchunks) CUDA_TRY(issue());
  }
  return 0;
}

}  // namespace hydro
