// The batched launches' item loop, shared by the two schemes' kernels
// (vnr.cu, euc.cu).
#ifndef MAHYCO_GB300_ITEMS_CUH
#define MAHYCO_GB300_ITEMS_CUH

#include "../internal.h"

namespace hydro {

// Batched launches: a persistent grid walks the tile table; every thread of
// a block works on the same tile (the block reductions of some phases rely
// on it).  The tile's run view is staged in shared memory by the whole
// block, so its fields are read where they are used instead of being held
// in registers for the whole tile.  scheme >= 0: the tiles of runs of the
// other scheme are skipped (a batch may hold both; the skip is uniform over
// the block).
template <class F>
__device__ __forceinline__ void batch_items(const BatchArgs& b, const F& f, int scheme = -1) {
  __shared__ RunView sv;
  constexpr int kWords = sizeof(RunView) / sizeof(unsigned long long);
  static_assert(sizeof(RunView) % sizeof(unsigned long long) == 0, "RunView size");
  const int n = *b.ntiles;
  const int tx = threadIdx.x & ((1 << b.tw_log2) - 1);
  const int ty = threadIdx.x >> b.tw_log2;
  const int th = kBatchThreads >> b.tw_log2;
  for (int t = blockIdx.x; t < n; t += gridDim.x) {
    const Tile T = b.tiles[t];
    const unsigned long long* src =
        reinterpret_cast<const unsigned long long*>(b.views + T.inst);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sv);
    for (int k = threadIdx.x; k < kWords; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    if (sv.ctrl->active && (scheme < 0 || sv.scheme == scheme))
      for (int r = 0; r < b.rows; ++r) f(sv, T.i0 + ty + r * th, T.j0 + tx);
    __syncthreads();
  }
}

}  // namespace hydro

#endif  // MAHYCO_GB300_ITEMS_CUH
