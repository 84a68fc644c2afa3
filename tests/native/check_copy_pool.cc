// The field fetch's host copy threads (host/copy_pool.h) on the CPU: many
// back-to-back copies of random sizes and alignments, below and above the
// size that splits a copy into pieces, with 0 to 7 worker threads.  Every
// destination byte in range equals the source, and the bytes around the
// range are untouched.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "host/copy_pool.h"

int main() {
  std::mt19937_64 rng(20261204);
  constexpr size_t kSize = 9u << 20;
  std::vector<unsigned char> src(kSize + 128), dst(kSize + 128);
  for (auto& b : src) b = (unsigned char)rng();
  long jobs = 0, bad = 0;
  for (int workers : {0, 1, 3, 7}) {
    hydro::CopyPool pool(workers);
    for (int it = 0; it < 240; ++it) {
      const size_t so = rng() % 64, d0 = 1 + rng() % 63;
      size_t n = (it % 4 == 0) ? rng() % 5000 : rng() % kSize;
      // the destination range and one guard byte either side hold the
      // complement of what the copy writes
      for (size_t k = 0; k < n; ++k) dst[d0 + k] = (unsigned char)~src[so + k];
      dst[d0 - 1] = 0x5a;
      dst[d0 + n] = 0xa5;
      pool.copy(dst.data() + d0, src.data() + so, n);
      ++jobs;
      if (std::memcmp(dst.data() + d0, src.data() + so, n) != 0) ++bad;
      if (dst[d0 - 1] != 0x5a || dst[d0 + n] != 0xa5) ++bad;
    }
  }
  std::printf("copy_pool: %ld jobs, %ld mismatches\n", jobs, bad);
  return bad != 0;
}
