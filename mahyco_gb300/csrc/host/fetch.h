// Device -> caller copies of run fields through pinned staging (fetch.cu).
#ifndef MAHYCO_GB300_FETCH_H
#define MAHYCO_GB300_FETCH_H

#include "runtime.h"

namespace hydro {

// K device planes (a null plane reads as zeros) of `count` values each.
struct FetchPlanes {
  const double* p[3];
  int k;
};

// dst[i * K + k] = plane k [i] for i < count, through the context's staging
// (created at the first call); *launches counts the pack kernels.
int fetch_planes(hydro_ctx* ctx, const FetchPlanes& g, long long count, double* dst,
                 long long* launches);

}  // namespace hydro

#endif
