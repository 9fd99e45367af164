// tbb/parallel_for.h stand-in - TEST INFRASTRUCTURE for oracle/_ref (see
// oracle/ref_shim/Eigen/Core). parallel_for(range, body) calls body on
// disjoint sub-ranges that cover the range, concurrently; here the pieces are
// chunks of kChunk values (at least the grain size) taken by OpenMP threads in
// dynamic order. The bodies the reference passes treat each value on its own,
// so the result does not depend on how the range is cut.
#pragma once

#include <omp.h>

#include <algorithm>

#include "blocked_range.h"

namespace tbb {

template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &range, const Body &body) {
  constexpr long long kChunk = 64;
  const long long n = static_cast<long long>(range.end() - range.begin());
  if (n <= 0) return;
  const long long chunk = std::max<long long>(kChunk, static_cast<long long>(range.grainsize()));
  const long long pieces = (n + chunk - 1) / chunk;
#pragma omp parallel for schedule(dynamic, 1)
  for (long long p = 0; p < pieces; ++p) {
    const Value b = static_cast<Value>(range.begin() + p * chunk);
    const Value e = static_cast<Value>(range.begin() + std::min(n, (p + 1) * chunk));
    body(blocked_range<Value>(b, e, range.grainsize()));
  }
}

}  // namespace tbb
