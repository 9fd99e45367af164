// tbb/parallel_sort.h stand-in - TEST INFRASTRUCTURE for oracle/_ref (see
// oracle/ref_shim/Eigen/Core): an unstable parallel comparison sort, as
// tbb::parallel_sort is (libstdc++ parallel mode over OpenMP).
#pragma once

#include <parallel/algorithm>

namespace tbb {

template <typename It, typename Compare>
void parallel_sort(It begin, It end, const Compare &comp) {
  __gnu_parallel::sort(begin, end, comp);
}

}  // namespace tbb
