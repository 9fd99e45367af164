// tbb/blocked_range.h stand-in - TEST INFRASTRUCTURE for oracle/_ref (see
// oracle/ref_shim/Eigen/Core): the half-open range [begin, end) that
// tbb::parallel_for hands to its body in pieces.
#pragma once

#include <cstddef>

namespace tbb {

template <typename Value>
class blocked_range {
 public:
  blocked_range(Value begin, Value end, std::size_t grainsize = 1)
      : b_(begin), e_(end), g_(grainsize ? grainsize : 1) {}
  Value begin() const { return b_; }
  Value end() const { return e_; }
  std::size_t size() const { return std::size_t(e_ - b_); }
  std::size_t grainsize() const { return g_; }
  bool empty() const { return !(b_ < e_); }

 private:
  Value b_, e_;
  std::size_t g_;
};

}  // namespace tbb
