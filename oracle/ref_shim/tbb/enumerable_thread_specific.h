// tbb/enumerable_thread_specific.h stand-in - TEST INFRASTRUCTURE for
// oracle/_ref (see oracle/ref_shim/Eigen/Core): one T per thread of the
// parallel loops; local() is the calling thread's, and iteration visits every
// thread's T (threads that never called local() contribute an empty T).
#pragma once

#include <omp.h>

#include <vector>

namespace tbb {

template <typename T>
class enumerable_thread_specific {
 public:
  enumerable_thread_specific() : slots_(std::size_t(omp_get_max_threads())) {}
  T &local() { return slots_[std::size_t(omp_get_thread_num())]; }
  std::size_t size() const { return slots_.size(); }
  typename std::vector<T>::iterator begin() { return slots_.begin(); }
  typename std::vector<T>::iterator end() { return slots_.end(); }
  typename std::vector<T>::const_iterator begin() const { return slots_.begin(); }
  typename std::vector<T>::const_iterator end() const { return slots_.end(); }

 private:
  std::vector<T> slots_;
};

}  // namespace tbb
