// Host-only check of the drop-in's resume cursor (include/stq_gpu.hpp):
// run_sweep_sharedqueue counts start boxes in tidstart and MAX_OVERLAP_CUTOFF,
// as the reference does (src/simulation.cu:563-564, 747), and maps them onto
// the positions of the prepared sweep order with start_position. For every
// box count N, position count length >= N and cutoff sequence (fixed, or
// halved as after overflows), the calls' position ranges must cover
// [0, length) in order, once, and the loop `while (tidstart < N)` must end.
// Prints "ok" or the first failing case.
#include <cstdio>
#include <cstdint>

#include "stq_gpu.hpp"

static bool check(int64_t N, int64_t length, int64_t cutoff, bool halving) {
  int64_t tidstart = 0, covered = 0, calls = 0;
  while (tidstart < N) {
    const int64_t t1 = tidstart + cutoff < N ? tidstart + cutoff : N;
    const int64_t p0 = stq::gpu::start_position(tidstart, N, length);
    const int64_t p1 = stq::gpu::start_position(t1, N, length);
    if (p0 != covered || p1 < p0) {
      std::printf("gap or overlap: N=%lld length=%lld cutoff=%lld tidstart=%lld p0=%lld p1=%lld covered=%lld\n",
                  (long long)N, (long long)length, (long long)cutoff, (long long)tidstart, (long long)p0,
                  (long long)p1, (long long)covered);
      return false;
    }
    covered = p1;
    tidstart += cutoff;
    if (halving && cutoff > 1 && (++calls % 3) == 0) cutoff /= 2;
    if (calls > 4 * N + 64) {
      std::printf("loop does not end: N=%lld\n", (long long)N);
      return false;
    }
  }
  if (covered != length) {
    std::printf("positions left: N=%lld length=%lld cutoff=%lld covered=%lld\n", (long long)N, (long long)length,
                (long long)cutoff, (long long)covered);
    return false;
  }
  return true;
}

int main() {
  const int64_t Ns[] = {1, 2, 3, 7, 64, 1000, 476806};
  for (int64_t N : Ns) {
    const int64_t lengths[] = {N, N + 2, 3 * N + 5, 17 * N + 1};
    for (int64_t length : lengths) {
      const int64_t cutoffs[] = {1, 2, 5, N / 3 + 1, N, 2 * N};
      for (int64_t cutoff : cutoffs)
        for (bool halving : {false, true})
          if (cutoff > 0 && !check(N, length, cutoff, halving)) return 1;
    }
  }
  // a single call with the default cutoff N sweeps everything
  if (stq::gpu::start_position(0, 5, 9) != 0 || stq::gpu::start_position(5, 5, 9) != 9) {
    std::printf("single call does not cover the scene\n");
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
