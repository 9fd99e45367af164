// ref_bridge.cpp - C entry points over the reference's own CPU machine builder and
// sweep. TEST INFRASTRUCTURE.
//
// The reference's src/cpu/aabb.cpp and src/cpu/sweep.cpp are compiled
// unchanged from the reference's source tree (oracle/Makefile, target `ref`),
// against the stand-in headers of oracle/ref_shim/ for the parts of Eigen,
// oneTBB and spdlog they use, into oracle/_ref/libstq_ref.so. The tests use
// this library to pin the oracle restatement (stq_oracle.cpp) to the
// reference's own code, and tests/golden/make_ref_golden.py uses it to write
// golden vectors that travel without the reference. Nothing in the product
// links or calls it.
#include <stq/cpu/aabb.hpp>
#include <stq/cpu/sweep.hpp>

#include <omp.h>

#include <cstdint>
#include <cstdlib>
#include <utility>
#include <vector>

namespace {

// The 44-byte record of the GPU library's boxes (stq::gpu::Aabb,
// src/aabb.cuh:15-43): id, min, max, vertexIds, ref_id.
struct Record {
  int32_t id;
  float min[3];
  float max[3];
  int32_t v[3];
  int32_t ref_id;
};
static_assert(sizeof(Record) == 44, "record layout");

}  // namespace

extern "C" {

// stq::cpu::constructBoxes (src/cpu/aabb.cpp:7-14) on row-major inputs; the
// records' ref_id is the box's index within its kind (vertex, edge, face),
// which the CPU Aabb does not hold.
void ref_construct_boxes(const double *V0, const double *V1, int64_t nV, const int32_t *E,
                         int64_t nE, const int32_t *F, int64_t nF, double inflation_radius,
                         int threads, void *out) {
  if (threads > 0) omp_set_num_threads(threads);
  Eigen::MatrixXd v0(nV, 3), v1(nV, 3);
  Eigen::MatrixXi e(nE, 2), f(nF, 3);
  for (int64_t i = 0; i < nV; ++i)
    for (int k = 0; k < 3; ++k) v0(i, k) = V0[3 * i + k], v1(i, k) = V1[3 * i + k];
  for (int64_t i = 0; i < nE; ++i)
    for (int k = 0; k < 2; ++k) e(i, k) = E[2 * i + k];
  for (int64_t i = 0; i < nF; ++i)
    for (int k = 0; k < 3; ++k) f(i, k) = F[3 * i + k];
  std::vector<stq::cpu::Aabb> boxes;
  stq::cpu::constructBoxes(v0, v1, e, f, boxes, inflation_radius);
  Record *r = static_cast<Record *>(out);
  for (size_t i = 0; i < boxes.size(); ++i) {
    const stq::cpu::Aabb &b = boxes[i];
    r[i].id = b.id;
    for (int k = 0; k < 3; ++k) {
      r[i].min[k] = b.min[k];
      r[i].max[k] = b.max[k];
      r[i].v[k] = b.vertexIds[size_t(k)];
    }
    const int64_t k = int64_t(i);
    r[i].ref_id = int32_t(k < nV ? k : (k < nV + nE ? k - nV : k - nV - nE));
  }
}

// The CPU app's sweep (app/main.cpp:147-151): sweep_cpu_single_batch over
// all boxes, called until it returns no pairs. *pairs receives the raw
// (a.id, b.id) pairs (malloc; free with ref_free); returns their count.
int64_t ref_broadphase(const void *records, int64_t n, int threads, int32_t **pairs) {
  if (threads > 0) omp_set_num_threads(threads);
  const Record *r = static_cast<const Record *>(records);
  std::vector<stq::cpu::Aabb> boxes(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    stq::cpu::ArrayMax3 lo, hi;
    lo.resize(3);
    hi.resize(3);
    for (int k = 0; k < 3; ++k) lo[k] = r[i].min[k], hi[k] = r[i].max[k];
    boxes[size_t(i)] = stq::cpu::Aabb(r[i].id, {{r[i].v[0], r[i].v[1], r[i].v[2]}}, lo, hi);
  }
  std::vector<std::pair<int, int>> overlaps, all;
  int N = int(n), nn = int(n);
  stq::cpu::sweep_cpu_single_batch(boxes, nn, N, overlaps);
  while (overlaps.size()) {
    all.insert(all.end(), overlaps.begin(), overlaps.end());
    stq::cpu::sweep_cpu_single_batch(boxes, nn, N, overlaps);
  }
  int32_t *out = static_cast<int32_t *>(std::malloc(sizeof(int32_t) * 2 * (all.size() + 1)));
  for (size_t k = 0; k < all.size(); ++k) {
    out[2 * k] = all[k].first;
    out[2 * k + 1] = all[k].second;
  }
  *pairs = out;
  return int64_t(all.size());
}

void ref_free(void *p) { std::free(p); }

}  // extern "C"
