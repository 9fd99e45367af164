// stq_oracle.cpp - CPU oracle for the STQ broad phase. TEST INFRASTRUCTURE.
//
// A plain C++17 + OpenMP restatement of the reference's CPU path
// (Ahdhn/broadphase-gpu src/cpu/aabb.cpp and src/cpu/sweep.cpp), used only
// by the tests, the smoke check and the bench's CPU baseline and reference
// legs, to check and time against. Nothing in the product links or calls it.
//
// Parity status: pinned to the reference's own code. The reference ships no
// tests, golden vectors or fixtures, but its src/cpu/aabb.cpp and
// src/cpu/sweep.cpp compile unchanged against the stand-in headers of
// oracle/ref_shim/ (the Eigen, oneTBB and spdlog subsets they use) into
// oracle/_ref/libstq_ref.so. The tests check this restatement against that
// library where the reference's tree is present, and everywhere against the
// golden vectors it wrote (tests/golden/ref_vectors.npz). The hand-derived
// known-answer cases of tests/golden/kat.json pin the corner cases on top.
//
// Build: without -ffast-math and without flush-to-zero, so that the outward
// rounding below (which subtracts the smallest denormal) behaves as IEEE 754
// specifies on the CPU the reference runs on.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>
#include <utility>
#include <vector>

#include <omp.h>
#include <parallel/algorithm>

namespace {

// Same 44-byte record as stq::gpu::Aabb (src/aabb.cuh:15-43). The CPU
// reference's Aabb (src/cpu/aabb.hpp:21-33) holds the same id, min, max and
// vertexIds; ref_id is filled as the GPU builder does (src/aabb.cu:224).
struct Box {
  int32_t id;
  float min[3];
  float max[3];
  int32_t v[3];
  int32_t ref_id;
};
static_assert(sizeof(Box) == 44, "Aabb layout");

// src/cpu/aabb.cpp:16-21
float nextafter_up(float x) {
  return std::nextafter(x, x + std::numeric_limits<float>::max());
}
float nextafter_down(float x) {
  return std::nextafter(x, x - std::numeric_limits<float>::max());
}

// src/cpu/sweep.cpp:17-30
bool is_face(const int32_t *v) { return v[2] >= 0; }
bool is_edge(const int32_t *v) { return v[2] < 0 && v[1] >= 0; }
bool is_vertex(const int32_t *v) { return v[2] < 0 && v[1] < 0; }
bool is_valid_pair(const int32_t *a, const int32_t *b) {
  return (is_vertex(a) && is_face(b)) || (is_face(a) && is_vertex(b)) ||
         (is_edge(a) && is_edge(b));
}

// src/cpu/sweep.cpp:32-37 (the sweep axis x is not tested, only y and z)
bool does_collide(const Box &a, const Box &b) {
  return a.max[1] >= b.min[1] && a.min[1] <= b.max[1] &&
         a.max[2] >= b.min[2] && a.min[2] <= b.max[2];
}

// src/cpu/sweep.cpp:39-43
bool covertex(const int32_t *a, const int32_t *b) {
  return a[0] == b[0] || a[0] == b[1] || a[0] == b[2] || a[1] == b[0] ||
         a[1] == b[1] || a[1] == b[2] || a[2] == b[0] || a[2] == b[1] ||
         a[2] == b[2];
}

int default_threads() {
  // app/main.cpp:139-141: min(hardware concurrency, 64)
  int hw = int(std::thread::hardware_concurrency());
  return std::max(1, std::min(hw, 64));
}

int pick_threads(int threads) { return threads > 0 ? threads : default_threads(); }

using Pairs = std::vector<std::pair<int32_t, int32_t>>;

// src/cpu/sweep.cpp:94-121: parallel over start boxes i < n; for each, scan
// j = i+1.. and break at the first b with a.max[0] < b.min[0].
void sweep(const Box *boxes, int64_t N, int64_t n_begin, int64_t n_end,
           int64_t stride, int threads, Pairs &out) {
  std::vector<Pairs> local(threads);
#pragma omp parallel num_threads(threads)
  {
    Pairs &mine = local[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = n_begin; i < n_end; i += stride) {
      const Box &a = boxes[i];
      for (int64_t j = i + 1; j < N; ++j) {
        const Box &b = boxes[j];
        if (a.max[0] < b.min[0]) break;
        if (does_collide(a, b) && is_valid_pair(a.v, b.v) && !covertex(a.v, b.v))
          mine.emplace_back(a.id, b.id);
      }
    }
  }
  // serial merge, src/cpu/sweep.cpp:79-92
  size_t total = 0;
  for (auto &l : local) total += l.size();
  out.clear();
  out.reserve(total);
  for (auto &l : local) out.insert(out.end(), l.begin(), l.end());
}

// src/cpu/sweep.cpp:72-74: sort by min[0] (tbb::parallel_sort, unstable)
void sort_along_xaxis(Box *boxes, int64_t n, int threads) {
  omp_set_num_threads(threads);
  __gnu_parallel::sort(boxes, boxes + n, [](const Box &a, const Box &b) {
    return a.min[0] < b.min[0];
  });
}

int32_t *to_malloc(const Pairs &p) {
  int32_t *out = static_cast<int32_t *>(std::malloc(sizeof(int32_t) * 2 * (p.size() + 1)));
  for (size_t k = 0; k < p.size(); ++k) {
    out[2 * k] = p[k].first;
    out[2 * k + 1] = p[k].second;
  }
  return out;
}

void canonicalize(Pairs &p, int threads) {
  for (auto &q : p)
    if (q.first > q.second) std::swap(q.first, q.second);
  omp_set_num_threads(threads);
  __gnu_parallel::sort(p.begin(), p.end());
  p.erase(std::unique(p.begin(), p.end()), p.end());
}

}  // namespace

extern "C" {

// stq::cpu::constructBoxes (src/cpu/aabb.cpp:7-13): vertices, then edges,
// then faces; id = offset + i, ref_id = i.
void oracle_construct_boxes(const double *V0, const double *V1, int64_t nV,
                            const int32_t *E, int64_t nE, const int32_t *F,
                            int64_t nF, double inflation_radius, void *out) {
  Box *boxes = static_cast<Box *>(out);
  // the float parameter of nextafter_up takes the double radius by value
  const float r_up = nextafter_up(static_cast<float>(inflation_radius));
  // addVertices, src/cpu/aabb.cpp:23-51 (float branch, lines 42-47)
  for (int64_t i = 0; i < nV; ++i) {
    Box &b = boxes[i];
    b.id = int32_t(i);
    b.ref_id = int32_t(i);
    b.v[0] = int32_t(i), b.v[1] = int32_t(-i - 1), b.v[2] = int32_t(-i - 1);
    for (int k = 0; k < 3; ++k) {
      const float t0 = static_cast<float>(V0[3 * i + k]);  // cast<Scalar>()
      const float t1 = static_cast<float>(V1[3 * i + k]);
      const float lo = t1 < t0 ? t1 : t0;  // cwise min
      const float hi = t0 < t1 ? t1 : t0;  // cwise max
      b.min[k] = nextafter_down(lo) - r_up;
      b.max[k] = nextafter_up(hi) + r_up;
    }
  }
  // addEdges, src/cpu/aabb.cpp:53-73: union of the two vertex boxes
  for (int64_t i = 0; i < nE; ++i) {
    Box &b = boxes[nV + i];
    const Box &p = boxes[E[2 * i]], &q = boxes[E[2 * i + 1]];
    b.id = int32_t(nV + i);
    b.ref_id = int32_t(i);
    b.v[0] = E[2 * i], b.v[1] = E[2 * i + 1], b.v[2] = -E[2 * i] - 1;
    for (int k = 0; k < 3; ++k) {
      b.min[k] = q.min[k] < p.min[k] ? q.min[k] : p.min[k];
      b.max[k] = p.max[k] < q.max[k] ? q.max[k] : p.max[k];
    }
  }
  // addFaces, src/cpu/aabb.cpp:75-95: union of the three vertex boxes
  for (int64_t i = 0; i < nF; ++i) {
    Box &b = boxes[nV + nE + i];
    const Box &p = boxes[F[3 * i]], &q = boxes[F[3 * i + 1]], &s = boxes[F[3 * i + 2]];
    b.id = int32_t(nV + nE + i);
    b.ref_id = int32_t(i);
    b.v[0] = F[3 * i], b.v[1] = F[3 * i + 1], b.v[2] = F[3 * i + 2];
    for (int k = 0; k < 3; ++k) {
      float lo = q.min[k] < p.min[k] ? q.min[k] : p.min[k];
      lo = s.min[k] < lo ? s.min[k] : lo;
      float hi = p.max[k] < q.max[k] ? q.max[k] : p.max[k];
      hi = hi < s.max[k] ? s.max[k] : hi;
      b.min[k] = lo;
      b.max[k] = hi;
    }
  }
}

void oracle_sort_along_xaxis(void *boxes, int64_t n, int threads) {
  sort_along_xaxis(static_cast<Box *>(boxes), n, pick_threads(threads));
}

// stq::cpu::sweep over start boxes [0, n_start) of boxes sorted along x.
// Returns the pair count; *pairs_out = malloc'd (a.id, b.id) pairs.
int64_t oracle_sweep(const void *sorted, int64_t N, int64_t n_start,
                     int threads, int32_t **pairs_out) {
  Pairs p;
  sweep(static_cast<const Box *>(sorted), N, 0, std::min(n_start, N), 1,
        pick_threads(threads), p);
  *pairs_out = to_malloc(p);
  return int64_t(p.size());
}

// Full oracle: copy, sort along x, sweep every start box, then the
// canonical form used for comparison: (min id, max id), sorted, unique.
int64_t oracle_broadphase(const void *boxes, int64_t n, int threads,
                          int32_t **pairs_out) {
  threads = pick_threads(threads);
  std::vector<Box> b(static_cast<const Box *>(boxes), static_cast<const Box *>(boxes) + n);
  sort_along_xaxis(b.data(), n, threads);
  Pairs p;
  sweep(b.data(), n, 0, n, 1, threads, p);
  canonicalize(p, threads);
  *pairs_out = to_malloc(p);
  return int64_t(p.size());
}

// Canonical form of an arbitrary pair list, in place; returns the new count.
int64_t oracle_canonicalize(int32_t *pairs, int64_t count, int threads) {
  Pairs p(count);
  for (int64_t k = 0; k < count; ++k) p[k] = {pairs[2 * k], pairs[2 * k + 1]};
  canonicalize(p, pick_threads(threads));
  for (size_t k = 0; k < p.size(); ++k) {
    pairs[2 * k] = p[k].first;
    pairs[2 * k + 1] = p[k].second;
  }
  return int64_t(p.size());
}

// Set comparison of two canonical (sorted, unique) pair lists, in the manner
// of compare_mathematica (src/groundtruth.cu:24-67) but counting both sides.
void oracle_compare(const int32_t *a, int64_t na, const int32_t *b, int64_t nb,
                    int64_t *only_a, int64_t *only_b) {
  int64_t i = 0, j = 0, oa = 0, ob = 0;
  auto key = [](const int32_t *p, int64_t k) {
    return (uint64_t(uint32_t(p[2 * k])) << 32) | uint32_t(p[2 * k + 1]);
  };
  while (i < na && j < nb) {
    const uint64_t x = key(a, i), y = key(b, j);
    if (x == y) ++i, ++j;
    else if (x < y) ++oa, ++i;
    else ++ob, ++j;
  }
  *only_a = oa + (na - i);
  *only_b = ob + (nb - j);
}

// CPU baseline timing: sorts all n boxes along x, then sweeps every
// `stride`-th start box. Returns seconds (sort, sweep) and the pair count
// of the sample.
int64_t oracle_time_sample(const void *boxes, int64_t n, int64_t stride,
                           int threads, double *sort_s, double *sweep_s) {
  threads = pick_threads(threads);
  std::vector<Box> b(static_cast<const Box *>(boxes), static_cast<const Box *>(boxes) + n);
  auto t0 = std::chrono::steady_clock::now();
  sort_along_xaxis(b.data(), n, threads);
  auto t1 = std::chrono::steady_clock::now();
  Pairs p;
  sweep(b.data(), n, 0, n, stride < 1 ? 1 : stride, threads, p);
  auto t2 = std::chrono::steady_clock::now();
  *sort_s = std::chrono::duration<double>(t1 - t0).count();
  *sweep_s = std::chrono::duration<double>(t2 - t1).count();
  return int64_t(p.size());
}

int oracle_default_threads(void) { return default_threads(); }

void oracle_free(void *p) { std::free(p); }

}  // extern "C"
