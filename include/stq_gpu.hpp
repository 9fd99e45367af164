// stq_gpu.hpp - C++ drop-in for the reference's stq::gpu host API, written
// on top of the C ABI (stq_abi.h) and the CUDA runtime. Header only.
//
// Recreated signatures (Ahdhn/broadphase-gpu):
//   stq::gpu::Aabb                  src/aabb.cuh:15-43
//   stq::gpu::MemHandler            src/memory.cuh:69-189 (broad-phase part)
//   stq::gpu::constructBoxes        src/io.cuh:9-13
//   stq::gpu::run_sweep_sharedqueue src/simulation.cuh:22-27
//   stq::gpu::run_sweep_multigpu    src/simulation.cuh:18-20 (one device)
//
// Matrix arguments are templates: any type with rows(), cols() and
// operator()(i, j) (Eigen::MatrixXd / MatrixXi among them) is accepted.
//
// Behaviour kept from the reference: boxes are ids in V, E, F order; the pair
// buffer d_overlaps and the counter d_count are allocated here and owned by the
// caller afterwards; MemHandler sizes the pair buffer from free device memory
// leaving room for the narrow phase, and on overflow grows it or halves
// MAX_OVERLAP_CUTOFF and sweeps again; tidstart is the resume cursor.
// Differences: pairs are (smaller id, larger id); errors throw
// stq::gpu::Error instead of calling exit(); devcount is ignored (one GPU).
// tidstart and MAX_OVERLAP_CUTOFF count start boxes as in the reference; the
// library's sweep order holds a box once per cell it touches, and a range of
// start boxes maps to a proportional range of those positions
// (start_position below).
//
// Compile-time option: STQ_GPU_MAX_OVERLAP_SIZE caps the pair buffer at that
// many pairs, as a device with less free memory would (to exercise the
// overflow-and-resume path on small scenes).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "stq_abi.h"

namespace stq::gpu {

typedef float Scalar;

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what)
      : std::runtime_error("stq status " + std::to_string(status) + ": " + what), status(status) {}
  int status;
};

// Field for field the reference's Aabb (44 bytes, Scalar = float).
class Aabb {
 public:
  int id;
  float3 min;
  float3 max;
  int3 vertexIds;
  int ref_id;
  Aabb() = default;
  Aabb(int assignid, int reference_id, const int *vids, const Scalar *tempmin,
       const Scalar *tempmax)
      : id(assignid), min(make_float3(tempmin[0], tempmin[1], tempmin[2])),
        max(make_float3(tempmax[0], tempmax[1], tempmax[2])),
        vertexIds(make_int3(vids[0], vids[1], vids[2])), ref_id(reference_id) {}
};
static_assert(sizeof(Aabb) == sizeof(stq_aabb), "Aabb must keep the 44-byte layout");

// sizeof of the reference's narrow-phase records (src/memory.cuh:21-67), used
// only to leave room for the narrow phase when sizing the pair buffer.
constexpr size_t kCCDConfigBytes = 56;
constexpr size_t kCCDDataBytes = 256;

struct MemHandler {
  size_t MAX_OVERLAP_CUTOFF = 0;
  size_t MAX_OVERLAP_SIZE = 0;
  size_t MAX_UNIT_SIZE = 0;
  size_t MAX_QUERIES = 0;
  int realcount = 0;
  int limitGB = 0;

  // min(0.95 free, limitGB GiB - used) (src/memory.cuh:78-94); limitGB = 0
  // means no user limit.
  size_t __getAllocatable() {
    size_t free_b = 0, total = 0;
    if (cudaMemGetInfo(&free_b, &total) != cudaSuccess) throw Error(STQ_ERR_CUDA, "cudaMemGetInfo");
    const size_t used = total - free_b;
    const size_t def = size_t(0.95 * double(free_b));
    if (limitGB <= 0) return def;
    const size_t lim = size_t(limitGB) << 30;
    return std::min(def, lim > used ? lim - used : size_t(0));
  }
  // src/memory.cuh:163-167
  size_t __getLargestOverlap() {
    const size_t a = __getAllocatable();
    const size_t n = a > kCCDConfigBytes ? (a - kCCDConfigBytes) / (kCCDDataBytes + 3 * sizeof(int2)) : 0;
#ifdef STQ_GPU_MAX_OVERLAP_SIZE
    return std::min<size_t>(n, size_t(STQ_GPU_MAX_OVERLAP_SIZE));
#else
    return n;
#endif
  }
  void setOverlapSize() { MAX_OVERLAP_SIZE = __getLargestOverlap(); }
  // src/memory.cuh:171-188
  void handleBroadPhaseOverflow(size_t desired_count) {
    MAX_OVERLAP_SIZE = std::min(__getLargestOverlap(), desired_count);
    if (MAX_OVERLAP_SIZE < desired_count) MAX_OVERLAP_CUTOFF = std::max<size_t>(1, MAX_OVERLAP_CUTOFF / 2);
  }
};

namespace detail {

inline void check(int st, stq_context *ctx = nullptr) {
  if (st != STQ_OK && st != STQ_OVERFLOW)
    throw Error(st, ctx ? stq_context_last_error(ctx) : stq_status_string(st));
}

inline void cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(STQ_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The process-wide context of the drop-in functions (device 0, default
// stream), as the reference keeps its state in globals.
inline stq_context *context() {
  static stq_context *ctx = [] {
    stq_context *c = nullptr;
    check(stq_context_create(0, nullptr, &c));
    return c;
  }();
  return ctx;
}

template <typename M, typename T>
std::vector<T> row_major(const M &m, int cols) {
  std::vector<T> out(size_t(m.rows()) * cols);
  for (long i = 0; i < long(m.rows()); ++i)
    for (int j = 0; j < cols; ++j) out[size_t(i) * cols + j] = T(m(i, j));
  return out;
}

template <typename T>
struct DeviceArray {
  T *p = nullptr;
  explicit DeviceArray(size_t n) { cuda(cudaMalloc(&p, sizeof(T) * (n ? n : 1)), "cudaMalloc"); }
  DeviceArray(const T *h, size_t n) : DeviceArray(n) {
    if (n) cuda(cudaMemcpy(p, h, sizeof(T) * n, cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  ~DeviceArray() { cudaFree(p); }
  DeviceArray(const DeviceArray &) = delete;
  DeviceArray &operator=(const DeviceArray &) = delete;
};

}  // namespace detail

// Swept boxes of vertices, edges and faces, built on the device.
template <typename MatD, typename MatI>
void constructBoxes(const MatD &vertices_t0, const MatD &vertices_t1, const MatI &edges,
                    const MatI &faces, std::vector<Aabb> &boxes, int threads = -1,
                    Scalar inflation_radius = 0) {
  (void)threads;  // host thread count of the reference's TBB build; unused here
  const auto V0 = detail::row_major<MatD, double>(vertices_t0, 3);
  const auto V1 = detail::row_major<MatD, double>(vertices_t1, 3);
  const auto E = detail::row_major<MatI, int32_t>(edges, 2);
  const auto F = detail::row_major<MatI, int32_t>(faces, 3);
  const int64_t nV = vertices_t0.rows(), nE = edges.rows(), nF = faces.rows();
  const size_t offset = boxes.size();
  detail::DeviceArray<double> dV0(V0.data(), V0.size()), dV1(V1.data(), V1.size());
  detail::DeviceArray<int32_t> dE(E.data(), E.size()), dF(F.data(), F.size());
  detail::DeviceArray<stq_aabb> dB(size_t(nV + nE + nF));
  stq_context *ctx = detail::context();
  detail::check(stq_build_boxes(ctx, dV0.p, dV1.p, nV, dE.p, nE, dF.p, nF, inflation_radius, dB.p), ctx);
  boxes.resize(offset + size_t(nV + nE + nF));
  detail::cuda(cudaMemcpy(boxes.data() + offset, dB.p, sizeof(stq_aabb) * size_t(nV + nE + nF),
                          cudaMemcpyDeviceToHost),
               "cudaMemcpy");
  // the reference numbers ids from the current size of `boxes`
  for (size_t i = offset; i < boxes.size(); ++i) boxes[i].id += int(offset);
}

// First sweep position of start box t (t in [0, N]) of a prepared scene with
// `length` positions: positions [pos(t0), pos(t1)) are the share of start
// boxes [t0, t1). pos(0) = 0, pos(N) = length, monotone, and since a scene has
// at least N positions (every box has at least one replica) every start box
// gets at least one position. The cursor and cutoff of run_sweep_sharedqueue
// count start boxes, as the reference's do, through this map.
inline int64_t start_position(int64_t t, int64_t N, int64_t length) {
  if (N <= 0 || t >= N) return length;
  return t <= 0 ? 0 : t * length / N;
}

// STQ sweep of host boxes; pairs stay on the device in d_overlaps[0..*d_count).
// One call sweeps start boxes [tidstart, tidstart + MAX_OVERLAP_CUTOFF) and
// advances tidstart by the cutoff (src/simulation.cu:747), so a single call
// with the default cutoff N sweeps the whole scene (app/main.cu:140-143), and
// a caller that loops `while (tidstart < N)` gets every pair exactly once. On
// overflow the call reruns its range with the buffer grown, or with the cutoff
// halved (src/memory.cuh:171-188), as the reference's loop does
// (src/simulation.cu:714-745). The sweep axis is x, as in the reference
// (src/simulation.cu:637), so every resumed call sees the same sorted order.
inline void run_sweep_sharedqueue(const Aabb *boxes, MemHandler *memhandle, int N, int nbox,
                                  std::vector<std::pair<int, int>> &finOverlaps,
                                  int2 *&d_overlaps, int *&d_count, int &threads, int &tidstart,
                                  int &devcount, const int memlimit = 0) {
  (void)nbox;
  (void)threads;
  (void)devcount;
  if (!memhandle->MAX_OVERLAP_CUTOFF) memhandle->MAX_OVERLAP_CUTOFF = size_t(N);
  if (memlimit) memhandle->limitGB = memlimit;
  stq_context *ctx = detail::context();
  {
    detail::DeviceArray<stq_aabb> dB(reinterpret_cast<const stq_aabb *>(boxes), size_t(N));
    detail::check(stq_prepare(ctx, dB.p, N, STQ_AXIS_X), ctx);
  }
  const int64_t length = stq_prepared_length(ctx);
  memhandle->setOverlapSize();
  detail::cuda(cudaMalloc(&d_count, sizeof(int)), "cudaMalloc");
  int64_t count = 0, next = 0, total = 0;
  while (true) {
    detail::cuda(cudaMalloc(&d_overlaps, sizeof(int2) * std::max<size_t>(1, memhandle->MAX_OVERLAP_SIZE)),
                 "cudaMalloc");
    const int64_t t1 = std::min<int64_t>(int64_t(N), int64_t(tidstart) + int64_t(memhandle->MAX_OVERLAP_CUTOFF));
    const int64_t p0 = start_position(tidstart, N, length), p1 = start_position(t1, N, length);
    if (p1 <= p0) {  // nothing left to sweep
      count = 0;
      break;
    }
    const int st = stq_sweep_prepared(ctx, p0, p1 - p0, reinterpret_cast<stq_pair *>(d_overlaps),
                                      int64_t(memhandle->MAX_OVERLAP_SIZE), &count, &next, &total);
    if (st == STQ_OK) break;
    if (st != STQ_OVERFLOW && st != STQ_ERR_CAPACITY) detail::check(st, ctx);
    // the partial result is dropped: the range is swept again whole
    cudaFree(d_overlaps);
    d_overlaps = nullptr;
    const size_t before = memhandle->MAX_OVERLAP_SIZE, cut = memhandle->MAX_OVERLAP_CUTOFF;
    memhandle->handleBroadPhaseOverflow(size_t(total));
    if (memhandle->MAX_OVERLAP_SIZE == before && memhandle->MAX_OVERLAP_CUTOFF == cut)
      throw Error(STQ_ERR_NO_MEMORY, "pair buffer cannot grow and the cutoff cannot shrink");
  }
  memhandle->realcount = int(count);
  tidstart = int(std::min<int64_t>(int64_t(tidstart) + int64_t(memhandle->MAX_OVERLAP_CUTOFF), INT32_MAX));
  const int c = int(count);
  detail::cuda(cudaMemcpy(d_count, &c, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
#ifdef KEEP_CPU_OVERLAPS
  std::vector<int2> h(static_cast<size_t>(count));
  if (count)
    detail::cuda(cudaMemcpy(h.data(), d_overlaps, sizeof(int2) * size_t(count), cudaMemcpyDeviceToHost),
                 "cudaMemcpy");
  finOverlaps.reserve(finOverlaps.size() + h.size());
  for (const int2 &p : h) finOverlaps.emplace_back(p.x, p.y);
#else
  (void)finOverlaps;
#endif
}

// Plain sweep with host output (the reference's default path); one device.
inline void run_sweep_multigpu(const Aabb *boxes, int N, int nbox,
                               std::vector<std::pair<int, int>> &finOverlaps, int &threads,
                               int &devcount) {
  (void)nbox;
  (void)threads;
  (void)devcount;
  stq_context *ctx = detail::context();
  finOverlaps.clear();
  int64_t cap = std::max<int64_t>(1024, int64_t(N) * 8);
  while (true) {
    std::vector<stq_pair> h(static_cast<size_t>(cap));
    int64_t count = 0, total = 0;
    const int st = stq_sweep_host(ctx, reinterpret_cast<const stq_aabb *>(boxes), N, STQ_AXIS_AUTO,
                                  h.data(), cap, &count, &total);
    detail::check(st, ctx);
    if (st == STQ_OK) {
      finOverlaps.reserve(size_t(count));
      for (int64_t i = 0; i < count; ++i) finOverlaps.emplace_back(h[size_t(i)].first, h[size_t(i)].second);
      return;
    }
    cap = total;  // the reference reruns once with the exact count (simulation.cu:473-489)
  }
}

}  // namespace stq::gpu
