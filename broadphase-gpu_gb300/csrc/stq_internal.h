// stq_internal.h - host-side internals shared by the CUDA translation units:
// the context object behind stq_context*, grow-only device buffers and the
// kernel launch wrappers.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/stq_abi.h"

namespace stq {

// Grow-only device allocation owned by a context.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t rounded = (want + 4095) & ~size_t(4095);
    cudaError_t e = cudaMalloc(&ptr, rounded);
    if (e == cudaSuccess) bytes = rounded;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// Device-side scalars of one sweep: counters, flags and results read back
// by the host in a single copy.
struct DevScalars {
  unsigned long long count;  // pairs found (keeps counting past capacity)
  int work;                  // start-box grab cursor of the sweep kernel
  int flags;                 // kFlag* bits set by kernels
  long long prefix;          // start boxes of the longest prefix that fits
  int axis;                  // sweep axis chosen on the device
  int pad[3];
};

enum : int {
  kFlagNaN = 1,        // a box bound is NaN
  kFlagBadIndex = 2,   // an edge or face index is outside [0, nV)
};

// Cell grid on the two non-sweep axes b, c (the other two axes in increasing
// order). A box is replicated into every cell its [min, max] range touches;
// cell coordinates are a monotone function of the bound, so a pair that
// overlaps shares the cell of its reference point (max of mins on b and c)
// and is emitted there only.
struct GridParams {
  int axis;       // sweep axis a
  int nb, nc;     // cells along b and c
  int ncells;     // nb * nc
  int cell_bits;  // bits of the largest cell id
  int inverted;   // some box has min > max on b or c: cells disabled
  float ob, oc;   // grid origin on b and c
  float ib, ic;   // cells per unit length on b and c
};

// Per-scene statistics gathered in one pass over the boxes.
struct SceneStats {
  unsigned int lo_key[3];   // order-preserving min of the minima
  unsigned int hi_key[3];   // order-preserving max of the maxima
  unsigned int hist[3][64]; // log2 histogram of the box extents
  int inverted;             // some box has min > max
  int pad;
};

// Sweep-kernel tuning (autotuned or set through stq_context_set_option).
struct SweepTuning {
  int lanes = 8;        // lanes sharing one pending start box (1..32)
  int queue = 64;       // warp queue depth (32, 64, 128)
  int block = 256;      // threads per block (128, 256, 512)
  int chunk = 256;      // start boxes per work grab
};

// Sorted scene in HBM, structure of arrays, one sentinel after the boxes
// (sx = NaN) followed by kSortedPad padding entries.
struct SortedScene {
  float2 *sx = nullptr;   // (min, max) on the sweep axis
  float4 *syz = nullptr;  // (min_b, min_c, max_b, max_c) on the other axes
  int4 *sv = nullptr;     // (vertexIds[0..2], id)
  int *scell = nullptr;   // cell id of each position (cells mode)
  int64_t length = 0;     // sweep positions (boxes; sentinels excluded at the end)
};

struct SweepParams {
  const float2 *sx;
  const float4 *syz;
  const int4 *sv;
  int32_t begin, end;        // start positions [begin, end)
  int32_t chunk;             // start positions per grab
  stq_pair *pairs;
  long long capacity;
  unsigned long long *count;
  int *work;
  int32_t *box_counts;       // count mode: pairs per start position (k - begin)
  const int *scell;          // cells mode: cell id per position, else null
  const GridParams *grid;    // cells mode: grid on the device
};

// ---- launch wrappers (each returns the launch error) -------------------------
cudaError_t launch_build_boxes(cudaStream_t s, const double *V0, const double *V1,
                               int64_t nV, const int32_t *E, int64_t nE,
                               const int32_t *F, int64_t nF, float r_up,
                               stq_aabb *out, int *flags);
// axis: partial sums then the final choice, written to *d_axis
cudaError_t launch_axis_select(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               double *partials, int nblocks, int *d_axis);
int axis_partial_blocks(int64_t n);
// keys/values for the sort; axis read from *d_axis
cudaError_t launch_prep_keys(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                             const int *d_axis, uint32_t *keys, uint32_t *vals,
                             int *flags);
cudaError_t launch_gather(cudaStream_t s, const stq_aabb *boxes,
                          const uint32_t *order, int64_t n, const int *d_axis,
                          SortedScene scene);

// ---- cells mode ------------------------------------------------------------------
// stats: one pass; grid: policy kernel (mode: -1 auto axis, else the axis;
// cells_opt: 0 automatic, 1 no cells, k > 1 a k x k grid; scale: cell side
// in median box extents)
size_t stats_partials_bytes(int64_t n);
cudaError_t launch_scene_stats(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               double *partials, SceneStats *stats, int *flags);
cudaError_t launch_grid_policy(cudaStream_t s, const double *partials, int64_t n,
                               const SceneStats *stats, int axis_mode, int cells_opt,
                               float scale, GridParams *grid, int *d_axis);
cudaError_t launch_replica_count(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                                 const GridParams *grid, uint32_t *counts);
cudaError_t launch_replica_emit(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                                const GridParams *grid, const uint32_t *offsets,
                                unsigned long long *keys, uint32_t *vals);
cudaError_t launch_fill_sentinels(cudaStream_t s, float2 *sx, int64_t slots);
cudaError_t launch_gather_cells(cudaStream_t s, const stq_aabb *boxes,
                                const unsigned long long *keys, const uint32_t *order,
                                int64_t R, const GridParams *grid, SortedScene scene);

// LSD radix sort of (uint32 key, uint32 value) or (uint64 key) pairs.
// kbuf/vbuf are double buffers; *which receives the buffer index holding the
// result. Returns workspace bytes when called with workspace == nullptr.
size_t radix_workspace_bytes(int64_t n, int key_bytes, int bits);
cudaError_t radix_sort_u32(cudaStream_t s, uint32_t *kbuf[2], uint32_t *vbuf[2],
                           int64_t n, int bits, void *workspace, int *which,
                           int64_t *launches);
cudaError_t radix_sort_u64(cudaStream_t s, unsigned long long *kbuf[2],
                           int64_t n, int begin_bit, int end_bit, void *workspace,
                           int *which, int64_t *launches);
cudaError_t radix_sort_u64_vals(cudaStream_t s, unsigned long long *kbuf[2],
                                uint32_t *vbuf[2], int64_t n, int begin_bit, int end_bit,
                                void *workspace, int *which, int64_t *launches);
// exclusive scan of n uint32 counts; *d_total receives the sum
size_t scan_workspace_bytes(int64_t n);
cudaError_t exclusive_scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n,
                               void *workspace, uint32_t *d_total, int64_t *launches);

cudaError_t launch_sweep(cudaStream_t s, const SweepParams &p,
                         const SweepTuning &t, bool count_mode, int num_sms);
// inclusive scan of box_counts[0..m) and the longest prefix whose pair sum
// is <= capacity -> scalars->prefix
size_t prefix_workspace_bytes(int64_t m);
cudaError_t launch_prefix_select(cudaStream_t s, const int32_t *box_counts,
                                 int64_t m, long long capacity, void *workspace,
                                 DevScalars *scalars, int64_t *launches);
cudaError_t launch_brute_force(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               stq_pair *pairs, long long capacity,
                               unsigned long long *count);
cudaError_t launch_pairs_to_keys(cudaStream_t s, const stq_pair *pairs, int64_t n,
                                 unsigned long long *keys, bool to_keys);

}  // namespace stq
