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
  kFlagReplicaOverflow = 4,  // cell replicas exceed the replica buffers
};

// Cells per axis of a scene's grid at most (automatic or STQ_OPT_CELLS); cell
// coordinates then fit 11 bits, as the per-box cell records pack them.
constexpr int kMaxGridSide = 2048;

// Cell grid on the two non-sweep axes b, c (the other two axes in increasing
// order). A box is replicated into every cell its [min, max] range touches;
// cell coordinates are a monotone function of the bound, so a pair that
// overlaps shares the cell of its reference point (max of mins on b and c)
// and is emitted there only.
// The policy sets the level-0 grid (nb0 x nc0 cells of the automatic side, or
// the requested grid); a cell of level L is a block of 2^L x 2^L level-0
// cells, and the level is chosen against the replica budget once the box-key
// pass has counted every level's replicas.
struct GridParams {
  int axis;       // sweep axis a
  int nb, nc;     // cells along b and c at the chosen level
  int ncells;     // nb * nc
  float ob, oc;   // grid origin on b and c
  float ib, ic;   // level-0 cells per unit length on b and c
  float Lb, Lc;   // extent of the scene on b and c
  int nb0, nc0;   // level-0 cells along b and c
  int shift;      // cell coordinate = level-0 coordinate >> shift (the chosen
                  // level; kCoordBits when no level fits: one cell)
  int pad;
};

constexpr int kGridLevels = 6;  // level L halves the level-0 grid L times
constexpr int kCoordBits = 11;  // level-0 cell coordinates are below 2^11
static_assert(kMaxGridSide <= (1 << kCoordBits), "level-0 cell coordinates fit kCoordBits");

// One scene of a batch: inputs written by the host, the rest computed on the
// device by the prepare kernels.
struct SceneRecord {
  // inputs
  int axis_mode;        // -1: largest variance, else the axis
  int cells_opt;        // 0 automatic, 1 no cells, k > 1 a k x k grid
  float cell_scale;     // automatic cell side in median box extents
  int pad0;
  // statistics
  double s1[3], s2[3];              // sum(min + max), sum(min^2 + max^2)
  unsigned int lo_key[3], hi_key[3];  // order-preserving min / max bounds
  unsigned int hist[3][64];         // log2 histogram of the extents
  int inverted;                     // some box has min > max on an axis
  int pad1;
  unsigned long long level_reps[kGridLevels];  // replicas per grid level
  // results
  GridParams grid;
};

// Per-scene inputs written by the host (copied into the records on reset).
struct SceneInput {
  int axis_mode;
  int cells_opt;
  float cell_scale;
  int pad;
};

// Device-side header of a prepared batch: sizes read by every kernel, so a
// captured graph can be replayed for any batch within its capacities.
struct BatchHeader {
  long long n_boxes;        // input: boxes in the batch
  int n_scenes;             // input: scenes
  int flags;                // kFlag* bits
  unsigned int replicas;    // R, cell replicas
  unsigned int cells;       // total cells of all scenes
  unsigned int length;      // sweep positions: R + 3 * cells - 1
  int work;                 // sweep grab cursor
  unsigned int long_items;  // runs handed from the lane sweep to the warp pass
  unsigned int long_work;   // warp pass grab cursor
  unsigned long long pairs; // pairs found by the last sweep
  long long prefix;         // overflow: start positions of the prefix that fits
  int axis;                 // sweep axis of scene 0
  int budget;               // replica budget: replicas <= budget * boxes per scene
  int n_tiles;              // input: entries of the tile table
  unsigned int max_list;    // longest (cell, type) list
  unsigned int box_count;   // input: n_boxes as the element count of the box sort
  unsigned long long candidates;  // candidates tested by the last sweep
  unsigned int lists;       // (cell, type) lists: 3 * cells
  unsigned int pad;
};

// A tile of at most kTileBoxes consecutive boxes of one scene (built by the
// host from the scene offsets), so that a block reduces per-scene values once.
constexpr int kTileBoxes = 4096;
struct TileRec {
  long long begin;  // first box of the tile
  int count;        // boxes in the tile
  int scene;        // scene of the tile
};

// Sweep shapes (STQ_OPT_SWEEP_SHAPE): a per-warp ring of pending start boxes
// taken by lanes or lane groups, or the flat shape (each warp's 32 starts'
// runs laid end to end, one candidate per lane and step).
constexpr int kShapeRing = 1;
constexpr int kShapeFlat = 2;

// Sweep-kernel tuning (autotuned or set through stq_context_set_option).
struct SweepTuning {
  int shape = kShapeFlat;  // kShapeFlat or kShapeRing
  int lanes = 1;        // lanes sharing one pending start box (1..32)
  int per_lane = 8;     // lanes = 1: candidates a lane tests per step (1, 2, 4, 8)
  int run_cap = 512;    // candidates per start box before the warp pass takes over
  int queue = 64;       // warp queue depth (32, 64, 128)
  int block = 256;      // threads per block (128, 256, 512)
  int chunk = 256;      // start boxes per work grab
};

// Sorted scene in HBM, structure of arrays, one sentinel after the boxes
// (xmin = xmax = NaN) followed by kSortedPad padding entries.
struct SortedScene {
  float *xmin = nullptr;  // min on the sweep axis (all a candidate needs)
  float *xmax = nullptr;  // max on the sweep axis (read once per start box)
  float4 *syz = nullptr;  // (min_b, min_c, max_b, max_c) on the other axes
  int4 *sv = nullptr;     // (vertexIds[0..2], id)
  int *sflag = nullptr;   // first-cell bits (0: along b, 1: along c), scene << 2
  float2 *sfloor = nullptr;  // per axis b, c: -inf where the cell is the box's
                             // first, else the cell's lower bound
  int *partner = nullptr; // first candidate position of each start position
  int *run_end = nullptr; // one past its last candidate on the sweep axis
  int64_t length = 0;     // sweep positions (boxes; sentinels excluded at the end)
};

// Counters of one sweep launch that runs beside another (a host call's
// windows alternate between two of these), in device memory.
struct WindowCounters {
  unsigned long long pairs;  // pairs found
  int work;                  // grab cursor
  unsigned int long_items;   // runs handed to the warp pass
  unsigned int long_work;    // warp pass grab cursor
  int pad;
};

// Where one sweep launch keeps its counters and handed-over runs.
struct SweepCursors {
  unsigned long long *count;
  int *work;
  int2 *long_list;
  unsigned int *long_items;
  unsigned int *long_work;
};

struct SweepParams {
  const float *xmin;
  const float *xmax;
  const float4 *syz;
  const int4 *sv;
  int32_t begin, end;        // start positions [begin, min(end, hdr->length))
  int32_t chunk;             // start positions per grab
  stq_pair *pairs;
  long long capacity;
  unsigned long long *count;
  int *work;
  int32_t *box_counts;       // count mode: pairs per start position (k - begin)
  const int *sflag;          // first-cell bits and scene of each position
  const float2 *sfloor;      // first-cell rule of a start position on b and c:
                             // a candidate passes if its minima are >= these
  const int *partner;        // first candidate position of each start position
  const int *run_end;        // one past its last candidate (null: not computed;
                             // the flat shape needs it)
  unsigned long long *scene_pairs;  // per-scene pair counters
  const BatchHeader *hdr;    // device sizes (length bounds the sweep range)
  unsigned long long *stats; // candidates tested (may be null)
  int typed;                 // every list holds one box type, so every candidate
                             // pair is V-F, F-V or E-E (is_valid_pair holds)
  int run_cap;               // candidates of one start box a lane (group) tests
                             // before it hands the rest of the run to the warp
                             // pass; 0 = never
  int2 *long_list;           // handed-over runs (start position, next candidate)
  unsigned int *long_items;  // their count
  unsigned int *long_work;   // warp pass grab cursor
};

// ---- launch wrappers (each returns the launch error) -------------------------
// points: 2 * nV float4 of scratch for the rounded positions
cudaError_t launch_build_boxes(cudaStream_t s, const double *V0, const double *V1,
                               int64_t nV, const int32_t *E, int64_t nE,
                               const int32_t *F, int64_t nF, float r_up,
                               stq_aabb *out, int *flags, float4 *points);

// ---- batch prepare (scene table) ---------------------------------------------------
// Buffers sized by host capacities; actual sizes come from the BatchHeader.
struct BatchBuffers {
  const stq_aabb *boxes;
  const long long *box_off;     // n_scenes + 1 box offsets
  const TileRec *tiles;         // n_tiles entries
  int tile_cap;
  const SceneInput *inputs;     // n_scenes entries
  unsigned long long *scene_pairs;  // n_scenes pair counters
  SceneRecord *scenes;
  unsigned int *cell_base;      // n_scenes + 1
  BatchHeader *hdr;
  uint32_t *counts, *offsets;   // per box position in sweep-axis order
  uint2 *box_cells;             // per box index: cell range and type
                                // (b0 | b1 << 11 | type << 22, c0 | c1 << 11)
  uint32_t *box_keys, *box_vals;  // box sort input (key, box index), double-buffered with
  uint32_t *box_keys2, *box_vals2;
  const uint32_t *order;        // boxes in sweep-axis order (box sort output)
  const uint32_t *sorted_keys;  // their sort keys (sweep-axis minimum images)
  unsigned long long *keys;     // replica keys (sort input)
  uint32_t *vals;               // replica box indices (sort input)
  uint32_t *seg_scan;           // first sorted replica of each segment (cell x type),
                                // seg_cap + 1 entries
  long long seg_cap;
  long long box_cap;            // capacities
  long long rep_cap;
  int scene_cap;
};
// reset and per-scene statistics (2 launches)
cudaError_t launch_batch_stats(cudaStream_t s, const BatchBuffers &b);
// sweep axis and level-0 grid per scene (1 launch)
cudaError_t launch_batch_policy(cudaStream_t s, const BatchBuffers &b);
// box sort keys, level-0 cell ranges and every level's replica count; then the
// level within the replica budget and the cell bases (2 launches)
cudaError_t launch_batch_box_keys(cudaStream_t s, const BatchBuffers &b);
// n: positions to cover (the box count, or the box capacity when only the
// device knows the count)
cudaError_t launch_batch_counts(cudaStream_t s, const BatchBuffers &b, int64_t n);
cudaError_t launch_batch_emit(cudaStream_t s, const BatchBuffers &b, int64_t n, int num_sms);
// list offsets from the list-sorted keys (and the longest list); the NaN
// sentinel after every list and the padding after the last
cudaError_t launch_list_offsets(cudaStream_t s, const unsigned long long *keys, BatchHeader *hdr, uint32_t *seg_scan,
                                int64_t seg_cap, const SortedScene &scene, int64_t slots_cap);

cudaError_t launch_gather_cells(cudaStream_t s, const stq_aabb *boxes,
                                const unsigned long long *keys, const uint32_t *order,
                                const BatchHeader *hdr, int64_t rep_cap,
                                const unsigned int *cell_base, const SceneRecord *scenes,
                                const uint32_t *seg_scan, float2 *cell_floor, int64_t cells_cap,
                                SortedScene scene);
// Batched box build: scene s has vertices [voff[s], voff[s+1]) etc.; box ids
// are global (box_off[s] + local), vertex ids local to the scene.
// points: 2 * vert_cap float4 of scratch for the rounded positions
cudaError_t launch_batch_build(cudaStream_t s, const double *V0, const double *V1,
                               const long long *voff, const int32_t *E, const long long *eoff,
                               const int32_t *F, const long long *foff, const long long *box_off,
                               BatchHeader *hdr, int64_t box_cap, float r_up, stq_aabb *out,
                               float4 *points, int64_t vert_cap);
// A scene held by the serving loop: its own device mesh and time-step state.
struct MeshRef {
  double *V0, *V1;
  const int32_t *E, *F;
  long long nV, nE, nF;
  unsigned long long seed;
  double sigma;
  int step;   // timestep about to run (0: the submitted positions)
  int pad;
};
cudaError_t launch_advance(cudaStream_t s, const MeshRef *refs, const long long *voff,
                           const BatchHeader *hdr, int64_t vert_cap);
cudaError_t launch_batch_build_refs(cudaStream_t s, const MeshRef *refs, const long long *box_off,
                                    BatchHeader *hdr, int64_t box_cap, float r_up, stq_aabb *out);
cudaError_t launch_pair_checksums(cudaStream_t s, const stq_pair *pairs, long long capacity,
                                  const BatchHeader *hdr, const long long *box_off,
                                  unsigned long long *checks, int scene_cap);
cudaError_t launch_reset_sweep(cudaStream_t s, BatchHeader *hdr, unsigned long long *scene_pairs,
                               int scene_cap);
// host_count: device address of page-locked, mapped host memory
cudaError_t launch_window_step(cudaStream_t s, WindowCounters *wc, unsigned long long *host_count);

// LSD radix sort of (uint32 key, uint32 value) or (uint64 key) pairs.
// kbuf/vbuf are double buffers; *which receives the buffer index holding the
// result. Returns workspace bytes when called with workspace == nullptr.
size_t radix_workspace_bytes(int64_t n, int key_bytes, int bits);
constexpr int kRadixTile = 2048;  // keys per radix tile (one per-digit count each)
cudaError_t radix_sort_u32(cudaStream_t s, uint32_t *kbuf[2], uint32_t *vbuf[2],
                           int64_t n, int bits, void *workspace, int *which,
                           int64_t *launches, const unsigned int *d_n = nullptr);
cudaError_t radix_sort_u64(cudaStream_t s, unsigned long long *kbuf[2],
                           int64_t n, int begin_bit, int end_bit, void *workspace,
                           int *which, int64_t *launches);
// d_hi (may be null): on the device, the number of distinct values of the
// keys' bits from begin_bit up; a pass whose digit is 0 in every key (all those
// values below 2^(its shift - begin_bit)) copies the keys through instead of
// ranking them, so a sort sized for a capacity (a captured graph) pays for
// the digits the actual keys use.
cudaError_t radix_sort_u64_vals(cudaStream_t s, unsigned long long *kbuf[2],
                                uint32_t *vbuf[2], int64_t n, int begin_bit, int end_bit,
                                void *workspace, int *which, int64_t *launches,
                                const unsigned int *d_n = nullptr, int bits = 8,
                                const unsigned int *d_hi = nullptr);
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
