// context.h - the object behind stq_context* and the pipeline helpers shared
// by the C ABI (abi.cu) and the serving loop (server.cu).
#pragma once

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "stq_device.cuh"
#include "stq_internal.h"

using namespace stq;

constexpr int kStages = 8;
const char *const kStageNames[kStages] = {"build", "axis", "keys", "sort",
                                          "gather", "sweep", "count_sweep", "pair_sort"};
enum Stage { kBuild, kAxis, kKeys, kSort, kGather, kSweep, kCountSweep, kPairSort };

// Input block uploaded with one copy before every prepare: the batch header,
// the scene offsets (boxes, and vertices/edges/faces for batched builds), the
// per-scene options and the tile table. Offsets are fixed by the capacities.
struct Staging {
  int scene_cap = 0, tile_cap = 0;
  size_t hdr = 0, box_off = 0, voff = 0, eoff = 0, foff = 0, inputs = 0, tiles = 0, total = 0;
  static Staging make(int scene_cap, int tile_cap) {
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    Staging st;
    st.scene_cap = scene_cap;
    st.tile_cap = tile_cap;
    size_t o = 0;
    st.hdr = o, o = up(o + sizeof(BatchHeader));
    const size_t offs = sizeof(long long) * size_t(scene_cap + 1);
    st.box_off = o, o = up(o + offs);
    st.voff = o, o = up(o + offs);
    st.eoff = o, o = up(o + offs);
    st.foff = o, o = up(o + offs);
    st.inputs = o, o = up(o + sizeof(SceneInput) * size_t(scene_cap));
    st.tiles = o, o = up(o + sizeof(TileRec) * size_t(tile_cap));
    st.total = o;
    return st;
  }
};

struct GraphKey {
  const void *ptr[7] = {};
  int64_t sizes[9] = {};
  int64_t opts[17] = {};  // every context option, then the inflation radius
  cudaStream_t stream = nullptr;
  bool operator==(const GraphKey &o) const {
    return std::memcmp(ptr, o.ptr, sizeof ptr) == 0 && std::memcmp(sizes, o.sizes, sizeof sizes) == 0 &&
           std::memcmp(opts, o.opts, sizeof opts) == 0 && stream == o.stream;
  }
};

struct stq_context {
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;  // created by a server for graph capture
  std::string error;
  int64_t launches = 0;
  SweepTuning tuning;
  int64_t options[16] = {};
  float cell_scale = 2.f;
  int budget = 4;

  // capacities of the batch buffers
  int scene_cap = 0, tile_cap = 0;
  int64_t box_cap = 0, rep_cap = 0, slot_cap = 0;
  Staging layout;
  DevBuf in_dev;
  char *in_host = nullptr;
  size_t in_host_bytes = 0;
  DevBuf scenes, cell_base, scene_pairs, counts, offsets, box_cells, scan_ws, keys64[2], vals[2], sort_ws;
  DevBuf points;  // fp64 vertex positions rounded to float once (box builds)
  DevBuf xmin, xmax, syz, sv, sflag, sfloor, partner, run_end, box_counts, prefix_ws, pair_keys[2];
  DevBuf cell_floor;  // lower bounds of each cell on b and c
  DevBuf long_list;  // runs handed from the lane sweep to the warp pass
  DevBuf seg_scan;  // first sorted replica of each (cell, type) list
  DevBuf bkeys[2], bvals[2];  // box sort: keys and box indices, double-buffered
  int order_buf = 0;          // which bvals buffer holds the sorted box order
  int64_t seg_cap = 0;
  DevBuf batch_boxes, e2e_boxes, e2e_pairs, e2e_mesh;
  DevBuf aux;  // header of calls outside a batch (box build, all-pairs check)

  // prepared batch (host view)
  bool prepared = false;
  int n_scenes = 0;
  int64_t n_boxes = 0, length = 0;
  SortedScene scene;
  BatchHeader *h_hdr = nullptr;             // pinned readback
  unsigned long long *h_scene_pairs = nullptr;  // pinned readback
  int h_scene_pairs_cap = 0;

  // captured graph of stq_batch_broadphase, on a private stream (the legacy
  // default stream cannot be captured)
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t graph_event = nullptr;
  cudaGraphExec_t graph = nullptr;
  GraphKey graph_key;
  bool capturing = false;

  // host-buffer calls: windows alternate between two sweep streams, each with
  // its own pair buffer, counters and long-run list (slot 0 is the context's
  // stream, e2e_pairs and long_list); a third stream copies pairs to the host
  static constexpr int kCopyWindows = 32;
  cudaStream_t copy_stream = nullptr, window_stream = nullptr;
  cudaEvent_t window_start = nullptr;
  cudaEvent_t window_done[kCopyWindows] = {};
  unsigned long long *h_window_pairs = nullptr;  // page-locked, mapped
  unsigned long long *d_window_pairs = nullptr;  // its device address
  DevBuf window_pairs, window_long_list, window_cursors;

  // autotuner cache: shape bucket -> options (lanes, queue, block, radix, scale)
  std::vector<std::pair<int64_t, std::vector<int64_t>>> tuned;

  // stage timers
  bool timing = false;
  cudaEvent_t ev[kStages][2] = {};
  bool pending[kStages] = {};
  double stage_ms[kStages] = {};
  int64_t stage_calls[kStages] = {};
};


namespace stq {
namespace ctxops {

struct DeviceGuard {
  int prev = -1;
  bool changed = false;
  explicit DeviceGuard(int dev);
  ~DeviceGuard();
};

int fail(stq_context *ctx, int status, const char *what, cudaError_t e = cudaSuccess);
void collect_stages(stq_context *ctx);
void stage_begin(stq_context *ctx, int st);
void stage_end(stq_context *ctx, int st);
BatchHeader *dev_hdr(stq_context *ctx);
int read_header(stq_context *ctx, const BatchHeader *src = nullptr);
int64_t tiles_for(const int64_t *box_off, int S);
int ensure_staging(stq_context *ctx, int scene_cap, int tile_cap);
void fill_staging(stq_context *ctx, const int64_t *box_off, int S, const int *axes, int axis,
                  const int64_t *voff, const int64_t *eoff, const int64_t *foff);
int upload_staging(stq_context *ctx);
BatchBuffers batch_buffers(stq_context *ctx, const stq_aabb *boxes);
int ensure_box_buffers(stq_context *ctx, int64_t box_cap);
int ensure_replica_buffers(stq_context *ctx, int64_t rep_cap, int64_t cells_cap);
int bits_for(int64_t v);
// Statistics, axis and grid per scene, the box sort along the sweep axis,
// replica counts per sorted position and their scan. n_boxes: the box count,
// or -1 when only the device knows it (graph capture, serving).
int enqueue_prepare_front(stq_context *ctx, const BatchBuffers &b, int64_t n_boxes);
// Replica emit in sweep-axis order, list counts and offsets, and the stable
// sort by list id (seg_bits bits) that turns it into x-sorted cell lists;
// then the sorted scene. replicas: the replica count, or -1 (device count).
int enqueue_prepare_back(stq_context *ctx, const BatchBuffers &b, int seg_bits, int64_t n_boxes,
                         int64_t replicas);
// Launches one sweep over start positions [begin, end). With cursors null it
// first clears the batch header's pair counter, cursors, per-scene counts and
// statistics and uses them and the context's long-run list; otherwise it uses
// the given counters (cleared by the caller on the launch stream) and
// launches on stream, keeping the header's statistics. timed: record the
// launch as one sweep stage (a windowed caller times its windows as one).
int run_sweep(stq_context *ctx, int64_t begin, int64_t end, stq_pair *pairs, long long capacity,
              bool count_mode, bool timed = true,
              const SweepCursors *cursors = nullptr, cudaStream_t stream = nullptr);

template <typename T>
T *dev_at(stq_context *ctx, size_t off) {
  return reinterpret_cast<T *>(ctx->in_dev.as<char>() + off);
}
template <typename T>
T *host_at(stq_context *ctx, size_t off) {
  return reinterpret_cast<T *>(ctx->in_host + off);
}

constexpr int64_t kMaxBoxes = int64_t(INT32_MAX) - 4 * kSortedPad;

}  // namespace ctxops
}  // namespace stq

#define STQ_CUDA(ctx, call, what)                                                              \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess)                                                                     \
      return ::stq::ctxops::fail((ctx), _e == cudaErrorMemoryAllocation ? STQ_ERR_NO_MEMORY    \
                                                                         : STQ_ERR_CUDA,       \
                                 (what), _e);                                                  \
  } while (0)

#define STQ_TRY(expr)              \
  do {                             \
    const int _st = (expr);        \
    if (_st != STQ_OK) return _st; \
  } while (0)
