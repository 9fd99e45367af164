// abi.cu - the C ABI of include/stq_abi.h: context, device buffers and the
// host driver of prepare -> sweep -> overflow-and-resume.
//
// Host driver reference: run_sweep_sharedqueue (src/simulation.cu:555-782).
// Differences that keep results exact and the call re-entrant per context:
// status codes instead of exit() (src/memory.cuh:8-19); grow-only buffers
// owned by the context instead of malloc/free per call; on overflow the
// pairs of the longest prefix of start boxes that fits are written and the
// resume cursor points after it, instead of rerunning with half the start
// boxes (src/memory.cuh:171-188, src/simulation.cu:714-747).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "stq_device.cuh"
#include "stq_internal.h"

using namespace stq;

constexpr int kStages = 8;
const char *const kStageNames[kStages] = {"build", "axis", "keys", "sort",
                                          "gather", "sweep", "count_sweep", "pair_sort"};
enum Stage { kBuild, kAxis, kKeys, kSort, kGather, kSweep, kCountSweep, kPairSort };

// Grid and replica count of the prepared scene, read back once per prepare.
struct PrepInfo {
  GridParams grid;
  uint32_t replicas;
  uint32_t pad;
};

struct stq_context {
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  std::string error;
  int64_t launches = 0;
  SweepTuning tuning;
  int64_t options[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int radix_bits = 8;

  // sorted scene
  bool prepared = false;
  int64_t n = 0;
  SortedScene scene;
  DevBuf sx, syz, sv;
  // sort and sweep scratch
  DevBuf keys[2], vals[2], sort_ws, scalars, partials, box_counts, prefix_ws;
  DevBuf pair_keys[2];
  // cells mode
  DevBuf stats, prep, counts, offsets, scan_ws, keys64[2], scell;
  PrepInfo *h_prep = nullptr;  // pinned readback
  float cell_scale = 4.f;
  // end-to-end staging
  DevBuf e2e_boxes, e2e_pairs, e2e_mesh;
  DevScalars *h_scalars = nullptr;  // pinned readback
  // stage timers
  bool timing = false;
  cudaEvent_t ev[kStages][2] = {};
  bool pending[kStages] = {};
  double stage_ms[kStages] = {};
  int64_t stage_calls[kStages] = {};
};

namespace {

struct DeviceGuard {
  int prev = -1;
  bool changed = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
      changed = cudaSetDevice(dev) == cudaSuccess;
    }
  }
  ~DeviceGuard() {
    if (changed) cudaSetDevice(prev);
  }
};

int fail(stq_context *ctx, int status, const char *what, cudaError_t e = cudaSuccess) {
  if (ctx) {
    char buf[512];
    if (e != cudaSuccess)
      std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    else
      std::snprintf(buf, sizeof buf, "%s", what);
    ctx->error = buf;
  }
  return status;
}

#define STQ_CUDA(ctx, call, what)                                        \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess)                                               \
      return fail((ctx), _e == cudaErrorMemoryAllocation ? STQ_ERR_NO_MEMORY : STQ_ERR_CUDA, \
                  (what), _e);                                           \
  } while (0)

__global__ void init_scalars_kernel(DevScalars *s, int axis) {
  s->count = 0;
  s->work = 0;
  s->flags = 0;
  s->prefix = 0;
  s->axis = axis;
}

__global__ void reset_sweep_kernel(DevScalars *s) {
  s->count = 0;
  s->work = 0;
}

void collect_stage(stq_context *ctx, int st) {
  if (!ctx->pending[st]) return;
  float ms = 0.f;
  if (cudaEventSynchronize(ctx->ev[st][1]) == cudaSuccess &&
      cudaEventElapsedTime(&ms, ctx->ev[st][0], ctx->ev[st][1]) == cudaSuccess) {
    ctx->stage_ms[st] += ms;
    ctx->stage_calls[st] += 1;
  }
  ctx->pending[st] = false;
}

void collect_stages(stq_context *ctx) {
  for (int st = 0; st < kStages; ++st) collect_stage(ctx, st);
}

void stage_begin(stq_context *ctx, int st) {
  if (!ctx->timing) return;
  collect_stage(ctx, st);
  cudaEventRecord(ctx->ev[st][0], ctx->stream);
}

void stage_end(stq_context *ctx, int st) {
  if (!ctx->timing) return;
  cudaEventRecord(ctx->ev[st][1], ctx->stream);
  ctx->pending[st] = true;
}

void apply_options(stq_context *ctx) {
  SweepTuning t;
  if (ctx->options[STQ_OPT_LANES_PER_ENTRY]) t.lanes = int(ctx->options[STQ_OPT_LANES_PER_ENTRY]);
  if (ctx->options[STQ_OPT_QUEUE_DEPTH]) t.queue = int(ctx->options[STQ_OPT_QUEUE_DEPTH]);
  if (ctx->options[STQ_OPT_BLOCK_SIZE]) t.block = int(ctx->options[STQ_OPT_BLOCK_SIZE]);
  ctx->tuning = t;
  ctx->radix_bits = ctx->options[STQ_OPT_RADIX_BITS] ? int(ctx->options[STQ_OPT_RADIX_BITS]) : 8;
  ctx->cell_scale = ctx->options[STQ_OPT_CELL_SCALE] ? float(ctx->options[STQ_OPT_CELL_SCALE]) : 4.f;
}

int read_scalars(stq_context *ctx) {
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_scalars, ctx->scalars.ptr, sizeof(DevScalars),
                                cudaMemcpyDeviceToHost, ctx->stream),
           "read back sweep counters");
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  collect_stages(ctx);
  if (ctx->h_scalars->flags & kFlagNaN)
    return fail(ctx, STQ_ERR_INVALID_INPUT, "a box bound is NaN");
  if (ctx->h_scalars->flags & kFlagBadIndex)
    return fail(ctx, STQ_ERR_INVALID_INPUT, "an edge or face vertex index is out of range");
  return STQ_OK;
}

constexpr int64_t kMaxBoxes = int64_t(INT32_MAX) - 4 * kSortedPad;

int run_sweep(stq_context *ctx, int64_t begin, int64_t end, stq_pair *pairs,
              long long capacity, bool count_mode) {
  SweepParams p;
  p.sx = ctx->scene.sx;
  p.syz = ctx->scene.syz;
  p.sv = ctx->scene.sv;
  p.begin = int32_t(begin);
  p.end = int32_t(end);
  // start positions per work grab: at least ~4 grabs per resident warp
  const int64_t span = end - begin;
  const int64_t want = int64_t(ctx->num_sms) * 64 * 4;
  int64_t chunk = ((span / want) + 31) / 32 * 32;
  p.chunk = int32_t(chunk < 32 ? 32 : (chunk > ctx->tuning.chunk ? ctx->tuning.chunk : chunk));
  p.pairs = pairs;
  p.capacity = capacity;
  DevScalars *ds = ctx->scalars.as<DevScalars>();
  p.count = &ds->count;
  p.work = &ds->work;
  p.box_counts = ctx->box_counts.as<int32_t>();
  p.scell = ctx->scene.scell;
  p.grid = ctx->scene.scell ? &ctx->prep.as<PrepInfo>()->grid : nullptr;
  reset_sweep_kernel<<<1, 1, 0, ctx->stream>>>(ds);
  STQ_CUDA(ctx, cudaGetLastError(), "reset sweep counters");
  stage_begin(ctx, count_mode ? kCountSweep : kSweep);
  STQ_CUDA(ctx, launch_sweep(ctx->stream, p, ctx->tuning, count_mode, ctx->num_sms),
           "launch sweep");
  stage_end(ctx, count_mode ? kCountSweep : kSweep);
  ctx->launches += (end > begin) ? 2 : 1;
  return STQ_OK;
}

}  // namespace

extern "C" {

int stq_abi_version(void) { return STQ_ABI_VERSION; }

const char *stq_status_string(int status) {
  switch (status) {
    case STQ_OK: return "ok";
    case STQ_OVERFLOW: return "overflow: partial result, resume from next_start";
    case STQ_ERR_INVALID_ARG: return "invalid argument";
    case STQ_ERR_INVALID_INPUT: return "invalid input (NaN bound or out-of-range index)";
    case STQ_ERR_CUDA: return "CUDA error";
    case STQ_ERR_NO_MEMORY: return "out of memory";
    case STQ_ERR_CAPACITY: return "pair buffer smaller than one start box's pairs";
    case STQ_ERR_TIMEOUT: return "bounded device wait expired";
    case STQ_ERR_NOT_PREPARED: return "no prepared scene";
    default: return "unknown status";
  }
}

int stq_context_create(int device, void *stream, stq_context **out) {
  if (!out) return STQ_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return STQ_ERR_INVALID_ARG;
  stq_context *ctx = new (std::nothrow) stq_context();
  if (!ctx) return STQ_ERR_NO_MEMORY;
  ctx->device = device;
  ctx->stream = static_cast<cudaStream_t>(stream);
  DeviceGuard g(device);
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMallocHost(&ctx->h_scalars, sizeof(DevScalars)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_prep, sizeof(PrepInfo)) != cudaSuccess ||
      ctx->scalars.ensure(sizeof(DevScalars)) != cudaSuccess ||
      ctx->stats.ensure(sizeof(SceneStats)) != cudaSuccess ||
      ctx->prep.ensure(sizeof(PrepInfo)) != cudaSuccess) {
    stq_context_destroy(ctx);
    return STQ_ERR_NO_MEMORY;
  }
  apply_options(ctx);
  *out = ctx;
  return STQ_OK;
}

void stq_context_destroy(stq_context *ctx) {
  if (!ctx) return;
  {
    DeviceGuard g(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    else cudaDeviceSynchronize();
    for (DevBuf *b : {&ctx->sx, &ctx->syz, &ctx->sv, &ctx->keys[0], &ctx->keys[1],
                      &ctx->vals[0], &ctx->vals[1], &ctx->sort_ws, &ctx->scalars,
                      &ctx->partials, &ctx->box_counts, &ctx->prefix_ws, &ctx->pair_keys[0],
                      &ctx->pair_keys[1], &ctx->e2e_boxes, &ctx->e2e_pairs})
      b->release();
    ctx->e2e_mesh.release();
    for (DevBuf *b : {&ctx->stats, &ctx->prep, &ctx->counts, &ctx->offsets, &ctx->scan_ws,
                      &ctx->keys64[0], &ctx->keys64[1], &ctx->scell})
      b->release();
    if (ctx->h_scalars) cudaFreeHost(ctx->h_scalars);
    if (ctx->h_prep) cudaFreeHost(ctx->h_prep);
    for (int st = 0; st < kStages; ++st)
      for (int k = 0; k < 2; ++k)
        if (ctx->ev[st][k]) cudaEventDestroy(ctx->ev[st][k]);
  }
  delete ctx;
}

int stq_context_set_stream(stq_context *ctx, void *stream) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return STQ_OK;
}

int stq_context_set_option(stq_context *ctx, int option, int64_t value) {
  if (!ctx || option < 1 || option > 6 || value < 0) return STQ_ERR_INVALID_ARG;
  auto pow2_in = [](int64_t v, int64_t lo, int64_t hi) {
    return v == 0 || (v >= lo && v <= hi && (v & (v - 1)) == 0);
  };
  switch (option) {
    case STQ_OPT_LANES_PER_ENTRY:
      if (!pow2_in(value, 1, 32)) return fail(ctx, STQ_ERR_INVALID_ARG, "lanes per entry: 1..32, power of 2");
      break;
    case STQ_OPT_QUEUE_DEPTH:
      if (!pow2_in(value, 32, 128)) return fail(ctx, STQ_ERR_INVALID_ARG, "queue depth: 32, 64 or 128");
      break;
    case STQ_OPT_BLOCK_SIZE:
      if (!pow2_in(value, 128, 512)) return fail(ctx, STQ_ERR_INVALID_ARG, "block size: 128, 256 or 512");
      break;
    case STQ_OPT_RADIX_BITS:
      if (value != 0 && value != 4 && value != 8) return fail(ctx, STQ_ERR_INVALID_ARG, "radix bits: 4 or 8");
      break;
    case STQ_OPT_CELLS:
      if (value > 2048) return fail(ctx, STQ_ERR_INVALID_ARG, "cells: 0 (auto), 1 (off) or a grid side <= 2048");
      break;
    case STQ_OPT_CELL_SCALE:
      if (value > 64) return fail(ctx, STQ_ERR_INVALID_ARG, "cell scale: 1..64");
      break;
    default:
      break;
  }
  ctx->options[option] = value;
  apply_options(ctx);
  return STQ_OK;
}

int64_t stq_context_get_option(const stq_context *ctx, int option) {
  if (!ctx || option < 1 || option > 6) return -1;
  switch (option) {
    case STQ_OPT_LANES_PER_ENTRY: return ctx->tuning.lanes;
    case STQ_OPT_QUEUE_DEPTH: return ctx->tuning.queue;
    case STQ_OPT_BLOCK_SIZE: return ctx->tuning.block;
    case STQ_OPT_RADIX_BITS: return ctx->radix_bits;
    case STQ_OPT_CELL_SCALE: return int64_t(ctx->cell_scale);
    default: return ctx->options[option];
  }
}

const char *stq_context_last_error(const stq_context *ctx) {
  return ctx ? ctx->error.c_str() : "null context";
}

int64_t stq_context_launch_count(const stq_context *ctx) { return ctx ? ctx->launches : -1; }

}  // extern "C"

namespace {

int enqueue_build(stq_context *ctx, const double *d_V0, const double *d_V1, int64_t nV,
                  const int32_t *d_E, int64_t nE, const int32_t *d_F, int64_t nF,
                  float inflation_radius, stq_aabb *d_boxes) {
  if (nV < 0 || nE < 0 || nF < 0 || nV + nE + nF > kMaxBoxes)
    return fail(ctx, STQ_ERR_INVALID_ARG, "box counts out of range");
  if ((nV > 0 && (!d_V0 || !d_V1)) || (nE > 0 && !d_E) || (nF > 0 && !d_F) ||
      (nV + nE + nF > 0 && !d_boxes))
    return fail(ctx, STQ_ERR_INVALID_ARG, "null buffer");
  const float r_up = ref_next_up(inflation_radius);
  DevScalars *ds = ctx->scalars.as<DevScalars>();
  init_scalars_kernel<<<1, 1, 0, ctx->stream>>>(ds, 0);
  STQ_CUDA(ctx, cudaGetLastError(), "init counters");
  stage_begin(ctx, kBuild);
  STQ_CUDA(ctx, launch_build_boxes(ctx->stream, d_V0, d_V1, nV, d_E, nE, d_F, nF, r_up,
                                   d_boxes, &ds->flags),
           "launch box build");
  stage_end(ctx, kBuild);
  ctx->launches += (nV + nE + nF > 0) ? 2 : 1;
  return STQ_OK;
}

}  // namespace

extern "C" {

int stq_build_boxes(stq_context *ctx, const double *d_V0, const double *d_V1, int64_t nV,
                    const int32_t *d_E, int64_t nE, const int32_t *d_F, int64_t nF,
                    float inflation_radius, stq_aabb *d_boxes) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  const int st = enqueue_build(ctx, d_V0, d_V1, nV, d_E, nE, d_F, nF, inflation_radius, d_boxes);
  if (st != STQ_OK) return st;
  return read_scalars(ctx);
}

int stq_select_axis(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int *axis_out) {
  if (!ctx || !axis_out || n < 0 || (n > 0 && !d_boxes)) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  const int nb = axis_partial_blocks(n);
  STQ_CUDA(ctx, ctx->partials.ensure(sizeof(double) * 6 * nb), "allocate axis partials");
  DevScalars *ds = ctx->scalars.as<DevScalars>();
  init_scalars_kernel<<<1, 1, 0, ctx->stream>>>(ds, 0);
  STQ_CUDA(ctx, launch_axis_select(ctx->stream, d_boxes, n, ctx->partials.as<double>(), nb,
                                   &ds->axis),
           "launch axis selection");
  ctx->launches += 3;
  int st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  *axis_out = ctx->h_scalars->axis;
  return STQ_OK;
}

int stq_prepare(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int axis) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n < 0 || n > kMaxBoxes) return fail(ctx, STQ_ERR_INVALID_ARG, "box count out of range");
  if (n > 0 && !d_boxes) return fail(ctx, STQ_ERR_INVALID_ARG, "null boxes");
  if (axis < STQ_AXIS_AUTO || axis > STQ_AXIS_Z) return fail(ctx, STQ_ERR_INVALID_ARG, "axis");
  DeviceGuard g(ctx->device);
  ctx->prepared = false;
  DevScalars *ds = ctx->scalars.as<DevScalars>();
  PrepInfo *pi = ctx->prep.as<PrepInfo>();
  init_scalars_kernel<<<1, 1, 0, ctx->stream>>>(ds, axis < 0 ? 0 : axis);
  STQ_CUDA(ctx, cudaGetLastError(), "init counters");
  ctx->launches += 1;
  // 1. statistics, sweep axis and cell grid (device), read back once
  STQ_CUDA(ctx, ctx->partials.ensure(stats_partials_bytes(n)), "allocate statistics");
  stage_begin(ctx, kAxis);
  STQ_CUDA(ctx, launch_scene_stats(ctx->stream, d_boxes, n, ctx->partials.as<double>(),
                                   ctx->stats.as<SceneStats>(), &ds->flags),
           "launch scene statistics");
  STQ_CUDA(ctx, launch_grid_policy(ctx->stream, ctx->partials.as<double>(), n,
                                   ctx->stats.as<SceneStats>(), axis,
                                   int(ctx->options[STQ_OPT_CELLS]), ctx->cell_scale, &pi->grid,
                                   &ds->axis),
           "launch grid policy");
  stage_end(ctx, kAxis);
  ctx->launches += 3;
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_prep, pi, sizeof(PrepInfo), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "read back grid");
  int st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  const GridParams grid = ctx->h_prep->grid;
  const size_t nn = size_t(n > 0 ? n : 1);

  if (grid.ncells <= 1) {
    // 2a. one cell: 32-bit keys, the sort of the reference's create_ds path
    const size_t slots = size_t(n) + 1 + kSortedPad;
    STQ_CUDA(ctx, ctx->sx.ensure(sizeof(float2) * slots), "allocate sorted scene");
    STQ_CUDA(ctx, ctx->syz.ensure(sizeof(float4) * slots), "allocate sorted scene");
    STQ_CUDA(ctx, ctx->sv.ensure(sizeof(int4) * slots), "allocate sorted scene");
    for (int b = 0; b < 2; ++b) {
      STQ_CUDA(ctx, ctx->keys[b].ensure(sizeof(uint32_t) * nn), "allocate sort keys");
      STQ_CUDA(ctx, ctx->vals[b].ensure(sizeof(uint32_t) * nn), "allocate sort values");
    }
    STQ_CUDA(ctx, ctx->sort_ws.ensure(radix_workspace_bytes(n, 4, ctx->radix_bits)),
             "allocate sort workspace");
    uint32_t *kb[2] = {ctx->keys[0].as<uint32_t>(), ctx->keys[1].as<uint32_t>()};
    uint32_t *vb[2] = {ctx->vals[0].as<uint32_t>(), ctx->vals[1].as<uint32_t>()};
    stage_begin(ctx, kKeys);
    STQ_CUDA(ctx, launch_prep_keys(ctx->stream, d_boxes, n, &ds->axis, kb[0], vb[0], &ds->flags),
             "launch key preparation");
    stage_end(ctx, kKeys);
    ctx->launches += n > 0 ? 1 : 0;
    int which = 0;
    stage_begin(ctx, kSort);
    STQ_CUDA(ctx, radix_sort_u32(ctx->stream, kb, vb, n, ctx->radix_bits, ctx->sort_ws.ptr,
                                 &which, &ctx->launches),
             "launch radix sort");
    stage_end(ctx, kSort);
    ctx->scene.sx = ctx->sx.as<float2>();
    ctx->scene.syz = ctx->syz.as<float4>();
    ctx->scene.sv = ctx->sv.as<int4>();
    ctx->scene.scell = nullptr;
    ctx->scene.length = n;
    stage_begin(ctx, kGather);
    STQ_CUDA(ctx, launch_gather(ctx->stream, d_boxes, vb[which], n, &ds->axis, ctx->scene),
             "launch gather");
    stage_end(ctx, kGather);
    ctx->launches += 1;
    ctx->n = n;
    ctx->prepared = true;
    return STQ_OK;
  }

  // 2b. cells: replicate each box into the cells it touches
  STQ_CUDA(ctx, ctx->counts.ensure(sizeof(uint32_t) * nn), "allocate replica counts");
  STQ_CUDA(ctx, ctx->offsets.ensure(sizeof(uint32_t) * nn), "allocate replica offsets");
  STQ_CUDA(ctx, ctx->scan_ws.ensure(scan_workspace_bytes(n)), "allocate scan workspace");
  stage_begin(ctx, kKeys);
  STQ_CUDA(ctx, launch_replica_count(ctx->stream, d_boxes, n, &pi->grid,
                                     ctx->counts.as<uint32_t>()),
           "launch replica count");
  STQ_CUDA(ctx, exclusive_scan_u32(ctx->stream, ctx->counts.as<uint32_t>(),
                                   ctx->offsets.as<uint32_t>(), n, ctx->scan_ws.ptr,
                                   &pi->replicas, &ctx->launches),
           "launch replica scan");
  ctx->launches += 1;
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_prep, pi, sizeof(PrepInfo), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "read back replica count");
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  const int64_t R = ctx->h_prep->replicas;
  if (R < n || R + grid.ncells + 1 + kSortedPad > int64_t(INT32_MAX))
    return fail(ctx, STQ_ERR_NO_MEMORY, "too many cell replicas for 32-bit positions");
  const size_t slots = size_t(R) + size_t(grid.ncells) + 1 + kSortedPad;
  STQ_CUDA(ctx, ctx->sx.ensure(sizeof(float2) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->syz.ensure(sizeof(float4) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->sv.ensure(sizeof(int4) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->scell.ensure(sizeof(int) * slots), "allocate sorted scene");
  for (int b = 0; b < 2; ++b) {
    STQ_CUDA(ctx, ctx->keys64[b].ensure(sizeof(unsigned long long) * size_t(R)), "allocate keys");
    STQ_CUDA(ctx, ctx->vals[b].ensure(sizeof(uint32_t) * size_t(R)), "allocate values");
  }
  STQ_CUDA(ctx, ctx->sort_ws.ensure(radix_workspace_bytes(R, 8, 8)), "allocate sort workspace");
  unsigned long long *kb[2] = {ctx->keys64[0].as<unsigned long long>(),
                               ctx->keys64[1].as<unsigned long long>()};
  uint32_t *vb[2] = {ctx->vals[0].as<uint32_t>(), ctx->vals[1].as<uint32_t>()};
  STQ_CUDA(ctx, launch_replica_emit(ctx->stream, d_boxes, n, &pi->grid,
                                    ctx->offsets.as<uint32_t>(), kb[0], vb[0]),
           "launch replica emit");
  stage_end(ctx, kKeys);
  ctx->launches += 1;
  int which = 0;
  stage_begin(ctx, kSort);
  STQ_CUDA(ctx, radix_sort_u64_vals(ctx->stream, kb, vb, R, 0, 32 + grid.cell_bits,
                                    ctx->sort_ws.ptr, &which, &ctx->launches),
           "launch radix sort");
  stage_end(ctx, kSort);
  ctx->scene.sx = ctx->sx.as<float2>();
  ctx->scene.syz = ctx->syz.as<float4>();
  ctx->scene.sv = ctx->sv.as<int4>();
  ctx->scene.scell = ctx->scell.as<int>();
  ctx->scene.length = R + grid.ncells;
  stage_begin(ctx, kGather);
  STQ_CUDA(ctx, launch_fill_sentinels(ctx->stream, ctx->scene.sx, int64_t(slots)),
           "launch sentinel fill");
  STQ_CUDA(ctx, launch_gather_cells(ctx->stream, d_boxes, kb[which], vb[which], R, &pi->grid,
                                    ctx->scene),
           "launch gather");
  stage_end(ctx, kGather);
  ctx->launches += 2;
  ctx->n = n;
  ctx->prepared = true;
  return STQ_OK;
}

int64_t stq_prepared_length(const stq_context *ctx) {
  return (ctx && ctx->prepared) ? ctx->scene.length : -1;
}

int stq_sweep_prepared(stq_context *ctx, int64_t start, int64_t max_start, stq_pair *d_pairs,
                       int64_t capacity, int64_t *count, int64_t *next_start, int64_t *total) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (!ctx->prepared) return fail(ctx, STQ_ERR_NOT_PREPARED, "call stq_prepare first");
  if (!count || !next_start || capacity < 0 || (capacity > 0 && !d_pairs))
    return fail(ctx, STQ_ERR_INVALID_ARG, "null output or negative capacity");
  const int64_t length = ctx->scene.length;
  if (start < 0 || start > length) return fail(ctx, STQ_ERR_INVALID_ARG, "start out of range");
  DeviceGuard g(ctx->device);
  const int64_t end = (max_start <= 0 || start + max_start > length) ? length : start + max_start;
  int st = run_sweep(ctx, start, end, d_pairs, capacity, false);
  if (st != STQ_OK) return st;
  st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  const int64_t found = int64_t(ctx->h_scalars->count);
  if (total) *total = found;
  if (found <= capacity) {
    *count = found;
    *next_start = end;
    return STQ_OK;
  }
  // Overflow: count pairs per start box, keep the longest prefix that fits,
  // and emit exactly that prefix again.
  const int64_t m = end - start;
  STQ_CUDA(ctx, ctx->box_counts.ensure(sizeof(int32_t) * size_t(m)), "allocate box counts");
  STQ_CUDA(ctx, ctx->prefix_ws.ensure(prefix_workspace_bytes(m)), "allocate prefix workspace");
  STQ_CUDA(ctx, cudaMemsetAsync(ctx->box_counts.ptr, 0, sizeof(int32_t) * size_t(m), ctx->stream),
           "clear box counts");
  st = run_sweep(ctx, start, end, nullptr, 0, true);
  if (st != STQ_OK) return st;
  STQ_CUDA(ctx, launch_prefix_select(ctx->stream, ctx->box_counts.as<int32_t>(), m, capacity,
                                     ctx->prefix_ws.ptr, ctx->scalars.as<DevScalars>(),
                                     &ctx->launches),
           "launch prefix selection");
  st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  const int64_t prefix = ctx->h_scalars->prefix;
  if (prefix <= 0) {
    *count = 0;
    *next_start = start;
    return fail(ctx, STQ_ERR_CAPACITY, "the first start box has more pairs than capacity");
  }
  st = run_sweep(ctx, start, start + prefix, d_pairs, capacity, false);
  if (st != STQ_OK) return st;
  st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  *count = int64_t(ctx->h_scalars->count);
  *next_start = start + prefix;
  if (*count > capacity) return fail(ctx, STQ_ERR_CUDA, "prefix re-sweep exceeded capacity");
  return STQ_OVERFLOW;
}

int stq_sweep(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int axis, int64_t start,
              int64_t max_start, stq_pair *d_pairs, int64_t capacity, int64_t *count,
              int64_t *next_start, int64_t *total) {
  int st = stq_prepare(ctx, d_boxes, n, axis);
  if (st != STQ_OK) return st;
  return stq_sweep_prepared(ctx, start, max_start, d_pairs, capacity, count, next_start, total);
}

int stq_sweep_host(stq_context *ctx, const stq_aabb *h_boxes, int64_t n, int axis,
                   stq_pair *h_pairs, int64_t capacity, int64_t *count, int64_t *total) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n < 0 || n > kMaxBoxes || (n > 0 && !h_boxes) || capacity < 0 ||
      (capacity > 0 && !h_pairs) || !count)
    return fail(ctx, STQ_ERR_INVALID_ARG, "invalid host sweep arguments");
  DeviceGuard g(ctx->device);
  STQ_CUDA(ctx, ctx->e2e_boxes.ensure(sizeof(stq_aabb) * size_t(n > 0 ? n : 1)),
           "allocate box staging");
  STQ_CUDA(ctx, ctx->e2e_pairs.ensure(sizeof(stq_pair) * size_t(capacity > 0 ? capacity : 1)),
           "allocate pair staging");
  if (n > 0)
    STQ_CUDA(ctx, cudaMemcpyAsync(ctx->e2e_boxes.ptr, h_boxes, sizeof(stq_aabb) * size_t(n),
                                  cudaMemcpyHostToDevice, ctx->stream),
             "copy boxes to device");
  int64_t next = 0;
  const int st = stq_sweep(ctx, ctx->e2e_boxes.as<stq_aabb>(), n, axis, 0, 0,
                           ctx->e2e_pairs.as<stq_pair>(), capacity, count, &next, total);
  if (st != STQ_OK && st != STQ_OVERFLOW) return st;
  if (*count > 0) {
    STQ_CUDA(ctx, cudaMemcpyAsync(h_pairs, ctx->e2e_pairs.ptr, sizeof(stq_pair) * size_t(*count),
                                  cudaMemcpyDeviceToHost, ctx->stream),
             "copy pairs to host");
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  }
  return st;
}

int stq_sort_pairs(stq_context *ctx, stq_pair *d_pairs, int64_t count) {
  if (!ctx || count < 0 || (count > 0 && !d_pairs)) return STQ_ERR_INVALID_ARG;
  if (count < 2) return STQ_OK;
  DeviceGuard g(ctx->device);
  for (int b = 0; b < 2; ++b)
    STQ_CUDA(ctx, ctx->pair_keys[b].ensure(sizeof(unsigned long long) * size_t(count)),
             "allocate pair keys");
  STQ_CUDA(ctx, ctx->sort_ws.ensure(radix_workspace_bytes(count, 8, 8)), "allocate sort workspace");
  unsigned long long *kb[2] = {ctx->pair_keys[0].as<unsigned long long>(),
                               ctx->pair_keys[1].as<unsigned long long>()};
  stage_begin(ctx, kPairSort);
  STQ_CUDA(ctx, launch_pairs_to_keys(ctx->stream, d_pairs, count, kb[0], true), "pairs to keys");
  int which = 0;
  STQ_CUDA(ctx, radix_sort_u64(ctx->stream, kb, count, 0, 64, ctx->sort_ws.ptr, &which,
                               &ctx->launches),
           "launch pair sort");
  STQ_CUDA(ctx, launch_pairs_to_keys(ctx->stream, d_pairs, count, kb[which], false), "keys to pairs");
  stage_end(ctx, kPairSort);
  ctx->launches += 2;
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  collect_stages(ctx);
  return STQ_OK;
}

int stq_broadphase_host(stq_context *ctx, const double *h_V0, const double *h_V1, int64_t nV,
                        const int32_t *h_E, int64_t nE, const int32_t *h_F, int64_t nF,
                        float inflation_radius, int axis, stq_pair *h_pairs, int64_t capacity,
                        int64_t *count, int64_t *total) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (nV < 0 || nE < 0 || nF < 0 || nV + nE + nF > kMaxBoxes || capacity < 0 || !count ||
      (capacity > 0 && !h_pairs) || (nV > 0 && (!h_V0 || !h_V1)) || (nE > 0 && !h_E) ||
      (nF > 0 && !h_F))
    return fail(ctx, STQ_ERR_INVALID_ARG, "invalid host mesh arguments");
  DeviceGuard g(ctx->device);
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  const size_t bv = sizeof(double) * 3 * size_t(nV), be = sizeof(int32_t) * 2 * size_t(nE),
               bf = sizeof(int32_t) * 3 * size_t(nF);
  const size_t oV1 = up16(bv), oE = oV1 + up16(bv), oF = oE + up16(be);
  STQ_CUDA(ctx, ctx->e2e_mesh.ensure(oF + up16(bf) + 16), "allocate mesh staging");
  const int64_t n = nV + nE + nF;
  STQ_CUDA(ctx, ctx->e2e_boxes.ensure(sizeof(stq_aabb) * size_t(n > 0 ? n : 1)),
           "allocate box staging");
  STQ_CUDA(ctx, ctx->e2e_pairs.ensure(sizeof(stq_pair) * size_t(capacity > 0 ? capacity : 1)),
           "allocate pair staging");
  char *base = ctx->e2e_mesh.as<char>();
  if (bv) {
    STQ_CUDA(ctx, cudaMemcpyAsync(base, h_V0, bv, cudaMemcpyHostToDevice, ctx->stream), "copy V0");
    STQ_CUDA(ctx, cudaMemcpyAsync(base + oV1, h_V1, bv, cudaMemcpyHostToDevice, ctx->stream), "copy V1");
  }
  if (be) STQ_CUDA(ctx, cudaMemcpyAsync(base + oE, h_E, be, cudaMemcpyHostToDevice, ctx->stream), "copy E");
  if (bf) STQ_CUDA(ctx, cudaMemcpyAsync(base + oF, h_F, bf, cudaMemcpyHostToDevice, ctx->stream), "copy F");
  int st = enqueue_build(ctx, reinterpret_cast<const double *>(base),
                         reinterpret_cast<const double *>(base + oV1), nV,
                         reinterpret_cast<const int32_t *>(base + oE), nE,
                         reinterpret_cast<const int32_t *>(base + oF), nF, inflation_radius,
                         ctx->e2e_boxes.as<stq_aabb>());
  if (st != STQ_OK) return st;
  st = stq_prepare(ctx, ctx->e2e_boxes.as<stq_aabb>(), n, axis);
  if (st != STQ_OK) return st;
  int64_t next = 0;
  st = stq_sweep_prepared(ctx, 0, 0, ctx->e2e_pairs.as<stq_pair>(), capacity, count, &next, total);
  if (st != STQ_OK && st != STQ_OVERFLOW) return st;
  if (*count > 0) {
    STQ_CUDA(ctx, cudaMemcpyAsync(h_pairs, ctx->e2e_pairs.ptr, sizeof(stq_pair) * size_t(*count),
                                  cudaMemcpyDeviceToHost, ctx->stream),
             "copy pairs to host");
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  }
  return st;
}

int stq_context_enable_timing(stq_context *ctx, int enable) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  if (enable && !ctx->ev[0][0]) {
    for (int st = 0; st < kStages; ++st)
      for (int k = 0; k < 2; ++k)
        STQ_CUDA(ctx, cudaEventCreate(&ctx->ev[st][k]), "create timing event");
  }
  if (!enable) collect_stages(ctx);
  ctx->timing = enable != 0;
  for (int st = 0; st < kStages; ++st) ctx->stage_ms[st] = 0.0, ctx->stage_calls[st] = 0;
  return STQ_OK;
}

int stq_context_stage_times(stq_context *ctx, double *ms, int64_t *calls, int max_stages) {
  if (!ctx || max_stages < 0) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  collect_stages(ctx);
  for (int st = 0; st < kStages && st < max_stages; ++st) {
    if (ms) ms[st] = ctx->stage_ms[st];
    if (calls) calls[st] = ctx->stage_calls[st];
  }
  return kStages;
}

const char *stq_stage_name(int stage) {
  return (stage >= 0 && stage < kStages) ? kStageNames[stage] : "unknown";
}

int stq_brute_force(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, stq_pair *d_pairs,
                    int64_t capacity, int64_t *count) {
  if (!ctx || !count || n < 0 || n > kMaxBoxes || (n > 0 && !d_boxes) || capacity < 0 ||
      (capacity > 0 && !d_pairs))
    return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  DevScalars *ds = ctx->scalars.as<DevScalars>();
  init_scalars_kernel<<<1, 1, 0, ctx->stream>>>(ds, 0);
  STQ_CUDA(ctx, launch_brute_force(ctx->stream, d_boxes, n, d_pairs, capacity, &ds->count),
           "launch brute force");
  ctx->launches += 2;
  const int st = read_scalars(ctx);
  if (st != STQ_OK) return st;
  *count = int64_t(ctx->h_scalars->count);
  return *count > capacity ? STQ_OVERFLOW : STQ_OK;
}

}  // extern "C"
