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
#include <vector>

#include <functional>

#include "context.h"

namespace stq {
namespace ctxops {

DeviceGuard::DeviceGuard(int dev) {
  if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) changed = cudaSetDevice(dev) == cudaSuccess;
}
DeviceGuard::~DeviceGuard() {
  if (changed) cudaSetDevice(prev);
}

int fail(stq_context *ctx, int status, const char *what, cudaError_t e) {
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
  if (!ctx->timing || ctx->capturing) return;
  collect_stage(ctx, st);
  cudaEventRecord(ctx->ev[st][0], ctx->stream);
}

void stage_end(stq_context *ctx, int st) {
  if (!ctx->timing || ctx->capturing) return;
  cudaEventRecord(ctx->ev[st][1], ctx->stream);
  ctx->pending[st] = true;
}

void apply_options(stq_context *ctx) {
  SweepTuning t;
  if (ctx->options[STQ_OPT_LANES_PER_ENTRY]) t.lanes = int(ctx->options[STQ_OPT_LANES_PER_ENTRY]);
  if (ctx->options[STQ_OPT_QUEUE_DEPTH]) t.queue = int(ctx->options[STQ_OPT_QUEUE_DEPTH]);
  if (ctx->options[STQ_OPT_BLOCK_SIZE]) t.block = int(ctx->options[STQ_OPT_BLOCK_SIZE]);
  if (ctx->options[STQ_OPT_CANDIDATES_PER_LANE]) t.per_lane = int(ctx->options[STQ_OPT_CANDIDATES_PER_LANE]);
  if (ctx->options[STQ_OPT_RUN_CAP]) t.run_cap = int(ctx->options[STQ_OPT_RUN_CAP]);
  if (ctx->options[STQ_OPT_SWEEP_SHAPE]) t.shape = int(ctx->options[STQ_OPT_SWEEP_SHAPE]);
  ctx->tuning = t;
  ctx->cell_scale = ctx->options[STQ_OPT_CELL_SCALE] ? float(ctx->options[STQ_OPT_CELL_SCALE]) : 2.f;
  ctx->budget = ctx->options[STQ_OPT_REPLICA_BUDGET] ? int(ctx->options[STQ_OPT_REPLICA_BUDGET]) : 4;
}

BatchHeader *dev_hdr(stq_context *ctx) {
  return reinterpret_cast<BatchHeader *>(ctx->in_dev.as<char>() + ctx->layout.hdr);
}
int read_header(stq_context *ctx, const BatchHeader *src) {
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_hdr, src ? src : dev_hdr(ctx), sizeof(BatchHeader),
                                cudaMemcpyDeviceToHost, ctx->stream),
           "read back batch header");
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  collect_stages(ctx);
  const int f = ctx->h_hdr->flags;
  if (f & kFlagNaN) return fail(ctx, STQ_ERR_INVALID_INPUT, "a box bound is NaN");
  if (f & kFlagBadIndex)
    return fail(ctx, STQ_ERR_INVALID_INPUT, "an edge or face vertex index is out of range");
  if (f & kFlagReplicaOverflow)
    return fail(ctx, STQ_ERR_NO_MEMORY, "cell replicas exceed the replica buffers");
  return STQ_OK;
}

int64_t tiles_for(const int64_t *box_off, int S) {
  int64_t t = 0;
  for (int s = 0; s < S; ++s) t += (box_off[s + 1] - box_off[s] + kTileBoxes - 1) / kTileBoxes;
  return t;
}

// Grows the staging block (pinned host mirror and device copy).
int ensure_staging(stq_context *ctx, int scene_cap, int tile_cap) {
  if (scene_cap <= ctx->scene_cap && tile_cap <= ctx->tile_cap && ctx->in_host) return STQ_OK;
  scene_cap = std::max(scene_cap, ctx->scene_cap);
  tile_cap = std::max(tile_cap, ctx->tile_cap);
  const Staging lay = Staging::make(scene_cap, tile_cap);
  if (ctx->in_host) {
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
    cudaFreeHost(ctx->in_host);
    ctx->in_host = nullptr;
  }
  STQ_CUDA(ctx, cudaMallocHost(&ctx->in_host, lay.total), "allocate pinned staging");
  std::memset(ctx->in_host, 0, lay.total);
  ctx->in_host_bytes = lay.total;
  STQ_CUDA(ctx, ctx->in_dev.ensure(lay.total), "allocate staging");
  STQ_CUDA(ctx, ctx->scenes.ensure(sizeof(SceneRecord) * size_t(scene_cap)), "allocate scenes");
  STQ_CUDA(ctx, ctx->cell_base.ensure(sizeof(unsigned) * size_t(scene_cap + 1)), "allocate cell bases");
  STQ_CUDA(ctx, ctx->scene_pairs.ensure(sizeof(unsigned long long) * size_t(scene_cap)),
           "allocate scene pair counters");
  if (scene_cap > ctx->h_scene_pairs_cap) {
    if (ctx->h_scene_pairs) cudaFreeHost(ctx->h_scene_pairs);
    ctx->h_scene_pairs = nullptr;
    STQ_CUDA(ctx, cudaMallocHost(&ctx->h_scene_pairs, sizeof(unsigned long long) * size_t(scene_cap)),
             "allocate pinned scene counters");
    ctx->h_scene_pairs_cap = scene_cap;
  }
  ctx->layout = lay;
  ctx->scene_cap = scene_cap;
  ctx->tile_cap = tile_cap;
  return STQ_OK;
}

// Writes the header, offsets, options and tiles into the pinned mirror.
void fill_staging(stq_context *ctx, const int64_t *box_off, int S, const int *axes, int axis,
                  const int64_t *voff, const int64_t *eoff, const int64_t *foff) {
  const Staging &L = ctx->layout;
  BatchHeader *h = host_at<BatchHeader>(ctx, L.hdr);
  std::memset(h, 0, sizeof(BatchHeader));
  h->n_boxes = box_off[S];
  h->box_count = uint32_t(box_off[S]);
  h->n_scenes = S;
  h->budget = ctx->budget;
  long long *bo = host_at<long long>(ctx, L.box_off);
  for (int s = 0; s <= S; ++s) bo[s] = box_off[s];
  if (voff) {
    long long *v = host_at<long long>(ctx, L.voff), *e = host_at<long long>(ctx, L.eoff),
              *f = host_at<long long>(ctx, L.foff);
    for (int s = 0; s <= S; ++s) v[s] = voff[s], e[s] = eoff[s], f[s] = foff[s];
  }
  SceneInput *in = host_at<SceneInput>(ctx, L.inputs);
  for (int s = 0; s < S; ++s) {
    in[s].axis_mode = axes ? axes[s] : axis;
    in[s].cells_opt = int(ctx->options[STQ_OPT_CELLS]);
    in[s].cell_scale = ctx->cell_scale;
    in[s].pad = 0;
  }
  TileRec *tr = host_at<TileRec>(ctx, L.tiles);
  int t = 0;
  for (int s = 0; s < S; ++s)
    for (int64_t b = box_off[s]; b < box_off[s + 1]; b += kTileBoxes) {
      tr[t].begin = b;
      tr[t].count = int(std::min<int64_t>(kTileBoxes, box_off[s + 1] - b));
      tr[t].scene = s;
      ++t;
    }
  h->n_tiles = t;
}

int upload_staging(stq_context *ctx) {
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->in_dev.ptr, ctx->in_host, ctx->layout.total,
                                cudaMemcpyHostToDevice, ctx->stream),
           "upload batch inputs");
  return STQ_OK;
}

BatchBuffers batch_buffers(stq_context *ctx, const stq_aabb *boxes) {
  BatchBuffers b;
  b.boxes = boxes;
  b.box_off = dev_at<long long>(ctx, ctx->layout.box_off);
  b.tiles = dev_at<TileRec>(ctx, ctx->layout.tiles);
  b.tile_cap = ctx->tile_cap;
  b.inputs = dev_at<SceneInput>(ctx, ctx->layout.inputs);
  b.scene_pairs = ctx->scene_pairs.as<unsigned long long>();
  b.scenes = ctx->scenes.as<SceneRecord>();
  b.cell_base = ctx->cell_base.as<unsigned>();
  b.hdr = dev_hdr(ctx);
  b.counts = ctx->counts.as<uint32_t>();
  b.offsets = ctx->offsets.as<uint32_t>();
  b.box_cells = ctx->box_cells.as<uint2>();
  b.keys = ctx->keys64[0].as<unsigned long long>();
  b.vals = ctx->vals[0].as<uint32_t>();
  b.box_keys = ctx->bkeys[0].as<uint32_t>();
  b.box_vals = ctx->bvals[0].as<uint32_t>();
  b.box_keys2 = ctx->bkeys[1].as<uint32_t>();
  b.box_vals2 = ctx->bvals[1].as<uint32_t>();
  b.order = ctx->bvals[ctx->order_buf].as<uint32_t>();
  b.sorted_keys = ctx->bkeys[ctx->order_buf].as<uint32_t>();
  b.seg_scan = ctx->seg_scan.as<uint32_t>();
  b.seg_cap = ctx->seg_cap;
  b.box_cap = ctx->box_cap;
  b.rep_cap = ctx->rep_cap;
  b.scene_cap = ctx->scene_cap;
  return b;
}

int ensure_box_buffers(stq_context *ctx, int64_t box_cap) {
  const size_t n = size_t(std::max<int64_t>(box_cap, 1));
  STQ_CUDA(ctx, ctx->counts.ensure(sizeof(uint32_t) * n), "allocate replica counts");
  STQ_CUDA(ctx, ctx->offsets.ensure(sizeof(uint32_t) * n), "allocate replica offsets");
  STQ_CUDA(ctx, ctx->box_cells.ensure(sizeof(uint2) * n), "allocate box cell ranges");
  STQ_CUDA(ctx, ctx->scan_ws.ensure(scan_workspace_bytes(int64_t(n))), "allocate scan workspace");
  for (int b = 0; b < 2; ++b) {
    STQ_CUDA(ctx, ctx->bkeys[b].ensure(sizeof(uint32_t) * n), "allocate box keys");
    STQ_CUDA(ctx, ctx->bvals[b].ensure(sizeof(uint32_t) * n), "allocate box order");
  }
  STQ_CUDA(ctx, ctx->sort_ws.ensure(std::max(radix_workspace_bytes(int64_t(n), 4, 8),
                                              radix_workspace_bytes(int64_t(n), 4, 4))),
           "allocate sort workspace");
  ctx->box_cap = int64_t(n);
  return STQ_OK;
}

int ensure_replica_buffers(stq_context *ctx, int64_t rep_cap, int64_t cells_cap) {
  const size_t r = size_t(std::max<int64_t>(rep_cap, 1));
  for (int b = 0; b < 2; ++b) {
    STQ_CUDA(ctx, ctx->keys64[b].ensure(sizeof(unsigned long long) * r), "allocate keys");
    STQ_CUDA(ctx, ctx->vals[b].ensure(sizeof(uint32_t) * r), "allocate values");
  }
  STQ_CUDA(ctx, ctx->sort_ws.ensure(std::max(radix_workspace_bytes(int64_t(r), 8, 8),
                                              radix_workspace_bytes(int64_t(r), 8, 4))),
           "allocate sort workspace");
  // three lists (vertices, edges, faces) per cell, each followed by a sentinel
  const int64_t segs = std::max<int64_t>(3 * cells_cap, ctx->seg_cap);
  STQ_CUDA(ctx, ctx->seg_scan.ensure(sizeof(uint32_t) * size_t(segs + 1)), "allocate segment offsets");
  ctx->seg_cap = segs;
  const size_t slots = r + size_t(segs) + 1 + kSortedPad;
  STQ_CUDA(ctx, ctx->xmin.ensure(sizeof(float) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->xmax.ensure(sizeof(float) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->syz.ensure(sizeof(float4) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->sv.ensure(sizeof(int4) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->sflag.ensure(sizeof(int) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->sfloor.ensure(sizeof(float2) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->partner.ensure(sizeof(int) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->run_end.ensure(sizeof(int) * slots), "allocate sorted scene");
  STQ_CUDA(ctx, ctx->cell_floor.ensure(sizeof(float2) * size_t(segs / 3 + 1)), "allocate cell bounds");
  STQ_CUDA(ctx, ctx->long_list.ensure(sizeof(int2) * slots), "allocate long-run list");
  ctx->rep_cap = int64_t(r);
  ctx->slot_cap = int64_t(slots);
  return STQ_OK;
}

int bits_for(int64_t v) {
  int b = 0;
  while ((int64_t(1) << b) < v) ++b;
  return b;
}

int enqueue_prepare_front(stq_context *ctx, const BatchBuffers &b, int64_t n_boxes) {
  stage_begin(ctx, kAxis);
  STQ_CUDA(ctx, launch_batch_stats(ctx->stream, b), "launch batch statistics");
  STQ_CUDA(ctx, launch_batch_policy(ctx->stream, b), "launch batch policy");
  stage_end(ctx, kAxis);
  // boxes in sweep-axis order: the emit then writes every list in key order
  stage_begin(ctx, kSort);
  STQ_CUDA(ctx, launch_batch_box_keys(ctx->stream, b), "launch box keys");
  uint32_t *kb[2] = {ctx->bkeys[0].as<uint32_t>(), ctx->bkeys[1].as<uint32_t>()};
  uint32_t *vb[2] = {ctx->bvals[0].as<uint32_t>(), ctx->bvals[1].as<uint32_t>()};
  const int rbits = ctx->options[STQ_OPT_RADIX_BITS] == 4 ? 4 : 8;
  const int64_t n = n_boxes >= 0 ? n_boxes : ctx->box_cap;
  STQ_CUDA(ctx, radix_sort_u32(ctx->stream, kb, vb, n, rbits, ctx->sort_ws.ptr, &ctx->order_buf, &ctx->launches,
                               n_boxes >= 0 ? nullptr : &b.hdr->box_count),
           "launch box sort");
  stage_end(ctx, kSort);
  BatchBuffers bs = b;
  bs.order = vb[ctx->order_buf];
  bs.sorted_keys = kb[ctx->order_buf];
  stage_begin(ctx, kKeys);
  STQ_CUDA(ctx, launch_batch_counts(ctx->stream, bs, n), "launch replica counts");
  STQ_CUDA(ctx, exclusive_scan_u32(ctx->stream, b.counts, b.offsets, ctx->box_cap, ctx->scan_ws.ptr,
                                   &b.hdr->replicas, &ctx->launches),
           "launch replica scan");
  ctx->launches += 6;  // reset, statistics, policy, box keys, choose, counts
  return STQ_OK;
}

int enqueue_prepare_back(stq_context *ctx, const BatchBuffers &b, int seg_bits, int64_t n_boxes,
                         int64_t replicas) {
  BatchBuffers bs = b;
  bs.order = ctx->bvals[ctx->order_buf].as<uint32_t>();
  bs.sorted_keys = ctx->bkeys[ctx->order_buf].as<uint32_t>();
  STQ_CUDA(ctx, launch_batch_emit(ctx->stream, bs, n_boxes >= 0 ? n_boxes : ctx->box_cap, ctx->num_sms),
           "launch replica emit");
  stage_end(ctx, kKeys);
  // the replicas arrive in sweep-axis order: a stable sort by list id alone
  // (the key's high half) leaves every list sorted by its minima
  unsigned long long *kb[2] = {ctx->keys64[0].as<unsigned long long>(),
                               ctx->keys64[1].as<unsigned long long>()};
  uint32_t *vb[2] = {ctx->vals[0].as<uint32_t>(), ctx->vals[1].as<uint32_t>()};
  int which = 0;
  stage_begin(ctx, kSort);
  const int rbits = ctx->options[STQ_OPT_RADIX_BITS] == 4 ? 4 : 8;
  const int64_t r = replicas >= 0 ? replicas : ctx->rep_cap;
  // seg_bits covers the capacity; passes above the actual list count copy through
  STQ_CUDA(ctx, radix_sort_u64_vals(ctx->stream, kb, vb, r, 32, 32 + std::max(seg_bits, 1), ctx->sort_ws.ptr,
                                    &which, &ctx->launches, &b.hdr->replicas, rbits, &b.hdr->lists),
           "launch list sort");
  stage_end(ctx, kSort);
  ctx->scene.xmin = ctx->xmin.as<float>();
  ctx->scene.xmax = ctx->xmax.as<float>();
  ctx->scene.syz = ctx->syz.as<float4>();
  ctx->scene.sv = ctx->sv.as<int4>();
  ctx->scene.sflag = ctx->sflag.as<int>();
  ctx->scene.sfloor = ctx->sfloor.as<float2>();
  ctx->scene.partner = ctx->partner.as<int>();
  ctx->scene.run_end = ctx->run_end.as<int>();
  stage_begin(ctx, kGather);
  STQ_CUDA(ctx, launch_list_offsets(ctx->stream, kb[which], b.hdr, b.seg_scan, b.seg_cap, ctx->scene, ctx->slot_cap),
           "launch list offsets");
  STQ_CUDA(ctx, launch_gather_cells(ctx->stream, b.boxes, kb[which], vb[which], b.hdr, r, b.cell_base, b.scenes,
                                    b.seg_scan, ctx->cell_floor.as<float2>(), ctx->seg_cap / 3,
                                    ctx->scene),
           "launch gather");
  stage_end(ctx, kGather);
  ctx->launches += 4;
  return STQ_OK;
}

// Prepares a batch with exact buffer sizes (one synchronisation after the
// replica count). Leaves the batch header read back in ctx->h_hdr.
int prepare_exact(stq_context *ctx, const stq_aabb *d_boxes, const int64_t *box_off, int S,
                  const int *axes, int axis) {
  ctx->prepared = false;
  const int64_t N = box_off[S];
  const int64_t T = tiles_for(box_off, S);
  STQ_TRY(ensure_staging(ctx, std::max(S, 1), int(std::max<int64_t>(T, 1))));
  STQ_TRY(ensure_box_buffers(ctx, N));
  fill_staging(ctx, box_off, S, axes, axis, nullptr, nullptr, nullptr);
  STQ_TRY(upload_staging(ctx));
  BatchBuffers b = batch_buffers(ctx, d_boxes);
  STQ_TRY(enqueue_prepare_front(ctx, b, N));
  STQ_TRY(read_header(ctx));
  const int64_t R = ctx->h_hdr->replicas, cells = ctx->h_hdr->cells;
  if (R + 3 * cells + 1 + kSortedPad > int64_t(INT32_MAX))
    return fail(ctx, STQ_ERR_NO_MEMORY, "too many cell replicas for 32-bit positions");
  STQ_TRY(ensure_replica_buffers(ctx, std::max(R, ctx->rep_cap), cells));
  b = batch_buffers(ctx, d_boxes);
  STQ_TRY(enqueue_prepare_back(ctx, b, bits_for(3 * cells), N, R));
  ctx->n_scenes = S;
  ctx->n_boxes = N;
  ctx->length = R > 0 ? R + 3 * cells - 1 : 0;
  ctx->scene.length = ctx->length;
  ctx->prepared = true;
  return STQ_OK;
}

int run_sweep(stq_context *ctx, int64_t begin, int64_t end, stq_pair *pairs,
              long long capacity, bool count_mode, bool timed, const SweepCursors *cursors,
              cudaStream_t stream) {
  BatchHeader *hdr = dev_hdr(ctx);
  cudaStream_t s = cursors && stream ? stream : ctx->stream;
  SweepParams p;
  p.xmin = ctx->scene.xmin;
  p.xmax = ctx->scene.xmax;
  p.syz = ctx->scene.syz;
  p.sv = ctx->scene.sv;
  p.begin = int32_t(begin);
  p.end = int32_t(std::min<int64_t>(end, INT32_MAX));
  // start positions per work grab: at least ~4 grabs per resident warp
  const int64_t span = std::min<int64_t>(end, ctx->slot_cap) - begin;
  const int64_t want = int64_t(ctx->num_sms) * 64 * 4;
  const int64_t chunk = ((std::max<int64_t>(span, 0) / want) + 31) / 32 * 32;
  p.chunk = int32_t(chunk < 32 ? 32 : (chunk > ctx->tuning.chunk ? ctx->tuning.chunk : chunk));
  p.pairs = pairs;
  p.capacity = capacity;
  p.count = &hdr->pairs;
  p.work = &hdr->work;
  p.box_counts = ctx->box_counts.as<int32_t>();
  p.sflag = ctx->scene.sflag;
  p.sfloor = ctx->scene.sfloor;
  p.partner = ctx->scene.partner;
  p.run_end = ctx->scene.run_end;
  p.scene_pairs = ctx->scene_pairs.as<unsigned long long>();
  p.hdr = hdr;
  p.stats = &hdr->candidates;
  p.typed = 1;
  p.run_cap = ctx->tuning.run_cap;
  p.long_list = ctx->long_list.as<int2>();
  p.long_items = &hdr->long_items;
  p.long_work = &hdr->long_work;
  if (cursors) {
    p.count = cursors->count;
    p.work = cursors->work;
    p.long_list = cursors->long_list;
    p.long_items = cursors->long_items;
    p.long_work = cursors->long_work;
  } else {
    STQ_CUDA(ctx, launch_reset_sweep(ctx->stream, hdr, p.scene_pairs, ctx->scene_cap), "reset sweep");
    ctx->launches += 1;
  }
  if (timed) stage_begin(ctx, count_mode ? kCountSweep : kSweep);
  STQ_CUDA(ctx, launch_sweep(s, p, ctx->tuning, count_mode, ctx->num_sms), "launch sweep");
  if (timed) stage_end(ctx, count_mode ? kCountSweep : kSweep);
  // the sweep, and the warp pass over handed-over runs when there is a run cap
  ctx->launches += p.end > p.begin ? (p.run_cap ? 2 : 1) : 0;
  return STQ_OK;
}

}  // namespace ctxops
}  // namespace stq

using namespace stq::ctxops;

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
  apply_options(ctx);
  if (cudaMallocHost(&ctx->h_hdr, sizeof(BatchHeader)) != cudaSuccess ||
      ctx->aux.ensure(sizeof(BatchHeader)) != cudaSuccess || ensure_staging(ctx, 1, 1) != STQ_OK) {
    stq_context_destroy(ctx);
    return STQ_ERR_NO_MEMORY;
  }
  *out = ctx;
  return STQ_OK;
}

void stq_context_destroy(stq_context *ctx) {
  if (!ctx) return;
  {
    DeviceGuard g(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    else cudaDeviceSynchronize();
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    if (ctx->graph_stream) cudaStreamDestroy(ctx->graph_stream);
    if (ctx->graph_event) cudaEventDestroy(ctx->graph_event);
    if (ctx->owns_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    for (DevBuf *b : {&ctx->points, &ctx->in_dev, &ctx->scenes, &ctx->cell_base, &ctx->scene_pairs, &ctx->counts, &ctx->box_cells,
                      &ctx->offsets, &ctx->scan_ws, &ctx->keys64[0], &ctx->keys64[1], &ctx->vals[0],
                      &ctx->vals[1], &ctx->sort_ws, &ctx->xmin, &ctx->xmax, &ctx->syz, &ctx->sv, &ctx->sflag, &ctx->sfloor, &ctx->cell_floor, &ctx->partner, &ctx->run_end, &ctx->long_list,
                      &ctx->seg_scan, &ctx->bkeys[0], &ctx->bkeys[1],
                      &ctx->bvals[0], &ctx->bvals[1],
                      &ctx->box_counts, &ctx->prefix_ws, &ctx->pair_keys[0], &ctx->pair_keys[1],
                      &ctx->batch_boxes, &ctx->e2e_boxes, &ctx->e2e_pairs, &ctx->e2e_mesh, &ctx->aux,
                      &ctx->window_pairs, &ctx->window_long_list, &ctx->window_cursors})
      b->release();
    if (ctx->in_host) cudaFreeHost(ctx->in_host);
    if (ctx->h_hdr) cudaFreeHost(ctx->h_hdr);
    if (ctx->h_scene_pairs) cudaFreeHost(ctx->h_scene_pairs);
    if (ctx->copy_stream) {
      cudaStreamSynchronize(ctx->copy_stream);
      cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->window_stream) {
      cudaStreamSynchronize(ctx->window_stream);
      cudaStreamDestroy(ctx->window_stream);
    }
    if (ctx->h_window_pairs) cudaFreeHost(ctx->h_window_pairs);
    if (ctx->window_start) cudaEventDestroy(ctx->window_start);
    for (cudaEvent_t e : ctx->window_done)
      if (e) cudaEventDestroy(e);
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
  if (!ctx || option < 1 || option > 13 || value < 0) return STQ_ERR_INVALID_ARG;
  auto pow2_in = [](int64_t v, int64_t lo, int64_t hi) {
    return v == 0 || (v >= lo && v <= hi && (v & (v - 1)) == 0);
  };
  switch (option) {
    case STQ_OPT_LANES_PER_ENTRY:
      if (!pow2_in(value, 1, 32)) return fail(ctx, STQ_ERR_INVALID_ARG, "lanes per entry: 1..32, power of 2");
      break;
    case STQ_OPT_QUEUE_DEPTH:
      if (!pow2_in(value, 16, 128)) return fail(ctx, STQ_ERR_INVALID_ARG, "queue depth: 16, 32, 64 or 128");
      break;
    case STQ_OPT_BLOCK_SIZE:
      if (!pow2_in(value, 128, 512)) return fail(ctx, STQ_ERR_INVALID_ARG, "block size: 128, 256 or 512");
      break;
    case STQ_OPT_RADIX_BITS:
      if (value != 0 && value != 4 && value != 8) return fail(ctx, STQ_ERR_INVALID_ARG, "radix bits: 4 or 8");
      break;
    case STQ_OPT_CELLS:
      if (value > kMaxGridSide)
        return fail(ctx, STQ_ERR_INVALID_ARG, "cells: 0 (auto), 1 (off) or a grid side <= 2048");
      break;
    case STQ_OPT_CELL_SCALE:
      if (value > 64) return fail(ctx, STQ_ERR_INVALID_ARG, "cell scale: 1..64");
      break;
    case STQ_OPT_REPLICA_BUDGET:
      if (value > 64) return fail(ctx, STQ_ERR_INVALID_ARG, "replica budget: 1..64");
      break;
    case STQ_OPT_GRAPH:
      if (value > 2) return fail(ctx, STQ_ERR_INVALID_ARG, "graph: 0 (default), 1 on, 2 off");
      break;
    case STQ_OPT_HOST_OVERLAP:
      if (value > 2) return fail(ctx, STQ_ERR_INVALID_ARG, "host overlap: 0 (default), 1 on, 2 off");
      break;
    case STQ_OPT_CANDIDATES_PER_LANE:
      if (!pow2_in(value, 1, 8)) return fail(ctx, STQ_ERR_INVALID_ARG, "candidates per lane: 1, 2, 4 or 8");
      break;
    case STQ_OPT_RUN_CAP:
      if (value > (int64_t(1) << 20)) return fail(ctx, STQ_ERR_INVALID_ARG, "run cap: 1..2^20");
      break;
    case STQ_OPT_HOST_WINDOWS:
      if (value == 1 || value > stq_context::kCopyWindows)
        return fail(ctx, STQ_ERR_INVALID_ARG, "host windows: 2..32");
      break;
    case STQ_OPT_SWEEP_SHAPE:
      if (value > 2) return fail(ctx, STQ_ERR_INVALID_ARG, "sweep shape: 1 queue, 2 flat");
      break;
    default:
      break;
  }
  ctx->options[option] = value;
  apply_options(ctx);
  return STQ_OK;
}

int64_t stq_context_get_option(const stq_context *ctx, int option) {
  if (!ctx || option < 1 || option > 13) return -1;
  switch (option) {
    case STQ_OPT_LANES_PER_ENTRY: return ctx->tuning.lanes;
    case STQ_OPT_QUEUE_DEPTH: return ctx->tuning.queue;
    case STQ_OPT_BLOCK_SIZE: return ctx->tuning.block;
    case STQ_OPT_RADIX_BITS: return ctx->options[STQ_OPT_RADIX_BITS] == 4 ? 4 : 8;
    case STQ_OPT_CELL_SCALE: return int64_t(ctx->cell_scale);
    case STQ_OPT_REPLICA_BUDGET: return ctx->budget;
    case STQ_OPT_GRAPH: return ctx->options[STQ_OPT_GRAPH] == 2 ? 2 : 1;
    case STQ_OPT_HOST_OVERLAP: return ctx->options[STQ_OPT_HOST_OVERLAP] == 2 ? 2 : 1;
    case STQ_OPT_CANDIDATES_PER_LANE: return ctx->tuning.per_lane;
    case STQ_OPT_RUN_CAP: return ctx->tuning.run_cap;
    case STQ_OPT_HOST_WINDOWS: return ctx->options[STQ_OPT_HOST_WINDOWS] ? ctx->options[STQ_OPT_HOST_WINDOWS] : 16;
    case STQ_OPT_SWEEP_SHAPE: return ctx->tuning.shape;
    default: return ctx->options[option];
  }
}

const char *stq_context_last_error(const stq_context *ctx) {
  return ctx ? ctx->error.c_str() : "null context";
}

int64_t stq_context_launch_count(const stq_context *ctx) { return ctx ? ctx->launches : -1; }

int64_t stq_context_candidates(const stq_context *ctx) {
  return ctx ? int64_t(ctx->h_hdr->candidates) : -1;
}

int stq_context_list_stats(stq_context *ctx, int64_t *out) {
  if (!ctx || !out) return STQ_ERR_INVALID_ARG;
  if (!ctx->prepared) return fail(ctx, STQ_ERR_NOT_PREPARED, "nothing prepared");
  DeviceGuard g(ctx->device);
  STQ_TRY(read_header(ctx));
  const BatchHeader &h = *ctx->h_hdr;
  out[0] = 3 * int64_t(h.cells);
  out[1] = int64_t(h.replicas);
  out[2] = int64_t(h.max_list);
  return STQ_OK;
}

int stq_build_boxes(stq_context *ctx, const double *d_V0, const double *d_V1, int64_t nV,
                    const int32_t *d_E, int64_t nE, const int32_t *d_F, int64_t nF,
                    float inflation_radius, stq_aabb *d_boxes) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (nV < 0 || nE < 0 || nF < 0 || nV + nE + nF > kMaxBoxes)
    return fail(ctx, STQ_ERR_INVALID_ARG, "box counts out of range");
  if ((nV > 0 && (!d_V0 || !d_V1)) || (nE > 0 && !d_E) || (nF > 0 && !d_F) ||
      (nV + nE + nF > 0 && !d_boxes))
    return fail(ctx, STQ_ERR_INVALID_ARG, "null buffer");
  if (nV + nE + nF == 0) return STQ_OK;
  DeviceGuard g(ctx->device);
  BatchHeader *aux = ctx->aux.as<BatchHeader>();
  STQ_CUDA(ctx, cudaMemsetAsync(aux, 0, sizeof(BatchHeader), ctx->stream), "clear flags");
  STQ_CUDA(ctx, ctx->points.ensure(2 * sizeof(float4) * size_t(std::max<int64_t>(nV, 1))),
           "allocate rounded positions");
  stage_begin(ctx, kBuild);
  STQ_CUDA(ctx, launch_build_boxes(ctx->stream, d_V0, d_V1, nV, d_E, nE, d_F, nF,
                                   ref_next_up(inflation_radius), d_boxes, &aux->flags,
                                   ctx->points.as<float4>()),
           "launch box build");
  stage_end(ctx, kBuild);
  ctx->launches += nV > 0 ? 2 : 1;
  return read_header(ctx, aux);
}

int stq_batch_build_boxes(stq_context *ctx, const double *d_V0, const double *d_V1,
                          const int64_t *h_vert_off, const int32_t *d_E, const int64_t *h_edge_off,
                          const int32_t *d_F, const int64_t *h_face_off, int n_scenes,
                          float inflation_radius, stq_aabb *d_boxes, int64_t *h_box_off) {
  if (!ctx || n_scenes < 0 || !h_vert_off || !h_edge_off || !h_face_off || !h_box_off)
    return STQ_ERR_INVALID_ARG;
  std::vector<int64_t> box_off(size_t(n_scenes) + 1, 0);
  for (int s = 0; s < n_scenes; ++s) {
    const int64_t nv = h_vert_off[s + 1] - h_vert_off[s], ne = h_edge_off[s + 1] - h_edge_off[s],
                  nf = h_face_off[s + 1] - h_face_off[s];
    if (nv < 0 || ne < 0 || nf < 0) return fail(ctx, STQ_ERR_INVALID_ARG, "decreasing mesh offsets");
    box_off[size_t(s) + 1] = box_off[size_t(s)] + nv + ne + nf;
  }
  const int64_t N = box_off[size_t(n_scenes)];
  if (N > kMaxBoxes) return fail(ctx, STQ_ERR_INVALID_ARG, "too many boxes");
  if (N > 0 && (!d_V0 || !d_V1 || !d_boxes)) return fail(ctx, STQ_ERR_INVALID_ARG, "null buffer");
  std::copy(box_off.begin(), box_off.end(), h_box_off);
  if (N == 0) return STQ_OK;
  DeviceGuard g(ctx->device);
  ctx->prepared = false;  // the staging block is reused
  STQ_TRY(ensure_staging(ctx, std::max(n_scenes, 1),
                         int(std::max<int64_t>(tiles_for(box_off.data(), n_scenes), 1))));
  fill_staging(ctx, box_off.data(), n_scenes, nullptr, STQ_AXIS_AUTO, h_vert_off, h_edge_off,
               h_face_off);
  STQ_TRY(upload_staging(ctx));
  const int64_t nv_all = h_vert_off[n_scenes];
  STQ_CUDA(ctx, ctx->points.ensure(2 * sizeof(float4) * size_t(std::max<int64_t>(nv_all, 1))),
           "allocate rounded positions");
  stage_begin(ctx, kBuild);
  STQ_CUDA(ctx, launch_batch_build(ctx->stream, d_V0, d_V1, dev_at<long long>(ctx, ctx->layout.voff),
                                   d_E, dev_at<long long>(ctx, ctx->layout.eoff), d_F,
                                   dev_at<long long>(ctx, ctx->layout.foff),
                                   dev_at<long long>(ctx, ctx->layout.box_off), dev_hdr(ctx), N,
                                   ref_next_up(inflation_radius), d_boxes, ctx->points.as<float4>(),
                                   std::max<int64_t>(nv_all, 1)),
           "launch batched box build");
  stage_end(ctx, kBuild);
  ctx->launches += 2;
  return read_header(ctx);
}

int stq_batch_prepare(stq_context *ctx, const stq_aabb *d_boxes, const int64_t *h_box_off,
                      int n_scenes, const int *h_axis, int axis) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n_scenes < 1 || !h_box_off) return fail(ctx, STQ_ERR_INVALID_ARG, "no scenes");
  if (h_box_off[0] != 0) return fail(ctx, STQ_ERR_INVALID_ARG, "box offsets must start at 0");
  for (int s = 0; s < n_scenes; ++s) {
    if (h_box_off[s + 1] < h_box_off[s]) return fail(ctx, STQ_ERR_INVALID_ARG, "decreasing box offsets");
    const int a = h_axis ? h_axis[s] : axis;
    if (a < STQ_AXIS_AUTO || a > STQ_AXIS_Z) return fail(ctx, STQ_ERR_INVALID_ARG, "axis");
  }
  if (h_box_off[n_scenes] > kMaxBoxes) return fail(ctx, STQ_ERR_INVALID_ARG, "too many boxes");
  if (h_box_off[n_scenes] > 0 && !d_boxes) return fail(ctx, STQ_ERR_INVALID_ARG, "null boxes");
  DeviceGuard g(ctx->device);
  return prepare_exact(ctx, d_boxes, h_box_off, n_scenes, h_axis, axis);
}

int stq_prepare(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int axis) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n < 0 || n > kMaxBoxes) return fail(ctx, STQ_ERR_INVALID_ARG, "box count out of range");
  const int64_t off[2] = {0, n};
  return stq_batch_prepare(ctx, d_boxes, off, 1, nullptr, axis);
}

int stq_select_axis(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int *axis_out) {
  if (!ctx || !axis_out || n < 0 || (n > 0 && !d_boxes)) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  ctx->prepared = false;  // the batch buffers are reused
  const int64_t off[2] = {0, n};
  STQ_TRY(ensure_staging(ctx, 1, int(std::max<int64_t>(tiles_for(off, 1), 1))));
  STQ_TRY(ensure_box_buffers(ctx, n));
  fill_staging(ctx, off, 1, nullptr, STQ_AXIS_AUTO, nullptr, nullptr, nullptr);
  STQ_TRY(upload_staging(ctx));
  BatchBuffers b = batch_buffers(ctx, d_boxes);
  STQ_CUDA(ctx, launch_batch_stats(ctx->stream, b), "launch statistics");
  STQ_CUDA(ctx, launch_batch_policy(ctx->stream, b), "launch policy");
  ctx->launches += 3;
  STQ_TRY(read_header(ctx));
  *axis_out = ctx->h_hdr->axis;
  return STQ_OK;
}

int64_t stq_prepared_length(const stq_context *ctx) {
  return (ctx && ctx->prepared) ? ctx->length : -1;
}

int stq_sweep_prepared(stq_context *ctx, int64_t start, int64_t max_start, stq_pair *d_pairs,
                       int64_t capacity, int64_t *count, int64_t *next_start, int64_t *total) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (!ctx->prepared) return fail(ctx, STQ_ERR_NOT_PREPARED, "call stq_prepare first");
  if (!count || !next_start || capacity < 0 || (capacity > 0 && !d_pairs))
    return fail(ctx, STQ_ERR_INVALID_ARG, "null output or negative capacity");
  const int64_t length = ctx->length;
  if (start < 0 || start > length) return fail(ctx, STQ_ERR_INVALID_ARG, "start out of range");
  DeviceGuard g(ctx->device);
  const int64_t end = (max_start <= 0 || start + max_start > length) ? length : start + max_start;
  STQ_TRY(run_sweep(ctx, start, end, d_pairs, capacity, false));
  STQ_TRY(read_header(ctx));
  const int64_t found = int64_t(ctx->h_hdr->pairs);
  if (total) *total = found;
  if (found <= capacity) {
    *count = found;
    *next_start = end;
    return STQ_OK;
  }
  // Overflow: count pairs per start position, keep the longest prefix that
  // fits, and emit exactly that prefix again.
  const int64_t m = end - start;
  STQ_CUDA(ctx, ctx->box_counts.ensure(sizeof(int32_t) * size_t(m)), "allocate box counts");
  STQ_CUDA(ctx, ctx->prefix_ws.ensure(prefix_workspace_bytes(m) + sizeof(DevScalars)),
           "allocate prefix workspace");
  STQ_CUDA(ctx, cudaMemsetAsync(ctx->box_counts.ptr, 0, sizeof(int32_t) * size_t(m), ctx->stream),
           "clear box counts");
  STQ_TRY(run_sweep(ctx, start, end, nullptr, 0, true));
  DevScalars *sel = reinterpret_cast<DevScalars *>(ctx->prefix_ws.as<char>() + prefix_workspace_bytes(m));
  STQ_CUDA(ctx, launch_prefix_select(ctx->stream, ctx->box_counts.as<int32_t>(), m, capacity,
                                     ctx->prefix_ws.ptr, sel, &ctx->launches),
           "launch prefix selection");
  DevScalars h_sel;
  STQ_CUDA(ctx, cudaMemcpyAsync(&h_sel, sel, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream),
           "read back prefix");
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  const int64_t prefix = h_sel.prefix;
  if (prefix <= 0) {
    *count = 0;
    *next_start = start;
    return fail(ctx, STQ_ERR_CAPACITY, "the first start box has more pairs than capacity");
  }
  STQ_TRY(run_sweep(ctx, start, start + prefix, d_pairs, capacity, false));
  STQ_TRY(read_header(ctx));
  *count = int64_t(ctx->h_hdr->pairs);
  *next_start = start + prefix;
  if (*count > capacity) return fail(ctx, STQ_ERR_CUDA, "prefix re-sweep exceeded capacity");
  return STQ_OVERFLOW;
}

int stq_sweep(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int axis, int64_t start,
              int64_t max_start, stq_pair *d_pairs, int64_t capacity, int64_t *count,
              int64_t *next_start, int64_t *total) {
  STQ_TRY(stq_prepare(ctx, d_boxes, n, axis));
  return stq_sweep_prepared(ctx, start, max_start, d_pairs, capacity, count, next_start, total);
}

int stq_batch_scene_pairs(stq_context *ctx, int64_t *h_counts, int n_scenes) {
  if (!ctx || !h_counts || n_scenes < 0) return STQ_ERR_INVALID_ARG;
  if (!ctx->prepared) return fail(ctx, STQ_ERR_NOT_PREPARED, "nothing prepared");
  if (n_scenes > ctx->n_scenes) return fail(ctx, STQ_ERR_INVALID_ARG, "more scenes than prepared");
  DeviceGuard g(ctx->device);
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_scene_pairs, ctx->scene_pairs.ptr,
                                sizeof(unsigned long long) * size_t(n_scenes), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "read back scene counts");
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  for (int s = 0; s < n_scenes; ++s) h_counts[s] = int64_t(ctx->h_scene_pairs[s]);
  return STQ_OK;
}

int stq_batch_broadphase(stq_context *ctx, const double *d_V0, const double *d_V1,
                         const int64_t *h_vert_off, const int32_t *d_E, const int64_t *h_edge_off,
                         const int32_t *d_F, const int64_t *h_face_off, int n_scenes,
                         float inflation_radius, int axis, stq_pair *d_pairs, int64_t capacity,
                         int64_t *count, int64_t *total, int64_t *h_scene_pairs) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n_scenes < 1 || !h_vert_off || !h_edge_off || !h_face_off || !count || capacity < 0 ||
      (capacity > 0 && !d_pairs) || axis < STQ_AXIS_AUTO || axis > STQ_AXIS_Z)
    return fail(ctx, STQ_ERR_INVALID_ARG, "invalid batch arguments");
  std::vector<int64_t> box_off(size_t(n_scenes) + 1, 0);
  for (int s = 0; s < n_scenes; ++s) {
    const int64_t nv = h_vert_off[s + 1] - h_vert_off[s], ne = h_edge_off[s + 1] - h_edge_off[s],
                  nf = h_face_off[s + 1] - h_face_off[s];
    if (nv < 0 || ne < 0 || nf < 0) return fail(ctx, STQ_ERR_INVALID_ARG, "decreasing mesh offsets");
    box_off[size_t(s) + 1] = box_off[size_t(s)] + nv + ne + nf;
  }
  const int64_t N = box_off[size_t(n_scenes)];
  if (N > kMaxBoxes / 8) return fail(ctx, STQ_ERR_INVALID_ARG, "too many boxes for one batch");
  if (N > 0 && (!d_V0 || !d_V1)) return fail(ctx, STQ_ERR_INVALID_ARG, "null mesh");
  DeviceGuard g(ctx->device);
  // capacities: replicas within the budget, cells within the policy's cap
  const int64_t T = std::max<int64_t>(tiles_for(box_off.data(), n_scenes), 1);
  const int64_t rep_cap = std::max<int64_t>(int64_t(ctx->budget) * N, 1);
  const int64_t cells_cap = N / 16 + n_scenes + 1;
  STQ_TRY(ensure_staging(ctx, n_scenes, int(T)));
  STQ_TRY(ensure_box_buffers(ctx, N));
  STQ_TRY(ensure_replica_buffers(ctx, rep_cap, cells_cap));
  STQ_CUDA(ctx, ctx->batch_boxes.ensure(sizeof(stq_aabb) * size_t(std::max<int64_t>(N, 1))),
           "allocate batch boxes");
  // the rounded positions: a graph replays for any batch whose vertices fit
  STQ_CUDA(ctx, ctx->points.ensure(2 * sizeof(float4) * size_t(std::max<int64_t>(h_vert_off[n_scenes], 1))),
           "allocate rounded positions");
  const int64_t vert_cap = int64_t(ctx->points.bytes / (2 * sizeof(float4)));
  fill_staging(ctx, box_off.data(), n_scenes, nullptr, axis, h_vert_off, h_edge_off, h_face_off);
  const stq_aabb *boxes = ctx->batch_boxes.as<stq_aabb>();
  const int cell_bits = bits_for(3 * cells_cap);
  auto enqueue_all = [&]() -> int {
    STQ_TRY(upload_staging(ctx));
    stage_begin(ctx, kBuild);
    STQ_CUDA(ctx, launch_batch_build(ctx->stream, d_V0, d_V1, dev_at<long long>(ctx, ctx->layout.voff),
                                     d_E, dev_at<long long>(ctx, ctx->layout.eoff), d_F,
                                     dev_at<long long>(ctx, ctx->layout.foff),
                                     dev_at<long long>(ctx, ctx->layout.box_off), dev_hdr(ctx),
                                     ctx->box_cap, ref_next_up(inflation_radius),
                                     ctx->batch_boxes.as<stq_aabb>(), ctx->points.as<float4>(), vert_cap),
             "launch batched box build");
    ctx->launches += 1;  // the rounding of the positions
    stage_end(ctx, kBuild);
    const BatchBuffers b = batch_buffers(ctx, boxes);
    STQ_TRY(enqueue_prepare_front(ctx, b, -1));
    STQ_TRY(enqueue_prepare_back(ctx, b, cell_bits, -1, -1));
    STQ_TRY(run_sweep(ctx, 0, ctx->slot_cap, d_pairs, capacity, false));
    STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_hdr, dev_hdr(ctx), sizeof(BatchHeader),
                                  cudaMemcpyDeviceToHost, ctx->stream),
             "read back batch header");
    STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_scene_pairs, ctx->scene_pairs.ptr,
                                  sizeof(unsigned long long) * size_t(n_scenes),
                                  cudaMemcpyDeviceToHost, ctx->stream),
             "read back scene counts");
    ctx->launches += 1;
    return STQ_OK;
  };
  const bool use_graph = ctx->options[STQ_OPT_GRAPH] != 2;
  if (use_graph) {
    if (!ctx->graph_stream) {
      STQ_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->graph_stream, cudaStreamNonBlocking),
               "create graph stream");
      STQ_CUDA(ctx, cudaEventCreateWithFlags(&ctx->graph_event, cudaEventDisableTiming),
               "create graph event");
    }
    // order after the caller's stream, then run on the private stream
    STQ_CUDA(ctx, cudaEventRecord(ctx->graph_event, ctx->stream), "record caller event");
    STQ_CUDA(ctx, cudaStreamWaitEvent(ctx->graph_stream, ctx->graph_event, 0), "wait caller event");
    cudaStream_t caller = ctx->stream;
    ctx->stream = ctx->graph_stream;
    GraphKey key;
    const void *ptrs[7] = {d_V0, d_V1, d_E, d_F, d_pairs, boxes, ctx->points.ptr};
    std::memcpy(key.ptr, ptrs, sizeof ptrs);
    const int64_t sizes[9] = {ctx->box_cap, ctx->rep_cap, ctx->slot_cap, ctx->scene_cap,
                              ctx->tile_cap, capacity, n_scenes, cell_bits, vert_cap};
    std::memcpy(key.sizes, sizes, sizeof sizes);
    static_assert(sizeof(ctx->options) / sizeof(ctx->options[0]) == 16, "options in the graph key");
    for (int o = 0; o < 16; ++o) key.opts[o] = ctx->options[o];
    key.opts[16] = int64_t(inflation_radius * 1e9f);
    key.stream = caller;
    int st = STQ_OK;
    if (!ctx->graph || !(key == ctx->graph_key)) {
      if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
      ctx->graph = nullptr;
      cudaGraph_t graph = nullptr;
      ctx->capturing = true;
      cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
      st = e == cudaSuccess ? enqueue_all() : fail(ctx, STQ_ERR_CUDA, "begin graph capture", e);
      cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
      ctx->capturing = false;
      if (st == STQ_OK && e2 != cudaSuccess) st = fail(ctx, STQ_ERR_CUDA, "end graph capture", e2);
      if (st == STQ_OK) {
        e = cudaGraphInstantiate(&ctx->graph, graph, 0);
        if (e != cudaSuccess) st = fail(ctx, STQ_ERR_CUDA, "graph instantiate", e);
      }
      if (graph) cudaGraphDestroy(graph);
      if (st == STQ_OK) ctx->graph_key = key;
    }
    if (st == STQ_OK) {
      const cudaError_t e = cudaGraphLaunch(ctx->graph, ctx->stream);
      if (e != cudaSuccess) st = fail(ctx, STQ_ERR_CUDA, "graph launch", e);
    }
    ctx->stream = caller;
    if (st != STQ_OK) return st;
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->graph_stream), "synchronise graph stream");
  } else {
    STQ_TRY(enqueue_all());
  }
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
  collect_stages(ctx);
  const BatchHeader &h = *ctx->h_hdr;
  if (h.flags & kFlagNaN) return fail(ctx, STQ_ERR_INVALID_INPUT, "a box bound is NaN");
  if (h.flags & kFlagBadIndex) return fail(ctx, STQ_ERR_INVALID_INPUT, "an edge or face vertex index is out of range");
  if (h.flags & kFlagReplicaOverflow)
    return fail(ctx, STQ_ERR_NO_MEMORY, "cell replicas exceed the replica buffers");
  ctx->n_scenes = n_scenes;
  ctx->n_boxes = N;
  ctx->length = int64_t(h.length);
  ctx->scene.length = ctx->length;
  ctx->prepared = true;
  if (h_scene_pairs)
    for (int s = 0; s < n_scenes; ++s) h_scene_pairs[s] = int64_t(ctx->h_scene_pairs[s]);
  const int64_t found = int64_t(h.pairs);
  if (total) *total = found;
  *count = std::min(found, capacity);
  return found <= capacity ? STQ_OK : STQ_OVERFLOW;
}

}  // extern "C"

namespace {

// Sweeps the prepared scene into h_pairs. The start positions are cut into
// windows (STQ_OPT_HOST_WINDOWS, default 16) that alternate between two
// slots: even windows sweep on the context's stream into e2e_pairs, odd
// windows on a second stream into window_pairs. A slot's pair counter runs on
// across its windows, so window w's pairs are the range of its slot's buffer
// between the counts after windows w - 2 and w; after each window a one-thread
// kernel stores the count in mapped host memory and restarts the slot's work
// cursor and long-run list. Both streams are filled at once, so one
// window's last blocks share the SMs with the next window's first instead of
// leaving them idle. Once window w has finished, the host reads its count and
// queues the copy of its range to the end of h_pairs filled so far on a third
// stream: the pair list's device-to-host transfer, the largest cost of a
// host-buffer call, runs beside the sweep instead of after it. If the pairs do
// not fit h_pairs the call falls back to the prefix rule of
// stq_sweep_prepared and one copy.
int sweep_to_host(stq_context *ctx, stq_pair *h_pairs, int64_t capacity, int64_t *count,
                  int64_t *total) {
  const size_t pair_bytes = sizeof(stq_pair) * size_t(capacity > 0 ? capacity : 1);
  STQ_CUDA(ctx, ctx->e2e_pairs.ensure(pair_bytes), "allocate pair staging");
  stq_pair *d_pairs = ctx->e2e_pairs.as<stq_pair>();
  const int64_t length = ctx->length;
  constexpr int64_t kMinWindow = int64_t(1) << 19;  // start positions
  const int64_t want = ctx->options[STQ_OPT_HOST_WINDOWS] ? ctx->options[STQ_OPT_HOST_WINDOWS] : 16;
  const int windows = int(std::min<int64_t>(want, length / kMinWindow));
  auto one_copy = [&]() -> int {
    int64_t next = 0;
    const int st = stq_sweep_prepared(ctx, 0, 0, d_pairs, capacity, count, &next, total);
    if (st != STQ_OK && st != STQ_OVERFLOW) return st;
    if (*count > 0) {
      STQ_CUDA(ctx, cudaMemcpyAsync(h_pairs, d_pairs, sizeof(stq_pair) * size_t(*count),
                                    cudaMemcpyDeviceToHost, ctx->stream),
               "copy pairs to host");
      STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise stream");
    }
    return st;
  };
  if (windows < 2 || capacity == 0 || ctx->options[STQ_OPT_HOST_OVERLAP] == 2) return one_copy();

  auto windowed = [&]() -> int {
    STQ_CUDA(ctx, ctx->window_pairs.ensure(pair_bytes), "allocate pair staging");
    STQ_CUDA(ctx, ctx->window_long_list.ensure(sizeof(int2) * size_t(ctx->slot_cap)), "allocate long-run list");
    STQ_CUDA(ctx, ctx->window_cursors.ensure(2 * sizeof(WindowCounters)), "allocate window cursors");
    for (cudaStream_t *st : {&ctx->copy_stream, &ctx->window_stream})
      if (!*st) STQ_CUDA(ctx, cudaStreamCreateWithFlags(st, cudaStreamNonBlocking), "create stream");
    if (!ctx->h_window_pairs) {
      STQ_CUDA(ctx, cudaHostAlloc(&ctx->h_window_pairs, sizeof(unsigned long long) * stq_context::kCopyWindows,
                                  cudaHostAllocMapped),
               "allocate window counters");
      STQ_CUDA(ctx, cudaHostGetDevicePointer(&ctx->d_window_pairs, ctx->h_window_pairs, 0),
               "map window counters");
    }
    for (cudaEvent_t *e : {&ctx->window_start, &ctx->window_done[0]})
      if (!*e) STQ_CUDA(ctx, cudaEventCreateWithFlags(e, cudaEventDisableTiming), "create event");
    for (int w = 1; w < windows; ++w)
      if (!ctx->window_done[w])
        STQ_CUDA(ctx, cudaEventCreateWithFlags(&ctx->window_done[w], cudaEventDisableTiming), "create event");

    WindowCounters *wc = ctx->window_cursors.as<WindowCounters>();
    stq_pair *slot_pairs[2] = {d_pairs, ctx->window_pairs.as<stq_pair>()};
    int2 *slot_list[2] = {ctx->long_list.as<int2>(), ctx->window_long_list.as<int2>()};
    cudaStream_t slot_stream[2] = {ctx->stream, ctx->window_stream};

    // the header reset (candidate statistics) and the stage timer run on the
    // context's stream; the second stream starts after them
    STQ_CUDA(ctx, launch_reset_sweep(ctx->stream, dev_hdr(ctx), ctx->scene_pairs.as<unsigned long long>(),
                                     ctx->scene_cap),
             "reset sweep");
    ctx->launches += 1;
    STQ_CUDA(ctx, cudaMemsetAsync(wc, 0, 2 * sizeof(WindowCounters), ctx->stream), "clear window cursors");
    stage_begin(ctx, kSweep);
    STQ_CUDA(ctx, cudaEventRecord(ctx->window_start, ctx->stream), "record window start");
    STQ_CUDA(ctx, cudaStreamWaitEvent(ctx->window_stream, ctx->window_start, 0), "order window stream");
    for (int w = 0; w < windows; ++w) {
      const int slot = w & 1;
      cudaStream_t s = slot_stream[slot];
      const SweepCursors cur{&wc[slot].pairs, &wc[slot].work, slot_list[slot], &wc[slot].long_items,
                             &wc[slot].long_work};
      const int64_t b = length * w / windows, e = length * (w + 1) / windows;
      STQ_TRY(run_sweep(ctx, b, e, slot_pairs[slot], capacity, false, false, &cur, s));
      // the count to the host by a kernel store: a copy here would wait behind
      // the pair copies on the copy engines and hold up this stream's next window
      STQ_CUDA(ctx, launch_window_step(s, &wc[slot], ctx->d_window_pairs + w), "publish window count");
      ctx->launches += 1;
      STQ_CUDA(ctx, cudaEventRecord(ctx->window_done[w], s), "record window");
    }
    // the stage (and the header read below) ends when both streams have
    for (int w = windows - 2; w < windows; ++w)
      STQ_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->window_done[w], 0), "join window streams");
    stage_end(ctx, kSweep);
    int64_t done = 0;
    for (int w = 0; w < windows; ++w) {
      STQ_CUDA(ctx, cudaEventSynchronize(ctx->window_done[w]), "wait for sweep window");
      const volatile unsigned long long *hc = ctx->h_window_pairs;
      const int64_t from = w >= 2 ? int64_t(hc[w - 2]) : 0;
      const int64_t c = int64_t(hc[w]) - from;
      if (c > capacity - done) {
        // overflow: let the windows in flight end, then take the prefix rule
        for (cudaStream_t st : {ctx->window_stream, ctx->stream, ctx->copy_stream})
          STQ_CUDA(ctx, cudaStreamSynchronize(st), "synchronise window streams");
        return one_copy();
      }
      if (c > 0)
        STQ_CUDA(ctx, cudaMemcpyAsync(h_pairs + done, slot_pairs[w & 1] + from, sizeof(stq_pair) * size_t(c),
                                      cudaMemcpyDeviceToHost, ctx->copy_stream),
                 "copy window pairs to host");
      done += c;
    }
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream), "synchronise copy stream");
    STQ_TRY(read_header(ctx));  // waits for both streams (joined above); input flags
    ctx->h_hdr->pairs = (unsigned long long)done;
    if (total) *total = done;
    *count = done;
    return STQ_OK;
  };
  const int st = windowed();
  if (st != STQ_OK && st != STQ_OVERFLOW) {
    // an error can leave windows in flight on the second stream and copies on
    // the third: wait for them, so that no later call on this context races them
    for (cudaStream_t sm : {ctx->window_stream, ctx->copy_stream, ctx->stream})
      if (sm) cudaStreamSynchronize(sm);
  }
  return st;
}

}  // namespace

extern "C" {

int stq_sweep_host(stq_context *ctx, const stq_aabb *h_boxes, int64_t n, int axis,
                   stq_pair *h_pairs, int64_t capacity, int64_t *count, int64_t *total) {
  if (!ctx) return STQ_ERR_INVALID_ARG;
  if (n < 0 || n > kMaxBoxes || (n > 0 && !h_boxes) || capacity < 0 ||
      (capacity > 0 && !h_pairs) || !count)
    return fail(ctx, STQ_ERR_INVALID_ARG, "invalid host sweep arguments");
  DeviceGuard g(ctx->device);
  STQ_CUDA(ctx, ctx->e2e_boxes.ensure(sizeof(stq_aabb) * size_t(n > 0 ? n : 1)),
           "allocate box staging");
  if (n > 0)
    STQ_CUDA(ctx, cudaMemcpyAsync(ctx->e2e_boxes.ptr, h_boxes, sizeof(stq_aabb) * size_t(n),
                                  cudaMemcpyHostToDevice, ctx->stream),
             "copy boxes to device");
  STQ_TRY(stq_prepare(ctx, ctx->e2e_boxes.as<stq_aabb>(), n, axis));
  return sweep_to_host(ctx, h_pairs, capacity, count, total);
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
  char *base = ctx->e2e_mesh.as<char>();
  if (bv) {
    STQ_CUDA(ctx, cudaMemcpyAsync(base, h_V0, bv, cudaMemcpyHostToDevice, ctx->stream), "copy V0");
    STQ_CUDA(ctx, cudaMemcpyAsync(base + oV1, h_V1, bv, cudaMemcpyHostToDevice, ctx->stream), "copy V1");
  }
  if (be) STQ_CUDA(ctx, cudaMemcpyAsync(base + oE, h_E, be, cudaMemcpyHostToDevice, ctx->stream), "copy E");
  if (bf) STQ_CUDA(ctx, cudaMemcpyAsync(base + oF, h_F, bf, cudaMemcpyHostToDevice, ctx->stream), "copy F");
  STQ_TRY(stq_build_boxes(ctx, reinterpret_cast<const double *>(base),
                          reinterpret_cast<const double *>(base + oV1), nV,
                          reinterpret_cast<const int32_t *>(base + oE), nE,
                          reinterpret_cast<const int32_t *>(base + oF), nF, inflation_radius,
                          ctx->e2e_boxes.as<stq_aabb>()));
  STQ_TRY(stq_prepare(ctx, ctx->e2e_boxes.as<stq_aabb>(), n, axis));
  return sweep_to_host(ctx, h_pairs, capacity, count, total);
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

int stq_autotune(stq_context *ctx, const stq_aabb *d_boxes, const int64_t *h_box_off, int n_scenes,
                 stq_pair *d_pairs, int64_t capacity, double *best_ms) {
  if (!ctx || !best_ms || n_scenes < 1 || !h_box_off || capacity < 0 || (capacity > 0 && !d_pairs))
    return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  *best_ms = 0.0;
  const int64_t key = (int64_t(bits_for(std::max<int64_t>(h_box_off[n_scenes], 1))) << 32) |
                      int64_t(bits_for(n_scenes));
  constexpr int kOpts = 8;
  const int opts[kOpts] = {STQ_OPT_LANES_PER_ENTRY, STQ_OPT_QUEUE_DEPTH, STQ_OPT_BLOCK_SIZE,
                           STQ_OPT_RADIX_BITS, STQ_OPT_CELL_SCALE, STQ_OPT_CANDIDATES_PER_LANE,
                           STQ_OPT_SWEEP_SHAPE, STQ_OPT_RUN_CAP};
  for (const auto &kv : ctx->tuned)
    if (kv.first == key) {
      for (int o = 0; o < kOpts; ++o) STQ_TRY(stq_context_set_option(ctx, opts[o], kv.second[size_t(o)]));
      return stq_batch_prepare(ctx, d_boxes, h_box_off, n_scenes, nullptr, STQ_AXIS_AUTO);
    }
  const bool was_timing = ctx->timing;
  ctx->timing = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  STQ_CUDA(ctx, cudaEventCreate(&e0), "create event");
  STQ_CUDA(ctx, cudaEventCreate(&e1), "create event");
  // each setting: the fastest of kReps timed runs (the GPU may be shared)
  constexpr int kReps = 5;
  auto elapsed = [&](const std::function<int()> &fn, float *ms) -> int {
    float best = 1e30f;
    for (int rep = 0; rep < kReps; ++rep) {
      STQ_CUDA(ctx, cudaEventRecord(e0, ctx->stream), "record");
      STQ_TRY(fn());
      STQ_CUDA(ctx, cudaEventRecord(e1, ctx->stream), "record");
      STQ_CUDA(ctx, cudaEventSynchronize(e1), "synchronise");
      float t = 0.f;
      STQ_CUDA(ctx, cudaEventElapsedTime(&t, e0, e1), "elapsed");
      best = std::min(best, t);
    }
    *ms = best;
    return STQ_OK;
  };
  // a sweep setting: shape, lanes per entry, candidates per lane (or filter
  // steps of the flat shape), queue depth, block size, and the run length past
  // which the warp pass takes a run over (the work split; 512 by default)
  struct Shape {
    int64_t shape, lanes, per_lane, queue, block, run_cap;
  };
  std::vector<Shape> space;
  for (int64_t per_lane : {2, 4, 8})  // one start box per lane: the ring holds >= 32
    for (int64_t queue : {32, 64})
      for (int64_t block : {128, 256, 512}) space.push_back({kShapeRing, 1, per_lane, queue, block, 512});
  for (int64_t lanes : {4, 8, 16})  // lane groups sharing a start box
    for (int64_t queue : {16, 32, 64})
      for (int64_t block : {128, 256, 512}) space.push_back({kShapeRing, lanes, 8, queue, block, 512});
  for (int64_t steps : {2, 4})  // flat: runs of 32 start boxes end to end
    for (int64_t block : {128, 256})
      for (int64_t run_cap : {512, 4096}) space.push_back({kShapeFlat, 1, steps, 64, block, run_cap});
  std::vector<int64_t> best_set(kOpts, 0);
  float best_total = 1e30f;
  int st = STQ_OK;
  for (int64_t scale : {1, 2, 4, 8}) {
    if ((st = stq_context_set_option(ctx, STQ_OPT_CELL_SCALE, scale)) != STQ_OK) break;
    // the radix width changes the prepare only: the sorted scene is the same
    float t_prep = 1e30f;
    int64_t best_radix = 8;
    for (int64_t radix : {8, 4}) {
      if ((st = stq_context_set_option(ctx, STQ_OPT_RADIX_BITS, radix)) != STQ_OK) break;
      float t = 0.f;
      st = elapsed([&] { return stq_batch_prepare(ctx, d_boxes, h_box_off, n_scenes, nullptr, STQ_AXIS_AUTO); },
                   &t);
      if (st != STQ_OK) break;
      if (t < t_prep) {
        t_prep = t;
        best_radix = radix;
      }
    }
    if (st != STQ_OK) break;
    for (const Shape &sh : space) {
      stq_context_set_option(ctx, STQ_OPT_SWEEP_SHAPE, sh.shape);
      stq_context_set_option(ctx, STQ_OPT_LANES_PER_ENTRY, sh.lanes);
      stq_context_set_option(ctx, STQ_OPT_CANDIDATES_PER_LANE, sh.per_lane);
      stq_context_set_option(ctx, STQ_OPT_QUEUE_DEPTH, sh.queue);
      stq_context_set_option(ctx, STQ_OPT_BLOCK_SIZE, sh.block);
      stq_context_set_option(ctx, STQ_OPT_RUN_CAP, sh.run_cap);
      float t_sweep = 0.f;
      int64_t count = 0, next = 0, total = 0;
      st = elapsed([&] {
        const int r = stq_sweep_prepared(ctx, 0, 0, d_pairs, capacity, &count, &next, &total);
        return r == STQ_OVERFLOW ? STQ_OK : r;
      }, &t_sweep);
      if (st != STQ_OK) break;
      if (t_prep + t_sweep < best_total) {
        best_total = t_prep + t_sweep;
        best_set = {sh.lanes, sh.queue, sh.block, best_radix, scale, sh.per_lane, sh.shape, sh.run_cap};
      }
    }
    if (st != STQ_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->timing = was_timing;
  if (st != STQ_OK) return st;
  for (int o = 0; o < kOpts; ++o) STQ_TRY(stq_context_set_option(ctx, opts[o], best_set[size_t(o)]));
  ctx->tuned.emplace_back(key, best_set);
  *best_ms = double(best_total);
  return stq_batch_prepare(ctx, d_boxes, h_box_off, n_scenes, nullptr, STQ_AXIS_AUTO);
}

int stq_brute_force(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, stq_pair *d_pairs,
                    int64_t capacity, int64_t *count) {
  if (!ctx || !count || n < 0 || n > kMaxBoxes || (n > 0 && !d_boxes) || capacity < 0 ||
      (capacity > 0 && !d_pairs))
    return STQ_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  BatchHeader *aux = ctx->aux.as<BatchHeader>();
  STQ_CUDA(ctx, cudaMemsetAsync(aux, 0, sizeof(BatchHeader), ctx->stream), "clear counters");
  STQ_CUDA(ctx, launch_brute_force(ctx->stream, d_boxes, n, d_pairs, capacity, &aux->pairs),
           "launch brute force");
  ctx->launches += 1;
  STQ_TRY(read_header(ctx, aux));
  *count = int64_t(ctx->h_hdr->pairs);
  return *count > capacity ? STQ_OVERFLOW : STQ_OK;
}

}  // extern "C"
