// server.cu - continuous batching of time-stepped broad-phase requests.
//
// Each tick runs the batched pipeline (box build from each request's own
// device mesh, per-scene axis and cells, one sort, one persistent sweep,
// per-request pair checksums) over the current timestep of every admitted
// request, as one captured CUDA graph whose capacities are fixed when the
// server is created. Between ticks the host admits queued requests in
// arrival order while they fit the HBM budget, the box capacity and the
// scene capacity; their uploads run on a copy stream while the previous tick
// is still on the GPU. A request's mesh stays in HBM for all its timesteps:
// the next step's positions are made on the device (t0 <- t1, t1 <- t1 + noise).
#include <cmath>
#include <deque>
#include <memory>
#include <unordered_map>

#include "context.h"

using namespace stq::ctxops;

namespace stq {
namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double unit(unsigned long long h) {  // [0, 1)
  return double(h >> 11) * 0x1.0p-53;
}

// t0 <- t1, t1 <- t1 + sigma * N(0, 1) for every coordinate of scenes whose
// step is past 0. The normal draw is Box-Muller over two counter-based
// uniforms keyed by (seed, step, coordinate index).
__global__ void __launch_bounds__(256)
advance_kernel(const MeshRef *__restrict__ refs, const long long *__restrict__ voff,
               const BatchHeader *hdr, int64_t vert_cap) {
  const int S = hdr->n_scenes;
  const long long total = voff[S] < vert_cap ? voff[S] : vert_cap;
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < total; i += gridDim.x * 256ll) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (voff[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const MeshRef &m = refs[lo];
    if (m.step == 0) continue;
    const long long v = i - voff[lo];
    const unsigned long long key = mix64(m.seed ^ mix64((unsigned long long)m.step));
    for (int k = 0; k < 3; ++k) {
      const unsigned long long c = (unsigned long long)(3 * v + k);
      const double u1 = 1.0 - unit(mix64(key ^ (2 * c)));
      const double u2 = unit(mix64(key ^ (2 * c + 1)));
      const double z = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
      const double x = m.V1[3 * v + k];
      m.V0[3 * v + k] = x;
      m.V1[3 * v + k] = x + m.sigma * z;
    }
  }
}

// XOR over each scene's pairs of mix64((lo << 32) | hi), ids local to the
// scene. A warp takes kChecksumChunk consecutive pairs, 32 per step (one per
// lane, coalesced), and keeps the XOR of the current scene in its lanes'
// registers. The pair list holds runs of one scene (each sweep warp appends
// 32 or more pairs of consecutive start positions at once), so the warp
// reduces its registers and flushes them with one atomic per run: at a scene
// change inside a step, the lanes still in the old scene add to the registers
// before the flush, and the lanes of the new scene after it. A lane whose pair
// lies in a third scene within one step adds it alone. Those XORs go to a
// per-block table of the scenes in shared memory when it fits (SMEM), and the
// block adds its table to the scenes' checksums once at the end: millions of
// runs would otherwise contend on a few dozen global addresses.
constexpr int kChecksumChunk = 1024;
constexpr int kChecksumSmemScenes = 4096;  // 32 KB of shared memory

__device__ __forceinline__ int scene_of(const long long *__restrict__ box_off, int S, long long id) {
  int lo = 0, hi = S - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (box_off[mid] <= id) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <bool SMEM>
__global__ void __launch_bounds__(256)
pair_checksum_kernel(const int2 *__restrict__ pairs, long long capacity, const BatchHeader *hdr,
                     const long long *__restrict__ box_off, unsigned long long *checks) {
  extern __shared__ unsigned long long block_checks[];  // SMEM: one per scene
  const long long n = min((long long)hdr->pairs, capacity);
  const int S = hdr->n_scenes;
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * 256ll + threadIdx.x) >> 5;
  const long long nwarps = (gridDim.x * 256ll) >> 5;
  unsigned long long *acc_to = SMEM ? block_checks : checks;
  if (SMEM) {
    for (int s = threadIdx.x; s < S; s += 256) block_checks[s] = 0ull;
    __syncthreads();
  }
  auto flush = [&](int cur, unsigned long long acc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc ^= __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && cur >= 0 && acc) atomicXor(&acc_to[cur], acc);
  };
  for (long long base = warp * kChecksumChunk; base < n; base += nwarps * kChecksumChunk) {
    const long long end = min(base + kChecksumChunk, n);
    int cur = -1;  // warp-uniform: scene of the registers' XOR
    long long b0 = 0, b1 = 0;
    unsigned long long acc = 0;
    for (long long q0 = base; q0 < end; q0 += 32) {
      const long long q = q0 + lane;
      const bool valid = q < end;
      int2 p = make_int2(0, 0);
      if (valid) p = pairs[q];
      const bool in = valid && p.x >= b0 && p.x < b1;
      if (in) {
        const unsigned long long a = (unsigned long long)(p.x - b0), c = (unsigned long long)(p.y - b0);
        acc ^= mix64((a << 32) | c);
      }
      const unsigned outm = __ballot_sync(0xffffffffu, valid && !in);
      if (outm) {
        // the scene changes: flush, and take the scene of the first lane outside
        flush(cur, acc);
        acc = 0;
        const int leader = __ffs(outm) - 1;
        int s = 0;
        if (lane == leader) s = scene_of(box_off, S, p.x);
        cur = __shfl_sync(0xffffffffu, s, leader);
        b0 = box_off[cur];
        b1 = box_off[cur + 1];
        if (valid && !in) {
          const bool in_new = p.x >= b0 && p.x < b1;
          const int t = in_new ? cur : scene_of(box_off, S, p.x);
          const unsigned long long a = (unsigned long long)(p.x - box_off[t]),
                                   c = (unsigned long long)(p.y - box_off[t]);
          const unsigned long long h = mix64((a << 32) | c);
          if (in_new) acc ^= h;
          else atomicXor(&acc_to[t], h);
        }
      }
    }
    flush(cur, acc);
  }
  if (SMEM) {
    __syncthreads();
    for (int s = threadIdx.x; s < S; s += 256)
      if (block_checks[s]) atomicXor(&checks[s], block_checks[s]);
  }
}

}  // namespace

cudaError_t launch_advance(cudaStream_t s, const MeshRef *refs, const long long *voff,
                           const BatchHeader *hdr, int64_t vert_cap) {
  int64_t g = (vert_cap + 255) / 256;
  g = g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
  advance_kernel<<<unsigned(g), 256, 0, s>>>(refs, voff, hdr, vert_cap);
  return cudaGetLastError();
}

cudaError_t launch_pair_checksums(cudaStream_t s, const stq_pair *pairs, long long capacity,
                                  const BatchHeader *hdr, const long long *box_off,
                                  unsigned long long *checks, int scene_cap) {
  cudaError_t e = cudaMemsetAsync(checks, 0, sizeof(unsigned long long) * size_t(scene_cap), s);
  if (e != cudaSuccess) return e;
  int64_t g = (capacity / kChecksumChunk + 7) / 8;  // 8 warps per block
  g = g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
  if (scene_cap <= kChecksumSmemScenes)
    pair_checksum_kernel<true><<<unsigned(g), 256, sizeof(unsigned long long) * size_t(scene_cap), s>>>(
        reinterpret_cast<const int2 *>(pairs), capacity, hdr, box_off, checks);
  else
    pair_checksum_kernel<false><<<unsigned(g), 256, 0, s>>>(reinterpret_cast<const int2 *>(pairs), capacity,
                                                            hdr, box_off, checks);
  return cudaGetLastError();
}

}  // namespace stq

namespace {

struct Request {
  int64_t id = 0;
  int steps = 1;
  double sigma = 0.0;
  uint64_t seed = 0;
  int64_t nV = 0, nE = 0, nF = 0;
  char *host = nullptr;  // pinned copy of the submitted mesh, until admitted
  void *dmem = nullptr;  // V0 | V1 | E | F on the device
  size_t oV1 = 0, oE = 0, oF = 0, bytes = 0;
  int step = 0;          // next timestep to run
  int64_t first_tick = -1, last_tick = -1;  // ticks that ran its first and last step
  int64_t est_pairs = 0;
  int64_t footprint = 0;
  std::vector<int64_t> counts;
  std::vector<uint64_t> checks;
  int64_t boxes() const { return nV + nE + nF; }
};

constexpr int64_t kInitialPairsPerBox = 12;

}  // namespace

struct stq_server {
  int device = 0;
  stq_context *ctx = nullptr;  // pipeline buffers, staging and stream
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_done = nullptr;
  int64_t budget = 0, max_boxes = 0, fixed = 0;
  int max_scenes = 0;
  int64_t next_id = 1, held = 0, ticks = 0;
  double density = 16.0;  // pairs per box seen so far (pair-buffer estimates)
  std::deque<Request *> queue;
  std::vector<Request *> active;
  std::unordered_map<int64_t, std::unique_ptr<Request>> all;
  bool in_flight = false;
  std::vector<Request *> batch;
  // tick tables: device copies and pinned host mirrors
  DevBuf refs_dev, voff_dev, checks_dev, pairs;
  MeshRef *refs_host = nullptr;
  long long *voff_host = nullptr;
  unsigned long long *checks_host = nullptr;
  int64_t pair_cap = 0;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_pair_cap = -1;
};

namespace {

int sfail(stq_server *s, int status, const char *what, cudaError_t e = cudaSuccess) {
  return fail(s->ctx, status, what, e);
}

int64_t active_boxes(const stq_server *s) {
  int64_t b = 0;
  for (const Request *r : s->active) b += r->boxes();
  return b;
}

// Everything of one tick on the context's stream: tables, advance (optional),
// build, prepare, sweep, checksums, read-back copies.
int enqueue_tick(stq_server *sv, bool advance) {
  stq_context *ctx = sv->ctx;
  const int S = int(sv->batch.size());
  STQ_CUDA(ctx, cudaMemcpyAsync(sv->refs_dev.ptr, sv->refs_host, sizeof(MeshRef) * size_t(sv->max_scenes),
                                cudaMemcpyHostToDevice, ctx->stream),
           "upload scene table");
  STQ_CUDA(ctx, cudaMemcpyAsync(sv->voff_dev.ptr, sv->voff_host, sizeof(long long) * size_t(sv->max_scenes + 1),
                                cudaMemcpyHostToDevice, ctx->stream),
           "upload vertex offsets");
  STQ_TRY(upload_staging(ctx));
  BatchHeader *hdr = dev_hdr(ctx);
  if (advance)
    STQ_CUDA(ctx, launch_advance(ctx->stream, sv->refs_dev.as<MeshRef>(), sv->voff_dev.as<long long>(),
                                 hdr, sv->max_boxes),
             "launch advance");
  const long long *box_off = dev_at<long long>(ctx, ctx->layout.box_off);
  STQ_CUDA(ctx, launch_batch_build_refs(ctx->stream, sv->refs_dev.as<MeshRef>(), box_off, hdr, ctx->box_cap,
                                        ref_next_up(0.f), ctx->batch_boxes.as<stq_aabb>()),
           "launch box build");
  const BatchBuffers b = batch_buffers(ctx, ctx->batch_boxes.as<stq_aabb>());
  STQ_TRY(enqueue_prepare_front(ctx, b, -1));
  STQ_TRY(enqueue_prepare_back(ctx, b, bits_for(3 * (sv->max_boxes / 16 + sv->max_scenes + 1)), -1, -1));
  STQ_TRY(run_sweep(ctx, 0, ctx->slot_cap, sv->pairs.as<stq_pair>(), sv->pair_cap, false));
  STQ_CUDA(ctx, launch_pair_checksums(ctx->stream, sv->pairs.as<stq_pair>(), sv->pair_cap, hdr, box_off,
                                      sv->checks_dev.as<unsigned long long>(), sv->max_scenes),
           "launch checksums");
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_hdr, hdr, sizeof(BatchHeader), cudaMemcpyDeviceToHost, ctx->stream),
           "read back header");
  STQ_CUDA(ctx, cudaMemcpyAsync(ctx->h_scene_pairs, ctx->scene_pairs.ptr,
                                sizeof(unsigned long long) * size_t(sv->max_scenes), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "read back scene counts");
  STQ_CUDA(ctx, cudaMemcpyAsync(sv->checks_host, sv->checks_dev.ptr,
                                sizeof(unsigned long long) * size_t(sv->max_scenes), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "read back checksums");
  (void)S;
  ctx->launches += 4;
  return STQ_OK;
}

// Fills the pinned tables for the current batch (sv->batch).
void fill_tables(stq_server *sv) {
  stq_context *ctx = sv->ctx;
  const int S = int(sv->batch.size());
  std::vector<int64_t> box_off(size_t(S) + 1, 0);
  sv->voff_host[0] = 0;
  for (int k = 0; k < S; ++k) {
    const Request *r = sv->batch[size_t(k)];
    char *d = static_cast<char *>(r->dmem);
    MeshRef &m = sv->refs_host[k];
    m.V0 = reinterpret_cast<double *>(d);
    m.V1 = reinterpret_cast<double *>(d + r->oV1);
    m.E = reinterpret_cast<const int32_t *>(d + r->oE);
    m.F = reinterpret_cast<const int32_t *>(d + r->oF);
    m.nV = r->nV, m.nE = r->nE, m.nF = r->nF;
    m.seed = r->seed;
    m.sigma = r->sigma;
    m.step = r->step;
    m.pad = 0;
    box_off[size_t(k) + 1] = box_off[size_t(k)] + r->boxes();
    sv->voff_host[k + 1] = sv->voff_host[k] + r->nV;
  }
  fill_staging(ctx, box_off.data(), S, nullptr, STQ_AXIS_AUTO, nullptr, nullptr, nullptr);
}

int launch_tick(stq_server *sv) {
  stq_context *ctx = sv->ctx;
  int64_t need = 0;
  for (const Request *r : sv->batch) need += r->est_pairs;
  if (need > sv->pair_cap) {
    const int64_t cap = need + need / 4 + 1024;
    STQ_CUDA(ctx, sv->pairs.ensure(sizeof(stq_pair) * size_t(cap)), "allocate pair buffer");
    sv->pair_cap = cap;
  }
  fill_tables(sv);
  STQ_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, sv->copy_done, 0), "wait for uploads");
  if (ctx->options[STQ_OPT_GRAPH] == 2) return enqueue_tick(sv, true);
  if (!sv->graph || sv->graph_pair_cap != sv->pair_cap) {
    if (sv->graph) cudaGraphExecDestroy(sv->graph);
    sv->graph = nullptr;
    cudaGraph_t g = nullptr;
    ctx->capturing = true;
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? enqueue_tick(sv, true) : sfail(sv, STQ_ERR_CUDA, "begin capture", e);
    const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
    ctx->capturing = false;
    if (st == STQ_OK && e2 != cudaSuccess) st = sfail(sv, STQ_ERR_CUDA, "end capture", e2);
    if (st == STQ_OK) {
      e = cudaGraphInstantiate(&sv->graph, g, 0);
      if (e != cudaSuccess) st = sfail(sv, STQ_ERR_CUDA, "instantiate", e);
    }
    if (g) cudaGraphDestroy(g);
    if (st != STQ_OK) return st;
    sv->graph_pair_cap = sv->pair_cap;
  }
  STQ_CUDA(ctx, cudaGraphLaunch(sv->graph, ctx->stream), "launch tick graph");
  return STQ_OK;
}

void release(Request *r) {
  if (r->dmem) cudaFree(r->dmem);
  r->dmem = nullptr;
  if (r->host) cudaFreeHost(r->host);
  r->host = nullptr;
}

// Waits for the tick in flight and hands its results to the requests.
int collect(stq_server *sv, int64_t *done_ids, int max_done, int *n_done) {
  stq_context *ctx = sv->ctx;
  STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise tick");
  sv->in_flight = false;
  const BatchHeader &h = *ctx->h_hdr;
  if (h.flags & (kFlagNaN | kFlagBadIndex)) return sfail(sv, STQ_ERR_INVALID_INPUT, "invalid request mesh");
  if (h.flags & kFlagReplicaOverflow) return sfail(sv, STQ_ERR_NO_MEMORY, "replica buffers exceeded");
  if (int64_t(h.pairs) > sv->pair_cap) {
    // the pair estimate was short: grow the buffer and sweep this step again
    // (positions are already advanced, so no second advance)
    const int64_t cap = int64_t(h.pairs) + int64_t(h.pairs) / 4 + 1024;
    STQ_CUDA(ctx, sv->pairs.ensure(sizeof(stq_pair) * size_t(cap)), "allocate pair buffer");
    sv->pair_cap = cap;
    STQ_TRY(enqueue_tick(sv, false));
    STQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "synchronise tick");
  }
  for (size_t k = 0; k < sv->batch.size(); ++k) {
    Request *r = sv->batch[k];
    const int64_t c = int64_t(ctx->h_scene_pairs[k]);
    r->counts.push_back(c);
    r->checks.push_back(uint64_t(sv->checks_host[k]));
    r->est_pairs = std::max(r->est_pairs, c + c / 4 + 64);
    sv->density = 0.9 * sv->density + 0.1 * double(c) / double(std::max<int64_t>(r->boxes(), 1));
    r->step += 1;
    if (r->step >= r->steps) {
      r->last_tick = sv->ticks - 1;
      release(r);
      sv->held -= r->footprint;
      sv->active.erase(std::find(sv->active.begin(), sv->active.end(), r));
      if (*n_done < max_done && done_ids) done_ids[*n_done] = r->id;
      ++*n_done;
    }
  }
  sv->batch.clear();
  return STQ_OK;
}

}  // namespace

extern "C" {

int stq_server_create(int device, void *stream, int64_t budget_bytes, int64_t max_boxes,
                      int max_scenes, stq_server **out) {
  if (!out || budget_bytes <= 0 || max_boxes <= 0 || max_scenes <= 0 || max_boxes > kMaxBoxes / 8)
    return STQ_ERR_INVALID_ARG;
  *out = nullptr;
  std::unique_ptr<stq_server> sv(new (std::nothrow) stq_server());
  if (!sv) return STQ_ERR_NO_MEMORY;
  int st = stq_context_create(device, stream, &sv->ctx);
  if (st != STQ_OK) return st;
  stq_context *ctx = sv->ctx;
  // serving batches of many dense time-stepped scenes sweep fastest in the
  // flat shape with four filter steps per round (measured on 24 cloth-pair
  // requests: 47 ms per tick against 66 ms for lane groups of 8);
  // stq_server_set_option changes it
  stq_context_set_option(ctx, STQ_OPT_SWEEP_SHAPE, kShapeFlat);
  stq_context_set_option(ctx, STQ_OPT_CANDIDATES_PER_LANE, 4);
  stq_context_set_option(ctx, STQ_OPT_BLOCK_SIZE, 256);
  DeviceGuard g(device);
  sv->device = device;
  sv->budget = budget_bytes;
  sv->max_boxes = max_boxes;
  sv->max_scenes = max_scenes;
  auto bad = [&](int s) {
    stq_server_destroy(sv.release());
    return s;
  };
  if (!ctx->stream) {
    // a private stream: the legacy default stream cannot be captured
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(STQ_ERR_CUDA);
    ctx->owns_stream = true;
  }
  if (cudaStreamCreateWithFlags(&sv->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&sv->copy_done, cudaEventDisableTiming) != cudaSuccess)
    return bad(STQ_ERR_CUDA);
  // pipeline buffers for the largest batch, counted against the budget
  const int64_t tiles = max_boxes / kTileBoxes + max_scenes + 1;
  if (ensure_staging(ctx, max_scenes, int(tiles)) != STQ_OK || ensure_box_buffers(ctx, max_boxes) != STQ_OK ||
      ensure_replica_buffers(ctx, int64_t(ctx->budget) * max_boxes, max_boxes / 16 + max_scenes + 1) != STQ_OK ||
      ctx->batch_boxes.ensure(sizeof(stq_aabb) * size_t(max_boxes)) != cudaSuccess ||
      sv->refs_dev.ensure(sizeof(MeshRef) * size_t(max_scenes)) != cudaSuccess ||
      sv->voff_dev.ensure(sizeof(long long) * size_t(max_scenes + 1)) != cudaSuccess ||
      sv->checks_dev.ensure(sizeof(unsigned long long) * size_t(max_scenes)) != cudaSuccess ||
      cudaMallocHost(&sv->refs_host, sizeof(MeshRef) * size_t(max_scenes)) != cudaSuccess ||
      cudaMallocHost(&sv->voff_host, sizeof(long long) * size_t(max_scenes + 1)) != cudaSuccess ||
      cudaMallocHost(&sv->checks_host, sizeof(unsigned long long) * size_t(max_scenes)) != cudaSuccess)
    return bad(STQ_ERR_NO_MEMORY);
  std::memset(sv->refs_host, 0, sizeof(MeshRef) * size_t(max_scenes));
  std::memset(sv->voff_host, 0, sizeof(long long) * size_t(max_scenes + 1));
  size_t free_b = 0, total = 0;
  cudaMemGetInfo(&free_b, &total);
  sv->fixed = int64_t(ctx->in_dev.bytes + ctx->counts.bytes + ctx->offsets.bytes + ctx->scan_ws.bytes +
                      ctx->keys64[0].bytes * 2 + ctx->vals[0].bytes * 2 + ctx->sort_ws.bytes + ctx->xmin.bytes + ctx->xmax.bytes +
                      ctx->syz.bytes + ctx->sv.bytes + ctx->sflag.bytes + ctx->sfloor.bytes +
                      ctx->cell_floor.bytes + ctx->partner.bytes + ctx->run_end.bytes +
                      ctx->seg_scan.bytes + ctx->batch_boxes.bytes);
  if (sv->fixed >= budget_bytes) return bad(STQ_ERR_NO_MEMORY);
  *out = sv.release();
  return STQ_OK;
}

void stq_server_destroy(stq_server *sv) {
  if (!sv) return;
  {
    DeviceGuard g(sv->device);
    if (sv->ctx && sv->ctx->stream) cudaStreamSynchronize(sv->ctx->stream);
    if (sv->copy_stream) cudaStreamSynchronize(sv->copy_stream);
    for (auto &kv : sv->all) release(kv.second.get());
    if (sv->graph) cudaGraphExecDestroy(sv->graph);
    sv->refs_dev.release();
    sv->voff_dev.release();
    sv->checks_dev.release();
    sv->pairs.release();
    if (sv->refs_host) cudaFreeHost(sv->refs_host);
    if (sv->voff_host) cudaFreeHost(sv->voff_host);
    if (sv->checks_host) cudaFreeHost(sv->checks_host);
    if (sv->copy_done) cudaEventDestroy(sv->copy_done);
    if (sv->copy_stream) cudaStreamDestroy(sv->copy_stream);
  }
  stq_context_destroy(sv->ctx);
  delete sv;
}

int stq_server_submit(stq_server *sv, const double *h_V0, const double *h_V1, int64_t nV,
                      const int32_t *h_E, int64_t nE, const int32_t *h_F, int64_t nF, int steps,
                      double sigma, uint64_t seed, int64_t *request_id) {
  if (!sv || !request_id || nV < 0 || nE < 0 || nF < 0 || steps < 1 || !(sigma >= 0.0) ||
      (nV > 0 && (!h_V0 || !h_V1)) || (nE > 0 && !h_E) || (nF > 0 && !h_F))
    return STQ_ERR_INVALID_ARG;
  if (nV + nE + nF > sv->max_boxes || nV + nE + nF == 0)
    return sfail(sv, STQ_ERR_CAPACITY, "request larger than one launch's box capacity, or empty");
  DeviceGuard g(sv->device);
  auto r = std::make_unique<Request>();
  r->id = sv->next_id++;
  r->steps = steps;
  r->sigma = sigma;
  r->seed = seed;
  r->nV = nV, r->nE = nE, r->nF = nF;
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t bv = sizeof(double) * 3 * size_t(nV);
  r->oV1 = up(bv);
  r->oE = r->oV1 + up(bv);
  r->oF = r->oE + up(sizeof(int32_t) * 2 * size_t(nE));
  r->bytes = r->oF + up(sizeof(int32_t) * 3 * size_t(nF));
  STQ_CUDA(sv->ctx, cudaMallocHost(&r->host, r->bytes), "allocate pinned request copy");
  std::memcpy(r->host, h_V0, bv);
  std::memcpy(r->host + r->oV1, h_V1, bv);
  if (nE) std::memcpy(r->host + r->oE, h_E, sizeof(int32_t) * 2 * size_t(nE));
  if (nF) std::memcpy(r->host + r->oF, h_F, sizeof(int32_t) * 3 * size_t(nF));
  r->est_pairs = int64_t(std::max(double(kInitialPairsPerBox), 1.3 * sv->density) * double(r->boxes()));
  r->footprint = int64_t(r->bytes) + int64_t(sizeof(stq_pair)) * r->est_pairs;
  *request_id = r->id;
  sv->queue.push_back(r.get());
  sv->all.emplace(r->id, std::move(r));
  return STQ_OK;
}

int stq_server_tick(stq_server *sv, int64_t *done_ids, int max_done, int *n_done) {
  if (!sv || !n_done || max_done < 0) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(sv->device);
  *n_done = 0;
  // 1. admit in arrival order while the head of the queue fits; its upload
  //    overlaps the tick in flight
  int64_t boxes = active_boxes(sv);
  while (!sv->queue.empty()) {
    Request *r = sv->queue.front();
    if (int(sv->active.size()) >= sv->max_scenes || boxes + r->boxes() > sv->max_boxes ||
        sv->fixed + sv->held + r->footprint > sv->budget)
      break;
    if (cudaMalloc(&r->dmem, r->bytes) != cudaSuccess) {
      r->dmem = nullptr;
      cudaGetLastError();
      break;
    }
    STQ_CUDA(sv->ctx, cudaMemcpyAsync(r->dmem, r->host, r->bytes, cudaMemcpyHostToDevice, sv->copy_stream),
             "upload request");
    sv->held += r->footprint;
    boxes += r->boxes();
    sv->active.push_back(r);
    sv->queue.pop_front();
  }
  STQ_CUDA(sv->ctx, cudaEventRecord(sv->copy_done, sv->copy_stream), "record uploads");
  // 2. results of the tick in flight; finished requests leave
  if (sv->in_flight) STQ_TRY(collect(sv, done_ids, max_done, n_done));
  // 3. next tick over the current timestep of every active request
  if (sv->active.empty()) return STQ_OK;
  sv->batch = sv->active;
  for (Request *r : sv->batch)
    if (r->first_tick < 0) r->first_tick = sv->ticks;
  STQ_TRY(launch_tick(sv));
  sv->in_flight = true;
  sv->ticks += 1;
  return STQ_OK;
}

int stq_server_result(stq_server *sv, int64_t request_id, int64_t *counts, uint64_t *checksums,
                      int max_steps, int *steps_done) {
  if (!sv || !steps_done || max_steps < 0) return STQ_ERR_INVALID_ARG;
  auto it = sv->all.find(request_id);
  if (it == sv->all.end()) return STQ_ERR_INVALID_ARG;
  const Request &r = *it->second;
  *steps_done = int(r.counts.size());
  for (int k = 0; k < *steps_done && k < max_steps; ++k) {
    if (counts) counts[k] = r.counts[size_t(k)];
    if (checksums) checksums[k] = r.checks[size_t(k)];
  }
  return STQ_OK;
}

int stq_server_request_ticks(stq_server *sv, int64_t request_id, int64_t *first_tick,
                             int64_t *last_tick) {
  if (!sv || !first_tick || !last_tick) return STQ_ERR_INVALID_ARG;
  auto it = sv->all.find(request_id);
  if (it == sv->all.end()) return STQ_ERR_INVALID_ARG;
  *first_tick = it->second->first_tick;
  *last_tick = it->second->last_tick;
  return STQ_OK;
}

int stq_server_mesh(stq_server *sv, int64_t request_id, double *h_V0, double *h_V1) {
  if (!sv || !h_V0 || !h_V1) return STQ_ERR_INVALID_ARG;
  auto it = sv->all.find(request_id);
  if (it == sv->all.end() || !it->second->dmem) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(sv->device);
  const Request &r = *it->second;
  STQ_CUDA(sv->ctx, cudaStreamSynchronize(sv->ctx->stream), "synchronise");
  STQ_CUDA(sv->ctx, cudaStreamSynchronize(sv->copy_stream), "synchronise uploads");
  const size_t bv = sizeof(double) * 3 * size_t(r.nV);
  STQ_CUDA(sv->ctx, cudaMemcpy(h_V0, r.dmem, bv, cudaMemcpyDeviceToHost), "read back V0");
  STQ_CUDA(sv->ctx, cudaMemcpy(h_V1, static_cast<char *>(r.dmem) + r.oV1, bv, cudaMemcpyDeviceToHost),
           "read back V1");
  return STQ_OK;
}

int stq_server_set_option(stq_server *sv, int option, int64_t value) {
  if (!sv) return STQ_ERR_INVALID_ARG;
  DeviceGuard g(sv->device);
  STQ_CUDA(sv->ctx, cudaStreamSynchronize(sv->ctx->stream), "synchronise");
  STQ_TRY(stq_context_set_option(sv->ctx, option, value));
  if (sv->graph) cudaGraphExecDestroy(sv->graph);
  sv->graph = nullptr;
  return STQ_OK;
}

int stq_server_stats(stq_server *sv, int64_t *active, int64_t *queued, int64_t *bytes, int64_t *ticks) {
  if (!sv) return STQ_ERR_INVALID_ARG;
  if (active) *active = int64_t(sv->active.size());
  if (queued) *queued = int64_t(sv->queue.size());
  if (bytes) *bytes = sv->fixed + sv->held;
  if (ticks) *ticks = sv->ticks;
  return STQ_OK;
}

}  // extern "C"
