/*
 * stq_abi.h - C ABI of the GB300 sweep-and-tiniest-queue (STQ) broad phase.
 *
 * Plain C: pointers, sizes and status codes only. Every pointer argument
 * named d_* is a device pointer on the context's device; h_* is host memory.
 * All work is enqueued on the context's stream. A call that returns a count
 * or a cursor to the host synchronises that stream before returning.
 *
 * Reference interfaces replaced (paths are within Ahdhn/broadphase-gpu):
 *   stq_aabb             <- stq::gpu::Aabb                src/aabb.cuh:15-43
 *   stq_build_boxes      <- stq::gpu::constructBoxes      src/io.cuh:9-13
 *                           (addVertices/addEdges/addFaces src/aabb.cu:193-304,
 *                            CPU twin src/cpu/aabb.cpp:7-95)
 *   stq_select_axis      <- calc_mean / calc_variance     src/sweep.cu:93-123
 *                           (axis choice, src/simulation.cu:594-637)
 *   stq_prepare          <- create_ds + thrust::sort_by_key
 *                           src/sweep.cu:125-161, src/simulation.cu:641-649
 *   stq_sweep_prepared   <- twostage_queue + add_overlap + the overflow loop
 *                           src/sweep.cu:226-279, src/collision.cu:50-74,
 *                           src/simulation.cu:690-747
 *   stq_sweep            <- stq::gpu::run_sweep_sharedqueue (device part)
 *                           src/simulation.cuh:22-27, src/simulation.cu:555-782
 *   stq_sweep_host       <- the same call with host boxes in and host pairs
 *                           out (H2D at simulation.cu:580, KEEP_CPU_OVERLAPS
 *                           copy-back at simulation.cu:763-780)
 *   stq_broadphase_host  <- constructBoxes + run_sweep_sharedqueue on host
 *                           meshes (app/main.cu:82-144)
 *   stq_context_*timing* <- CudaTimer / recordLaunch   src/timer.cuh:7-72
 *   stq_brute_force      <- get_collision_pairs (all-pairs checker)
 *                           src/collision.cu:91-154
 */
#ifndef STQ_ABI_H
#define STQ_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STQ_ABI_VERSION 1

/* Status codes. Negative values are errors; STQ_OVERFLOW is a partial result. */
typedef enum stq_status {
  STQ_OK = 0,
  /* The pairs of the requested start-box range did not fit in the caller's
   * buffer. The call wrote every pair of the longest prefix of start boxes
   * that fits, set *next_start to the first start box not yet swept and
   * *total to the pair count of the whole requested range. Call again from
   * *next_start (the reference's tidstart resume cursor). */
  STQ_OVERFLOW = 1,
  STQ_ERR_INVALID_ARG = -1,   /* null pointer, negative size, bad option     */
  STQ_ERR_INVALID_INPUT = -2, /* a box bound is NaN, or an index is out of range */
  STQ_ERR_CUDA = -3,          /* a CUDA runtime call failed (see last_error)  */
  STQ_ERR_NO_MEMORY = -4,     /* device or host allocation failed            */
  STQ_ERR_CAPACITY = -5,      /* one start box alone has more pairs than the buffer holds */
  STQ_ERR_TIMEOUT = -6,       /* a bounded device-side wait expired          */
  STQ_ERR_NOT_PREPARED = -7   /* stq_sweep_prepared without a prepared scene */
} stq_status;

/* Swept box, 44 bytes, field for field the reference's stq::gpu::Aabb
 * (src/aabb.cuh:15-43, Scalar = float): id, min, max, vertexIds, ref_id.
 * Box type is encoded in the signs of vertexIds (src/aabb.cu:12-40):
 *   vertex: {v, -v-1, -v-1}, edge: {e0, e1, -e0-1}, face: {f0, f1, f2}. */
typedef struct stq_aabb {
  int32_t id;
  float min[3];
  float max[3];
  int32_t vertex_ids[3];
  int32_t ref_id;
} stq_aabb;

/* One overlap, written as (smaller id, larger id). Layout of CUDA int2. */
typedef struct stq_pair {
  int32_t first;
  int32_t second;
} stq_pair;

/* Sweep axis. STQ_AXIS_AUTO picks the axis of largest box-corner variance. */
enum { STQ_AXIS_AUTO = -1, STQ_AXIS_X = 0, STQ_AXIS_Y = 1, STQ_AXIS_Z = 2 };

/* Tuning knobs for stq_context_set_option (0 restores the automatic choice). */
typedef enum stq_option {
  STQ_OPT_LANES_PER_ENTRY = 1, /* queue shape: lanes that share one queue entry:
                                  1 (default), 2, 4, 8, 16, 32                      */
  STQ_OPT_QUEUE_DEPTH = 2,     /* entries per warp queue: 16, 32, 64 (default) or
                                  128; with one lane per entry the queue holds at
                                  least 32 (16 acts as 32)                         */
  STQ_OPT_BLOCK_SIZE = 3,      /* sweep block size: 128, 256 (default) or 512     */
  STQ_OPT_CELLS = 4,           /* cell grid on the two non-sweep axes: 0 automatic,
                                  1 no cells (plain sweep), k > 1 a k x k grid      */
  STQ_OPT_RADIX_BITS = 5,      /* radix digit width: 4 or 8 (single-cell sort)     */
  STQ_OPT_CELL_SCALE = 6,      /* automatic cell side in median box extents (1..64,
                                  default 2); a scene of n boxes gets at most
                                  n / max(16, 8 * scale) cells                      */
  STQ_OPT_REPLICA_BUDGET = 7,  /* cell replicas per box a scene may use (1..64,
                                  default 4); finer grids beyond it are coarsened   */
  STQ_OPT_GRAPH = 8,           /* stq_batch_broadphase: 1 capture and replay a CUDA
                                  graph (default), 2 plain stream launches          */
  STQ_OPT_HOST_OVERLAP = 9,    /* stq_sweep_host / stq_broadphase_host: 1 sweep in
                                  windows, each window's pairs copied to the host
                                  while the next is swept (default), 2 one copy
                                  after the whole sweep                            */
  STQ_OPT_CANDIDATES_PER_LANE = 10, /* with one lane per entry: candidates a lane
                                  tests per step, 1, 2, 4 or 8 (default); with the
                                  flat shape: steps of 32 candidates whose loads
                                  are issued together, 2 or 4 (default 8 acts as 4) */
  STQ_OPT_RUN_CAP = 11,        /* candidates of one start box a lane (group) tests
                                  before a whole warp takes over the rest of its
                                  run (1..2^20, default 512)                      */
  STQ_OPT_HOST_WINDOWS = 12,   /* stq_sweep_host / stq_broadphase_host: windows a
                                  sweep is cut into (2..32, default 16; fewer when
                                  the scene has under 2^19 positions per window) */
  STQ_OPT_SWEEP_SHAPE = 13     /* 2 (default): flat, each warp lays the runs of 32
                                  start boxes end to end and tests one candidate
                                  per lane and step (block size 128 or 256; 512
                                  acts as 256); 1: a per-warp queue of pending
                                  start boxes taken by lanes or lane groups
                                  (STQ_OPT_LANES_PER_ENTRY, STQ_OPT_QUEUE_DEPTH)  */
} stq_option;

typedef struct stq_context stq_context;

int stq_abi_version(void);
const char *stq_status_string(int status);

/* Creates a context bound to `device` and `stream` (a cudaStream_t; NULL =
 * the legacy default stream). The context owns a grow-only device arena. */
int stq_context_create(int device, void *stream, stq_context **out);
void stq_context_destroy(stq_context *ctx);
int stq_context_set_stream(stq_context *ctx, void *stream);
int stq_context_set_option(stq_context *ctx, int option, int64_t value);
int64_t stq_context_get_option(const stq_context *ctx, int option);
const char *stq_context_last_error(const stq_context *ctx);
/* Kernel launches this context issued since it was created. */
int64_t stq_context_launch_count(const stq_context *ctx);
/* Candidates (x-overlapping start box / candidate pairs) the last sweep
 * tested, a measure of the sweep's work beyond the pairs it found. */
int64_t stq_context_candidates(const stq_context *ctx);
/* Shape of the prepared scene's (cell, type) lists: out[0] lists (3 per
 * cell), out[1] cell replicas, out[2] the longest list. Synchronises. */
int stq_context_list_stats(stq_context *ctx, int64_t out[3]);

/* Swept boxes from vertex trajectories. d_V0/d_V1 are row-major [nV x 3]
 * fp64 positions at t0 and t1, d_E [nE x 2] and d_F [nF x 3] int32 vertex
 * indices. Writes nV + nE + nF boxes in id order (vertices, edges, faces):
 * per coordinate, min over the trajectory points in fp64, rounded to float,
 * moved one ulp outward, then widened by nextafter_up(inflation_radius). */
int stq_build_boxes(stq_context *ctx, const double *d_V0, const double *d_V1,
                    int64_t nV, const int32_t *d_E, int64_t nE,
                    const int32_t *d_F, int64_t nF, float inflation_radius,
                    stq_aabb *d_boxes);

/* Axis of largest variance of the box corners (0, 1 or 2). Reuses the batch
 * buffers: a previously prepared scene must be prepared again. */
int stq_select_axis(stq_context *ctx, const stq_aabb *d_boxes, int64_t n,
                    int *axis_out);

/* Sorts the boxes along `axis` into the context's sorted scene (keys,
 * bounds, vertex ids). The boxes buffer may be reused after return. */
int stq_prepare(stq_context *ctx, const stq_aabb *d_boxes, int64_t n,
                int axis);

/* Number of sweep positions of the prepared scene: the start-box cursor of
 * stq_sweep_prepared runs over [0, length). Boxes are replicated into the
 * cells they touch (one cell when STQ_OPT_CELLS = 1); every cell holds a
 * vertex, an edge and a face list, each followed by one empty position, so
 * length = replicas + 3 * cells - 1 (n + 2 with one cell; 0 with no boxes).
 * -1 if nothing is prepared. */
int64_t stq_prepared_length(const stq_context *ctx);

/* Sweeps start boxes [start, start + max_start) of the prepared scene in
 * sorted order (max_start <= 0 means all). Every overlapping pair whose
 * earlier box lies in that range is written once to d_pairs as
 * (smaller id, larger id), in no particular order. *count = pairs written,
 * *next_start = first start box not swept, *total (may be NULL) = pairs of
 * the whole range. Returns STQ_OK or STQ_OVERFLOW (see above). */
int stq_sweep_prepared(stq_context *ctx, int64_t start, int64_t max_start,
                       stq_pair *d_pairs, int64_t capacity, int64_t *count,
                       int64_t *next_start, int64_t *total);

/* stq_prepare + stq_sweep_prepared in one call. */
int stq_sweep(stq_context *ctx, const stq_aabb *d_boxes, int64_t n, int axis,
              int64_t start, int64_t max_start, stq_pair *d_pairs,
              int64_t capacity, int64_t *count, int64_t *next_start,
              int64_t *total);

/* End-to-end call on host memory: copies h_boxes to the device, sweeps all
 * start boxes, copies the pairs back to h_pairs (capacity entries). Same
 * return codes as stq_sweep; on STQ_OVERFLOW h_pairs holds the prefix.
 * Scenes of 2^20 or more sweep positions are swept in windows of start
 * positions, two at a time on two streams; each window's pairs are copied to
 * h_pairs on a third stream while later windows are swept
 * (STQ_OPT_HOST_OVERLAP = 2: one copy after the sweep). A page-locked h_pairs (cudaHostAlloc / cudaHostRegister) lets those
 * copies run asynchronously. The same holds for stq_broadphase_host. */
int stq_sweep_host(stq_context *ctx, const stq_aabb *h_boxes, int64_t n,
                   int axis, stq_pair *h_pairs, int64_t capacity,
                   int64_t *count, int64_t *total);

/* End-to-end call on a host mesh: copies V0/V1 ([nV x 3] fp64), E and F
 * (int32) to the device, builds the swept boxes, sweeps every start box and
 * copies the pairs back to h_pairs (capacity entries). The reference path
 * this replaces is constructBoxes on the host followed by
 * run_sweep_sharedqueue with KEEP_CPU_OVERLAPS (app/main.cu:83-144). */
int stq_broadphase_host(stq_context *ctx, const double *h_V0, const double *h_V1,
                        int64_t nV, const int32_t *h_E, int64_t nE,
                        const int32_t *h_F, int64_t nF, float inflation_radius,
                        int axis, stq_pair *h_pairs, int64_t capacity,
                        int64_t *count, int64_t *total);

/* Per-stage device timers (CUDA events on the context's stream; replaces
 * the reference's CudaTimer / recordLaunch, src/timer.cuh:7-72). Stages:
 * 0 build, 1 axis, 2 keys, 3 sort, 4 gather, 5 sweep, 6 count sweep,
 * 7 pair sort. stq_context_stage_times fills up to max_stages entries of
 * accumulated milliseconds and call counts and returns the stage count. */
int stq_context_enable_timing(stq_context *ctx, int enable);
int stq_context_stage_times(stq_context *ctx, double *ms, int64_t *calls,
                            int max_stages);
const char *stq_stage_name(int stage);

/* ---- batches of scenes (one launch sequence for many scenes) ----------------
 * Scene s owns boxes [box_off[s], box_off[s+1]) of one box array. Every scene
 * gets its own sweep axis and cell grid; cells of all scenes are sorted and
 * swept together, and no pair crosses scenes. Pair ids are the boxes' `id`
 * fields (batch-global when the boxes come from stq_batch_build_boxes). */

/* Swept boxes of a batch of meshes. Scene s has vertices [h_vert_off[s],
 * h_vert_off[s+1]) of d_V0/d_V1, edges [h_edge_off[s], ...) of d_E and faces
 * [h_face_off[s], ...) of d_F, with vertex indices local to the scene. Boxes
 * are written scene after scene (vertices, edges, faces of each); a box's id
 * is its batch index, its vertex ids are local. h_box_off receives the
 * n_scenes + 1 box offsets. Reuses the batch buffers: a previously prepared
 * scene must be prepared again. */
int stq_batch_build_boxes(stq_context *ctx, const double *d_V0, const double *d_V1,
                          const int64_t *h_vert_off, const int32_t *d_E,
                          const int64_t *h_edge_off, const int32_t *d_F,
                          const int64_t *h_face_off, int n_scenes,
                          float inflation_radius, stq_aabb *d_boxes,
                          int64_t *h_box_off);

/* Prepares a batch (h_axis: n_scenes axes, or NULL for one `axis` for all);
 * stq_sweep_prepared then sweeps every scene of it. */
int stq_batch_prepare(stq_context *ctx, const stq_aabb *d_boxes,
                      const int64_t *h_box_off, int n_scenes, const int *h_axis,
                      int axis);

/* Pairs per scene found by the last sweep (n_scenes entries). */
int stq_batch_scene_pairs(stq_context *ctx, int64_t *h_counts, int n_scenes);

/* The whole batched pipeline on device meshes (build, prepare, sweep of all
 * start boxes) with no host synchronisation until the end. With
 * STQ_OPT_GRAPH = 1 the launch sequence is captured once as a CUDA graph and
 * replayed for any later batch that fits the same capacities and buffers.
 * Writes the pairs to d_pairs; *count = pairs written; h_scene_pairs (may be
 * NULL) receives per-scene counts. STQ_OVERFLOW: more pairs than capacity
 * (the first capacity pairs are written; call again with a larger buffer). */
int stq_batch_broadphase(stq_context *ctx, const double *d_V0, const double *d_V1,
                         const int64_t *h_vert_off, const int32_t *d_E,
                         const int64_t *h_edge_off, const int32_t *d_F,
                         const int64_t *h_face_off, int n_scenes,
                         float inflation_radius, int axis, stq_pair *d_pairs,
                         int64_t capacity, int64_t *count, int64_t *total,
                         int64_t *h_scene_pairs);

/* Sorts d_pairs[0..count) lexicographically on the device (deterministic
 * output order for callers that need one). */
int stq_sort_pairs(stq_context *ctx, stq_pair *d_pairs, int64_t count);

/* ---- autotuning --------------------------------------------------------------
 * Times prepare + sweep of the given batch (as stq_batch_prepare, all start
 * boxes), each setting five times (the fastest counts), over cell scale
 * {1, 2, 4, 8} and radix digit width {4, 8} (the prepare), and over the sweep
 * shapes (the work split of the start boxes' runs): one start box per lane
 * with 2, 4 or 8 candidates per step (queue depth {32, 64}), lane groups of
 * 4, 8 or 16 lanes (queue depth {16, 32, 64}), each with block size
 * {128, 256, 512}, and the flat shape with 2 or 4 filter steps per round,
 * block size {128, 256} and run cap {512, 4096} (the run length past which the
 * warp pass takes a run over). Keeps the fastest prepare + sweep as the
 * context's options (cell scale, radix width, sweep shape, lanes per entry,
 * candidates per lane, queue depth, block size, run cap). Settings are cached
 * per shape bucket
 * (log2 of the box count, log2 of the scene count): a later call whose batch
 * falls in a tuned bucket applies them without timing. *best_ms receives the
 * prepare + sweep time of the chosen settings (0 on a cache hit). The batch is
 * left prepared. Replaces the reference's fixed launch setup (src/util.cu:9-56). */
int stq_autotune(stq_context *ctx, const stq_aabb *d_boxes, const int64_t *h_box_off,
                 int n_scenes, stq_pair *d_pairs, int64_t capacity, double *best_ms);

/* ---- serving: continuous batching of time-stepped requests ------------------
 * No single counterpart in the reference (its apps run one scene per
 * process); each tick runs the batched pipeline above over the current
 * timestep of every admitted request. A request is a mesh (host memory,
 * copied at submit) run for `steps` timesteps: step 0 sweeps the given
 * trajectories, every later step first sets t0 <- t1 and t1 <- t1 + N(0,
 * sigma^2) per coordinate on the device (counter-based generator seeded by
 * `seed`), so the scene stays in HBM between steps. Requests are admitted
 * first come, first served while they fit the HBM budget (mesh + estimated
 * pair buffer), the box capacity of one launch and the scene capacity.
 * Uploads of newly admitted requests overlap the launch in flight. */
typedef struct stq_server stq_server;

int stq_server_create(int device, void *stream, int64_t budget_bytes, int64_t max_boxes,
                      int max_scenes, stq_server **out);
void stq_server_destroy(stq_server *server);
int stq_server_submit(stq_server *server, const double *h_V0, const double *h_V1, int64_t nV,
                      const int32_t *h_E, int64_t nE, const int32_t *h_F, int64_t nF, int steps,
                      double sigma, uint64_t seed, int64_t *request_id);
/* Collects the launch in flight, retires finished requests (their ids go to
 * done_ids, up to max_done; *n_done = how many finished), admits queued
 * requests and launches the next tick without waiting for it. */
int stq_server_tick(stq_server *server, int64_t *done_ids, int max_done, int *n_done);
/* Per-timestep results of a request: pair count and the XOR over its pairs
 * of splitmix64((lo << 32) | hi) with ids local to the request's mesh. */
int stq_server_result(stq_server *server, int64_t request_id, int64_t *counts,
                      uint64_t *checksums, int max_steps, int *steps_done);
/* Ticks of a request: the index (0-based, in launch order) of the tick that
 * ran its first timestep and of the one that ran its last; -1 until then. */
int stq_server_request_ticks(stq_server *server, int64_t request_id, int64_t *first_tick,
                             int64_t *last_tick);
/* Current positions of an active request (t0 and t1 of its last step). */
int stq_server_mesh(stq_server *server, int64_t request_id, double *h_V0, double *h_V1);
/* active, queued, bytes held for admitted requests, ticks launched */
int stq_server_stats(stq_server *server, int64_t *active, int64_t *queued, int64_t *bytes,
                     int64_t *ticks);
/* stq_context_set_option on the server's pipeline; the next tick captures
 * its launch sequence again with the new setting. */
int stq_server_set_option(stq_server *server, int option, int64_t value);

/* ---- sweep without any allocation -----------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory when they need a broad phase: simulation steps that must stay within
 * memory reserved up front (an out-of-memory error in mid-step is not
 * recoverable for them), hosts whose own pooling allocator owns the device
 * memory and forbids the CUDA runtime's, and real-time loops that cannot take
 * the device-wide synchronisation cudaFree may cause. It sorts and sweeps one
 * scene (no cells) along `axis` (0, 1 or 2) on `stream` using only a scratch
 * array of about 4.5 MB that is static in this library: every GPU that loads
 * the library holds it until the process exits, and it keeps the last call's
 * contents (each call clears what must start at zero). No context, no
 * cudaMalloc, no cudaFree.
 *   - n above STQ_STATIC_MAX_BOXES is rejected with STQ_ERR_CAPACITY before
 *     any GPU work (use stq_sweep for larger scenes);
 *   - the first call on a device looks up the scratch array's device address
 *     (with that device current); make that first call before any stream
 *     capture begins;
 *   - all calls on a device share the array: calls that overlap on the GPU
 *     (other streams, other host threads) race and must be serialised;
 *   - pairs as stq_sweep; *count = pairs written, *total (may be NULL) = pairs
 *     found; STQ_OVERFLOW if they did not all fit (no resume cursor);
 *     STQ_ERR_INVALID_INPUT if a bound is NaN.
 * The call synchronises `stream` before returning. */
#define STQ_STATIC_MAX_BOXES 65536
int stq_sweep_static(const stq_aabb *d_boxes, int64_t n, int axis, stq_pair *d_pairs,
                     int64_t capacity, int64_t *count, int64_t *total, void *stream);

/* All-pairs checker, O(n^2): same filter and output form as the sweep.
 * Meant for small n (cross-checks). */
int stq_brute_force(stq_context *ctx, const stq_aabb *d_boxes, int64_t n,
                    stq_pair *d_pairs, int64_t capacity, int64_t *count);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* STQ_ABI_H */
