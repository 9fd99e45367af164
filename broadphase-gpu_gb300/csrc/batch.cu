// batch.cu - prepare kernels of the scene table: per-scene statistics, sweep
// axis and cell grid, cell replicas with their sort keys, and the sorted-scene
// gather with one NaN sentinel after every cell.
//
// Reference: create_ds (src/sweep.cu:125-161) and the axis choice of
// calc_mean / calc_variance (src/sweep.cu:93-123); the reference sorts one
// scene along x. Here every scene of a batch gets its own sweep axis and
// y/z cell grid, all scenes' cells get global ids, and one sort orders every
// replica by (cell, min on the sweep axis).
//
// All sizes are read from the BatchHeader on the device, so one captured
// graph serves any batch within the buffer capacities.
#include <mutex>
#include <utility>
#include <vector>

#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {

namespace {

constexpr int kBlock = 256;
constexpr int kHistBias = 40;  // extent bucket = binary exponent + 40
constexpr int kSampleBoxes = 1024;

__device__ __forceinline__ float key_float(uint32_t k) {
  const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(b);
}

__device__ __forceinline__ void axes_bc(int a, int &b, int &c) {
  b = a == 0 ? 1 : 0;
  c = a == 2 ? 1 : 2;
}

// Block sums of K values per thread with one shared-memory exchange; out[k]
// is valid in thread 0.
template <typename T, int K>
__device__ void block_sums(const T (&v)[K], T (&out)[K], T (*red)[K]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    T x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFullMask, x, o);
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      T t = 0;
      for (int w = 0; w < kBlock / 32; ++w) t += red[w][k];
      out[k] = t;
    }
  }
}

// ---- 0. reset the per-scene accumulators ------------------------------------------
__global__ void __launch_bounds__(kBlock)
batch_reset_kernel(SceneRecord *scenes, const SceneInput *__restrict__ inputs,
                   unsigned long long *scene_pairs, BatchHeader *hdr) {
  const int S = hdr->n_scenes;
  for (int s = blockIdx.x * kBlock + threadIdx.x; s < S; s += gridDim.x * kBlock) {
    SceneRecord &r = scenes[s];
    r.axis_mode = inputs[s].axis_mode;
    r.cells_opt = inputs[s].cells_opt;
    r.cell_scale = inputs[s].cell_scale;
    scene_pairs[s] = 0ull;
    for (int k = 0; k < 3; ++k) {
      r.s1[k] = 0.0;
      r.s2[k] = 0.0;
      r.lo_key[k] = 0xffffffffu;
      r.hi_key[k] = 0u;
    }
    r.inverted = 0;
    for (int l = 0; l < kGridLevels; ++l) r.level_reps[l] = 0ull;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hdr->flags = 0;
    hdr->replicas = 0;
    hdr->cells = 0;
    hdr->lists = 0;
    hdr->length = 0;
    hdr->work = 0;
    hdr->pairs = 0;
    hdr->prefix = 0;
  }
}

// ---- 1. statistics: one tile (one scene) per block ------------------------------
__global__ void __launch_bounds__(kBlock)
batch_stats_kernel(const stq_aabb *__restrict__ boxes, const TileRec *__restrict__ tiles,
                   SceneRecord *scenes, BatchHeader *hdr) {
  if (int(blockIdx.x) >= hdr->n_tiles) return;
  const TileRec t = tiles[blockIdx.x];
  // moments about the tile's first box centre, in fp32 per thread (fp64 is
  // slow on this part); the block combines them in fp64 and shifts them back
  float c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float m = 0.5f * (boxes[t.begin].min[k] + boxes[t.begin].max[k]);
    c[k] = isfinite(m) ? m : 0.f;
  }
  float s1[3] = {0.f, 0.f, 0.f}, s2[3] = {0.f, 0.f, 0.f};
  uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  bool inverted = false, nan = false;
  // thread i takes boxes i, i + kBlock, ...: each warp load instruction covers
  // 32 consecutive boxes, and the unrolled loop keeps several boxes in flight
  const stq_aabb *tb = boxes + t.begin;
#pragma unroll 4
  for (int i = threadIdx.x; i < t.count; i += kBlock) {
    const stq_aabb &x = tb[i];
    float l[3], h[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) l[k] = x.min[k], h[k] = x.max[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      nan |= (l[k] != l[k]) | (h[k] != h[k]);
      inverted |= l[k] > h[k];
      const float dl = l[k] - c[k], dh = h[k] - c[k];
      s1[k] += dl + dh;
      s2[k] += dl * dl + dh * dh;
      lo[k] = min(lo[k], float_key(l[k]));
      hi[k] = max(hi[k], float_key(h[k]));
    }
  }
  // warp sums in fp32 (a fixed shuffle tree); the 8 warp sums of each moment
  // are combined in fp64 by one lane each, and each value reaches the scene
  // record with one atomic per block (fp64 and same-address atomics are slow)
  constexpr int kWarps = kBlock / 32;
  __shared__ float wsum[6][kWarps];
  __shared__ uint32_t wkey[6][kWarps];
  __shared__ int wflag[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float m[6] = {s1[0], s1[1], s1[2], s2[0], s2[1], s2[2]};
#pragma unroll
  for (int k = 0; k < 6; ++k)
    for (int o = 16; o > 0; o >>= 1) m[k] += __shfl_down_sync(kFullMask, m[k], o);
  uint32_t kk[6];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    kk[k] = __reduce_min_sync(kFullMask, lo[k]);
    kk[3 + k] = __reduce_max_sync(kFullMask, hi[k]);
  }
  const int fl = (__any_sync(kFullMask, inverted) ? 1 : 0) | (__any_sync(kFullMask, nan) ? 2 : 0);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 6; ++k) wsum[k][warp] = m[k], wkey[k][warp] = kk[k];
    wflag[warp] = fl;
  }
  __syncthreads();
  if (warp != 0) return;
  SceneRecord &r = scenes[t.scene];
  double tot = 0.0;  // lane k < 6: moment k of the block
  uint32_t key = lane < 3 ? 0xffffffffu : 0u;  // lanes 0-2 minima, 3-5 maxima
  int flags = 0;
  if (lane < 6) {
    for (int w = 0; w < kWarps; ++w) {
      tot += double(wsum[lane][w]);
      key = lane < 3 ? min(key, wkey[lane][w]) : max(key, wkey[lane][w]);
      flags |= wflag[w];
    }
  }
  // sum(l + h) = S1 + 2 n c; sum(l^2 + h^2) = S2 + 2 c S1 + 2 n c^2
  const double a1 = __shfl_sync(kFullMask, tot, lane < 3 ? lane : lane - 3);
  if (lane < 6) {
    const int k = lane < 3 ? lane : lane - 3;
    const double ck = k == 0 ? c[0] : (k == 1 ? c[1] : c[2]), n = double(t.count);
    if (lane < 3) {
      atomicAdd(&r.s1[k], tot + 2.0 * n * ck);
      atomicMin(&r.lo_key[k], key);
    } else {
      atomicAdd(&r.s2[k], tot + 2.0 * ck * a1 + 2.0 * n * ck * ck);
      atomicMax(&r.hi_key[k], key);
    }
  }
  if (lane == 0 && (flags & 1)) atomicOr(&r.inverted, 1);
  if (lane == 0 && (flags & 2)) atomicOr(&hdr->flags, kFlagNaN);
}

__device__ int grid_side(float L, float h) {
  if (!(L > 0.f) || !(h > 0.f) || !isfinite(L)) return 1;
  const float s = ceilf(L / h);
  return s > float(kMaxGridSide) ? kMaxGridSide : (s < 1.f ? 1 : int(s));
}

__device__ __forceinline__ float inv_side(int n, float L) { return n > 1 ? float(n) / L : 0.f; }

// ---- 2. policy: one block per scene ---------------------------------------------
// Sweep axis of largest corner variance (x, then y, preferred on ties, as
// src/simulation.cu:630-635) unless fixed; level-0 cell side = cell_scale x
// median box extent (from a strided sample of the scene's boxes), at most
// 2048 cells per axis and at most max(1, n / max(16, 8 x cell_scale)) cells.
__global__ void __launch_bounds__(kBlock)
batch_policy_kernel(const stq_aabb *__restrict__ boxes, const long long *__restrict__ box_off,
                    SceneRecord *scenes, BatchHeader *hdr) {
  const int s = blockIdx.x;
  if (s >= hdr->n_scenes) return;
  SceneRecord &r = scenes[s];
  const long long b0 = box_off[s], n = box_off[s + 1] - b0;
  int axis = r.axis_mode;
  if (axis < 0) {
    double var[3];
    const double m = n > 0 ? 2.0 * double(n) : 1.0;
    for (int k = 0; k < 3; ++k) {
      const double mean = r.s1[k] / m;
      var[k] = r.s2[k] - m * mean * mean;
    }
    axis = 0;
    if (var[1] > var[axis]) axis = 1;
    if (var[2] > var[axis]) axis = 2;
  }
  int b, c;
  axes_bc(axis, b, c);
  __shared__ unsigned hist[2][64];
  for (int i = threadIdx.x; i < 128; i += kBlock) (&hist[0][0])[i] = 0u;
  __syncthreads();
  const bool automatic = r.cells_opt == 0 && !r.inverted && n > 1;
  if (automatic) {
    const long long step = n > kSampleBoxes ? n / kSampleBoxes : 1;
    for (long long i = threadIdx.x; i < kSampleBoxes && i * step < n; i += kBlock) {
      const stq_aabb &x = boxes[b0 + i * step];
      const int ax[2] = {b, c};
      for (int q = 0; q < 2; ++q) {
        const float ext = x.max[ax[q]] - x.min[ax[q]];
        int bucket = 0;
        if (ext > 0.f) {
          int e;
          frexpf(ext, &e);
          bucket = min(63, max(1, e + kHistBias));
        }
        atomicAdd(&hist[q][bucket], 1u);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const float lob = key_float(r.lo_key[b]), hib = key_float(r.hi_key[b]);
  const float loc = key_float(r.lo_key[c]), hic = key_float(r.hi_key[c]);
  const float Lb = hib - lob, Lc = hic - loc;
  int nb = 1, nc = 1;
  if (r.cells_opt > 1 && !r.inverted && n > 1) {
    nb = nc = r.cells_opt;
  } else if (automatic) {
    float w[2];
    for (int q = 0; q < 2; ++q) {
      unsigned total = 0, run = 0;
      for (int k = 0; k < 64; ++k) total += hist[q][k];
      w[q] = 0.f;
      for (int k = 0; k < 64; ++k) {
        run += hist[q][k];
        if (2 * run >= total && total > 0) {
          w[q] = k == 0 ? 0.f : 0.75f * exp2f(float(k - kHistBias));
          break;
        }
      }
    }
    if (!(w[0] > 0.f)) w[0] = Lb / 1024.f;
    if (!(w[1] > 0.f)) w[1] = Lc / 1024.f;
    nb = grid_side(Lb, r.cell_scale * w[0]);
    nc = grid_side(Lc, r.cell_scale * w[1]);
    // at least max(16, 8 * scale) boxes per cell on average: dense scenes of
    // small boxes would otherwise be cut into lists of a few boxes, and their
    // prepare would outweigh the sweep (the buffers are sized for n / 16 cells)
    const long long per_cell = max(16ll, (long long)(8.f * r.cell_scale));
    const long long max_cells = max(1ll, min(1ll << 20, n / per_cell));
    while ((long long)nb * nc > max_cells) {
      if (nb >= nc) nb = (nb + 1) / 2;
      else nc = (nc + 1) / 2;
    }
  }
  if (!(Lb > 0.f) || !isfinite(Lb)) nb = 1;
  if (!(Lc > 0.f) || !isfinite(Lc)) nc = 1;
  GridParams &g = r.grid;
  g.axis = axis;
  g.ob = lob;
  g.oc = loc;
  g.Lb = Lb;
  g.Lc = Lc;
  g.ib = inv_side(nb, Lb);
  g.ic = inv_side(nc, Lc);
  g.nb0 = g.ib == 0.f ? 1 : nb;
  g.nc0 = g.ic == 0.f ? 1 : nc;
  if (s == 0) hdr->axis = axis;
}

struct Range {
  int b0, b1, c0, c1;
};

__device__ __forceinline__ Range cell_range(const stq_aabb &x, int a, float ob, float ib, int nb,
                                            float oc, float ic, int nc) {
  int b, c;
  axes_bc(a, b, c);
  Range r;
  r.b0 = cell_coord(x.min[b], ob, ib, nb);
  r.b1 = cell_coord(x.max[b], ob, ib, nb);
  r.c0 = cell_coord(x.min[c], oc, ic, nc);
  r.c1 = cell_coord(x.max[c], oc, ic, nc);
  return r;
}

// Scene of box bi: the last scene whose first box is <= bi.
__device__ __forceinline__ int scene_of(const long long *__restrict__ box_off, int S, uint32_t bi) {
  int lo = 0, hi = S - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (box_off[mid] <= (long long)bi) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ---- 4. choose the finest level within the replica budget; cell bases ----------
__global__ void __launch_bounds__(1024)
batch_choose_kernel(const long long *__restrict__ box_off, SceneRecord *scenes,
                    unsigned int *cell_base, BatchHeader *hdr) {
  __shared__ unsigned int warp_tot[32];
  __shared__ unsigned int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int S = hdr->n_scenes;
  const long long budget = hdr->budget;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < S; base += 1024) {
    const int s = base + threadIdx.x;
    unsigned int cells = 0;
    if (s < S) {
      SceneRecord &r = scenes[s];
      const long long n = box_off[s + 1] - box_off[s];
      int level = kCoordBits;  // none fits: every coordinate shifts to cell 0
      if (r.cells_opt > 1) {
        level = 0;  // a requested grid is kept as is
      } else {
        for (int l = 0; l < kGridLevels; ++l)
          if ((long long)r.level_reps[l] <= budget * n) {
            level = l;
            break;
          }
      }
      GridParams &g = r.grid;
      g.shift = level;
      g.nb = ((g.nb0 - 1) >> level) + 1;
      g.nc = ((g.nc0 - 1) >> level) + 1;
      g.ncells = g.nb * g.nc;
      cells = unsigned(g.ncells);
    }
    // block exclusive scan of the cell counts
    unsigned int x = cells;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int y = __shfl_up_sync(kFullMask, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned int w = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(kFullMask, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const unsigned int excl = carry + (warp > 0 ? warp_tot[warp - 1] : 0u) + x - cells;
    if (s < S) cell_base[s] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cell_base[S] = carry;
    hdr->cells = carry;
    hdr->lists = 3u * carry;
  }
}

// ---- 5. per-box replica counts in sweep-axis order (zero past the last box, up
// to the capacity), from the level-0 cell ranges by box index that the
// box-key kernel wrote, at the scene's chosen level
__device__ __forceinline__ uint32_t cells_count(uint2 r, int shift) {
  return (((r.x >> 11 & 2047u) >> shift) - ((r.x & 2047u) >> shift) + 1u) *
         (((r.y >> 11 & 2047u) >> shift) - ((r.y & 2047u) >> shift) + 1u);
}

__global__ void __launch_bounds__(kBlock)
batch_count_kernel(const uint32_t *__restrict__ order, const uint2 *__restrict__ box_cells,
                   const long long *__restrict__ box_off, const SceneRecord *__restrict__ scenes,
                   const BatchHeader *hdr, uint32_t *__restrict__ counts, long long box_cap) {
  const long long N = hdr->n_boxes;
  const int S = hdr->n_scenes;
  for (long long p = blockIdx.x * (long long)kBlock + threadIdx.x; p < N; p += (long long)gridDim.x * kBlock) {
    const uint32_t bi = order[p];
    counts[p] = cells_count(box_cells[bi], scenes[scene_of(box_off, S, bi)].grid.shift);
  }
  // positions past the batch contribute nothing to the scan
  for (long long i = N + blockIdx.x * (long long)kBlock + threadIdx.x; i < box_cap;
       i += (long long)gridDim.x * kBlock)
    counts[i] = 0u;
}

// ---- 6. replica keys: (segment << 32) | order-preserving min, where the
// segment is (global cell, box type): every cell holds a vertex, an edge and
// a face list.
__global__ void __launch_bounds__(kBlock)
batch_emit_kernel(const uint2 *__restrict__ box_cells, const uint32_t *__restrict__ sorted_keys,
                  const uint32_t *__restrict__ order,
                  const long long *__restrict__ box_off, const SceneRecord *__restrict__ scenes,
                  const unsigned int *__restrict__ cell_base, BatchHeader *hdr,
                  const uint32_t *__restrict__ offsets, unsigned long long *__restrict__ keys,
                  uint32_t *__restrict__ vals, long long rep_cap, long long seg_cap) {
  const bool fits = (long long)hdr->replicas <= rep_cap && 3ll * hdr->cells <= seg_cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // each of the 3 lists of a cell is followed by its sentinel; the last
    // sentinel is not a start position. On overflow nothing is emitted.
    hdr->length = fits && hdr->cells > 0 && hdr->replicas > 0 ? hdr->replicas + 3 * hdr->cells - 1 : 0u;
    hdr->max_list = 0u;
    if (!fits) {
      atomicOr(&hdr->flags, kFlagReplicaOverflow);
      hdr->replicas = 0;
    }
  }
  if (!fits) return;
  const long long N = hdr->n_boxes;
  const int S = hdr->n_scenes;
  // positions in sweep-axis order: every list receives its replicas in key
  // order, which the stable sort by list id keeps
  for (long long p = blockIdx.x * (long long)kBlock + threadIdx.x; p < N; p += (long long)gridDim.x * kBlock) {
    const uint32_t bi = order[p];
    const int sc = scene_of(box_off, S, bi);
    const int nc = scenes[sc].grid.nc, sh = scenes[sc].grid.shift;
    const unsigned long long cb0 = cell_base[sc];
    // the box's level-0 cell range and type (8 bytes, by box index) and its
    // sort key, instead of the 44-byte box
    const uint2 r = box_cells[bi];
    const int b0 = int(r.x & 2047u) >> sh, b1 = int(r.x >> 11 & 2047u) >> sh;
    const int c0 = int(r.y & 2047u) >> sh, c1 = int(r.y >> 11 & 2047u) >> sh;
    const unsigned long long type = r.x >> 22;
    const unsigned long long xk = sorted_keys[p];
    uint32_t o = offsets[p];
    for (int cb = b0; cb <= b1; ++cb)
      for (int cc = c0; cc <= c1; ++cc) {
        const unsigned long long seg = (cb0 + (unsigned long long)(cb * nc + cc)) * 3ull + type;
        keys[o] = (seg << 32) | xk;
        vals[o] = bi;
        ++o;
      }
  }
}

// ---- 3. sort keys of the boxes (the order-preserving image of the minimum on
// the scene's sweep axis, with the box index as value), each box's level-0
// cell range and type, and the replicas of every grid level, per scene
__global__ void __launch_bounds__(kBlock)
batch_box_keys_kernel(const stq_aabb *__restrict__ boxes, const TileRec *__restrict__ tiles,
                      SceneRecord *scenes, const BatchHeader *hdr,
                      uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, uint2 *__restrict__ box_cells) {
  if (int(blockIdx.x) >= hdr->n_tiles) return;
  const TileRec t = tiles[blockIdx.x];
  SceneRecord &r = scenes[t.scene];
  const GridParams g = r.grid;
  // a thread sees at most kTileBoxes / kBlock = 16 boxes of at most 2048^2
  // cells each: 32-bit sums per thread, 64-bit per block
  static_assert(uint64_t(kTileBoxes / kBlock) * kMaxGridSide * kMaxGridSide < (uint64_t(1) << 32),
                "per-thread level sums");
  unsigned reps[kGridLevels] = {};
  for (int i = threadIdx.x; i < t.count; i += kBlock) {
    const long long bi = t.begin + i;
    const stq_aabb &x = boxes[bi];
    keys[bi] = float_key(x.min[g.axis]);
    vals[bi] = uint32_t(bi);
    // the box's cell range and type, by box index, while the box is read in
    // order (level-0 coordinates fit kCoordBits = 11 bits)
    const Range q = cell_range(x, g.axis, g.ob, g.ib, g.nb0, g.oc, g.ic, g.nc0);
    const unsigned type = unsigned(type_of(x.vertex_ids[1], x.vertex_ids[2]));
    box_cells[bi] = make_uint2(unsigned(q.b0) | unsigned(q.b1) << 11 | type << 22,
                               unsigned(q.c0) | unsigned(q.c1) << 11);
#pragma unroll
    for (int l = 0; l < kGridLevels; ++l)
      reps[l] += unsigned((q.b1 >> l) - (q.b0 >> l) + 1) * unsigned((q.c1 >> l) - (q.c0 >> l) + 1);
  }
  __shared__ unsigned long long red[kBlock / 32][kGridLevels];
  unsigned long long wide[kGridLevels], tot[kGridLevels];
#pragma unroll
  for (int l = 0; l < kGridLevels; ++l) wide[l] = reps[l];
  block_sums(wide, tot, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int l = 0; l < kGridLevels; ++l) atomicAdd(&r.level_reps[l], tot[l]);
}

// First position of every (cell, type) list in the sorted replicas, and one
// entry past the last (the replica count): the keys are sorted by list id, so
// each offset is the lower bound of its id. Sorted replica p of list s sits at
// position p + s, so list s ends at position offset[s + 1] + s: the slot after
// it gets the NaN sentinel (NaN bounds end every run there; its partner is
// itself, so the sweep's refill test of a sentinel reads inside the scene and
// fails), and so do kSortedPad slots of padding after the last list. The
// gather writes every other position. Also the longest list, a statistic of
// the prepared scene.
__global__ void __launch_bounds__(kBlock)
list_offsets_kernel(const unsigned long long *__restrict__ keys, BatchHeader *__restrict__ hdr,
                    uint32_t *__restrict__ seg_scan, long long seg_cap, SortedScene scene, int64_t slots_cap) {
  // nothing was emitted past the capacity (the emit flags that overflow)
  const uint32_t nseg = uint32_t(min(3ll * hdr->cells, seg_cap));
  const uint32_t R = hdr->replicas;
  const float q = __int_as_float(0x7fc00000);
  auto sentinel = [&](int64_t k) {
    if (k < slots_cap) {
      scene.xmin[k] = q;
      scene.xmax[k] = q;
      scene.partner[k] = int(k);
      scene.run_end[k] = int(k);
    }
  };
  uint32_t mx = 0;
  auto lower = [&](uint32_t s) {
    uint32_t a = 0, e = R;
    while (a < e) {
      const uint32_t mid = (a + e) >> 1;
      if (uint32_t(keys[mid] >> 32) < s) a = mid + 1;
      else e = mid;
    }
    return a;
  };
  const uint32_t stride = gridDim.x * kBlock;
  for (uint32_t s = blockIdx.x * kBlock + threadIdx.x; s <= nseg; s += stride) {
    const uint32_t lo = s < nseg ? lower(s) : R;
    seg_scan[s] = lo;
    if (s < nseg) {
      const uint32_t hi = lower(s + 1);
      mx = max(mx, hi - lo);
      sentinel(int64_t(hi) + s);
    }
  }
  for (uint32_t t = blockIdx.x * kBlock + threadIdx.x; t < uint32_t(kSortedPad); t += stride)
    sentinel(int64_t(R) + nseg + t);
  mx = __reduce_max_sync(kFullMask, mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&hdr->max_list, mx);
}

// Lower bounds of every cell on the two non-sweep axes (-inf for the first
// row or column, where no box can start below the cell).
__global__ void __launch_bounds__(kBlock)
cell_floor_kernel(const unsigned int *__restrict__ cell_base, const SceneRecord *__restrict__ scenes,
                  const BatchHeader *hdr, float2 *__restrict__ cell_floor, long long cells_cap) {
  // more cells than the buffers hold is the replica overflow: nothing is swept
  const unsigned int cells = (long long)hdr->cells <= cells_cap ? hdr->cells : 0u;
  const int S = hdr->n_scenes;
  for (unsigned int cell = blockIdx.x * kBlock + threadIdx.x; cell < cells; cell += gridDim.x * kBlock) {
    int lo = 0, hi = S - 1;  // scene of the cell
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cell_base[mid] <= cell) lo = mid;
      else hi = mid - 1;
    }
    const GridParams g = scenes[lo].grid;
    const int local = int(cell - cell_base[lo]);
    const int cb = local / g.nc, cc = local - cb * g.nc;
    // cell cb of the chosen level starts at level-0 cell cb << shift
    cell_floor[cell] = make_float2(cb > 0 ? cell_lower_bound(cb << g.shift, g.ob, g.ib) : -INFINITY,
                                   cc > 0 ? cell_lower_bound(cc << g.shift, g.oc, g.ic) : -INFINITY);
  }
}

// Sorted replica p of segment s (cell c, type t; s = 3c + t) goes to
// position p + s: every list is followed by one NaN slot, which ends every
// run at its list (and cell, and scene) boundary.
// sflag of a position: bit 0 set if the cell is the box's first cell along b,
// bit 1 if it is its first cell along c, scene index above. Since the cell
// coordinate is monotone, the cell of a pair's reference point (max of the
// two minima on b, on c) is the max of the two boxes' first cells; both boxes
// lie in this cell, so the reference point is here exactly when, on each of
// b and c, one of the two replicas is its box's first cell.
// sfloor of a position: on b and on c, -inf if the cell is the box's first
// cell there, else the cell's lower bound; a candidate is in its first cell
// on an axis exactly when its minimum there is >= that bound, so the sweep
// tests the rule on the candidate's bounds, which it loads anyway.
// partner of a position: its first candidate. An edge's candidates are the
// edges after it in its list; a vertex's are the cell's faces whose min is
// >= its min (lower bound), a face's the cell's vertices whose min is > its
// min (upper bound): every V-F pair that overlaps on the sweep axis is found
// once, from the box with the smaller min (the vertex on ties), and vertex-
// vertex, edge-face and face-face candidates are never tested.
__global__ void __launch_bounds__(kBlock)
gather_cells_kernel(const stq_aabb *__restrict__ boxes, const unsigned long long *__restrict__ keys,
                    const uint32_t *__restrict__ order, const BatchHeader *hdr,
                    const unsigned int *__restrict__ cell_base,
                    const SceneRecord *__restrict__ scenes, const uint32_t *__restrict__ seg_scan,
                    float *__restrict__ xmin,
                    float *__restrict__ xmax,
                    const float2 *__restrict__ cell_floor, float4 *__restrict__ syz,
                    int4 *__restrict__ sv, int *__restrict__ sflag, float2 *__restrict__ sfloor,
                    int *__restrict__ partner, int *__restrict__ run_end) {
  const int64_t R = hdr->replicas;
  const int S = hdr->n_scenes;
  for (int64_t p = blockIdx.x * int64_t(kBlock) + threadIdx.x; p < R;
       p += int64_t(gridDim.x) * kBlock) {
    const unsigned long long key = keys[p];
    const unsigned int seg = unsigned(key >> 32);
    const unsigned int cell = seg / 3u, type = seg - 3u * cell;
    const uint32_t bi = order[p];
    int lo = 0, hi = S - 1;  // scene of the cell
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cell_base[mid] <= cell) lo = mid;
      else hi = mid - 1;
    }
    const GridParams g = scenes[lo].grid;
    int b, c;
    axes_bc(g.axis, b, c);
    const stq_aabb &x = boxes[bi];
    const int local = int(cell - cell_base[lo]);
    const int cb = local / g.nc, cc = local - cb * g.nc;
    const int fb = (cell_coord(x.min[b], g.ob, g.ib, g.nb0) >> g.shift) == cb;
    const int fc = (cell_coord(x.min[c], g.oc, g.ic, g.nc0) >> g.shift) == cc;
    const int64_t k = p + seg;
    int64_t first = k + 1;
    // the candidate list: the edge's own list after it, or the other type's
    // list of the cell from the bound search below
    unsigned int cand = seg;
    uint32_t run_a = uint32_t(p) + 1u, run_e = seg_scan[seg + 1];
    if (type != 1u) {
      // bound search of this min among the other list's sorted keys
      const unsigned int other = 3u * cell + (type == 0u ? 2u : 0u);
      const uint32_t xk = uint32_t(key & 0xffffffffu);
      uint32_t a = seg_scan[other], e = seg_scan[other + 1];
      run_e = e;
      while (a < e) {
        const uint32_t mid = (a + e) >> 1;
        const uint32_t mk = uint32_t(keys[mid] & 0xffffffffu);
        if (type == 0u ? mk < xk : mk <= xk) a = mid + 1;
        else e = mid;
      }
      first = int64_t(a) + other;
      cand = other;
      run_a = a;
    }
    if (run_end) {
      // end of the run: the first candidate whose min is above this max
      // (keys order as floats, -0 = +0, so the key test is the sweep's x
      // test); galloping from the run's start, then a bisection
      const uint32_t xk = float_key(x.max[g.axis]);
      uint32_t a = run_a, step = 8;
      while (a + step <= run_e && uint32_t(keys[a + step - 1] & 0xffffffffu) <= xk) {
        a += step;
        step <<= 1;
      }
      uint32_t e = min(a + step, run_e);
      while (a < e) {
        const uint32_t mid = (a + e) >> 1;
        if (uint32_t(keys[mid] & 0xffffffffu) <= xk) a = mid + 1;
        else e = mid;
      }
      run_end[k] = int(int64_t(a) + cand);
    }
    xmin[k] = x.min[g.axis];
    xmax[k] = x.max[g.axis];
    syz[k] = make_float4(x.min[b], x.min[c], x.max[b], x.max[c]);
    sv[k] = make_int4(x.vertex_ids[0], x.vertex_ids[1], x.vertex_ids[2], x.id);
    sflag[k] = (lo << 2) | (fc << 1) | fb;
    float2 fl = make_float2(-INFINITY, -INFINITY);
    if (!(fb && fc)) {
      const float2 cf = cell_floor[cell];
      if (!fb) fl.x = cf.x;
      if (!fc) fl.y = cf.y;
    }
    sfloor[k] = fl;
    partner[k] = int(first);
  }
}

int blocks_for(int64_t n, int cap = 152 * 16) {
  int64_t g = (n + kBlock - 1) / kBlock;
  return int(g < 1 ? 1 : (g > cap ? cap : g));
}

// Blocks of kBlock threads of a grid-stride kernel over n items: one per
// kBlock items, at most one wave of resident blocks. Every block of a grid-
// stride loop takes the same share, so a grid of 2.7 waves would run its last
// wave on two thirds of the block slots.
int wave_blocks(const void *kernel, int64_t n) {
  static std::mutex m;
  static std::vector<std::pair<const void *, int>> per_sm;  // kernel -> resident blocks per SM
  int resident = 0;
  {
    std::lock_guard<std::mutex> g(m);
    for (const auto &e : per_sm)
      if (e.first == kernel) resident = e.second;
    if (!resident) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kernel, kBlock, 0) != cudaSuccess ||
          resident < 1) {
        (void)cudaGetLastError();
        resident = 1;
      }
      per_sm.emplace_back(kernel, resident);
    }
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms < 1) {
    (void)cudaGetLastError();
    sms = 152;
  }
  return blocks_for(n, sms * resident);
}

__global__ void __launch_bounds__(kBlock)
reset_sweep_kernel(BatchHeader *hdr, unsigned long long *scene_pairs) {
  const int S = hdr->n_scenes;
  for (int s = blockIdx.x * kBlock + threadIdx.x; s < S; s += gridDim.x * kBlock)
    scene_pairs[s] = 0ull;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hdr->pairs = 0ull;
    hdr->work = 0;
    hdr->long_items = 0u;
    hdr->long_work = 0u;
    hdr->candidates = 0ull;
  }
}

// After a window of a host-buffer sweep: stores the slot's running pair count
// in page-locked host memory (a kernel store, so that no copy-engine work sits
// between two windows of a stream while the engines move pair lists) and
// restarts the slot's cursors for its next window.
__global__ void window_step_kernel(WindowCounters *wc, unsigned long long *host_count) {
  if (threadIdx.x != 0) return;
  *reinterpret_cast<volatile unsigned long long *>(host_count) = wc->pairs;
  wc->work = 0;
  wc->long_items = 0u;
  wc->long_work = 0u;
  __threadfence_system();
}

}  // namespace

cudaError_t launch_window_step(cudaStream_t s, WindowCounters *wc, unsigned long long *host_count) {
  window_step_kernel<<<1, 32, 0, s>>>(wc, host_count);
  return cudaGetLastError();
}

cudaError_t launch_reset_sweep(cudaStream_t s, BatchHeader *hdr, unsigned long long *scene_pairs,
                               int scene_cap) {
  reset_sweep_kernel<<<blocks_for(scene_cap, 64), kBlock, 0, s>>>(hdr, scene_pairs);
  return cudaGetLastError();
}

cudaError_t launch_batch_stats(cudaStream_t s, const BatchBuffers &b) {
  batch_reset_kernel<<<blocks_for(b.scene_cap, 64), kBlock, 0, s>>>(b.scenes, b.inputs,
                                                                      b.scene_pairs, b.hdr);
  batch_stats_kernel<<<unsigned(b.tile_cap), kBlock, 0, s>>>(b.boxes, b.tiles, b.scenes, b.hdr);
  return cudaGetLastError();
}

cudaError_t launch_batch_policy(cudaStream_t s, const BatchBuffers &b) {
  batch_policy_kernel<<<unsigned(b.scene_cap), kBlock, 0, s>>>(b.boxes, b.box_off, b.scenes, b.hdr);
  return cudaGetLastError();
}

cudaError_t launch_batch_box_keys(cudaStream_t s, const BatchBuffers &b) {
  batch_box_keys_kernel<<<unsigned(b.tile_cap), kBlock, 0, s>>>(b.boxes, b.tiles, b.scenes, b.hdr, b.box_keys,
                                                                b.box_vals, b.box_cells);
  batch_choose_kernel<<<1, 1024, 0, s>>>(b.box_off, b.scenes, b.cell_base, b.hdr);
  return cudaGetLastError();
}

cudaError_t launch_batch_counts(cudaStream_t s, const BatchBuffers &b, int64_t n) {
  const int64_t m = std::max<int64_t>(n, b.box_cap);
  batch_count_kernel<<<wave_blocks((const void *)batch_count_kernel, m), kBlock, 0, s>>>(
      b.order, b.box_cells, b.box_off, b.scenes, b.hdr, b.counts, b.box_cap);
  return cudaGetLastError();
}

cudaError_t launch_batch_emit(cudaStream_t s, const BatchBuffers &b, int64_t n, int num_sms) {
  batch_emit_kernel<<<wave_blocks((const void *)batch_emit_kernel, n), kBlock, 0, s>>>(
      b.box_cells, b.sorted_keys, b.order, b.box_off, b.scenes, b.cell_base, b.hdr, b.offsets, b.keys, b.vals,
      b.rep_cap, b.seg_cap);
  return cudaGetLastError();
}

cudaError_t launch_list_offsets(cudaStream_t s, const unsigned long long *keys, BatchHeader *hdr, uint32_t *seg_scan,
                                int64_t seg_cap, const SortedScene &scene, int64_t slots_cap) {
  list_offsets_kernel<<<blocks_for(seg_cap + 1), kBlock, 0, s>>>(keys, hdr, seg_scan, seg_cap, scene, slots_cap);
  return cudaGetLastError();
}

cudaError_t launch_gather_cells(cudaStream_t s, const stq_aabb *boxes,
                                const unsigned long long *keys, const uint32_t *order,
                                const BatchHeader *hdr, int64_t rep_cap,
                                const unsigned int *cell_base, const SceneRecord *scenes,
                                const uint32_t *seg_scan, float2 *cell_floor, int64_t cells_cap,
                                SortedScene scene) {
  cell_floor_kernel<<<blocks_for(cells_cap), kBlock, 0, s>>>(cell_base, scenes, hdr, cell_floor, cells_cap);
  gather_cells_kernel<<<wave_blocks((const void *)gather_cells_kernel, rep_cap), kBlock, 0, s>>>(
      boxes, keys, order, hdr, cell_base, scenes, seg_scan, scene.xmin, scene.xmax, cell_floor, scene.syz,
      scene.sv, scene.sflag, scene.sfloor, scene.partner, scene.run_end);
  return cudaGetLastError();
}

}  // namespace stq
