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
  constexpr int W = 11;  // words per box
  __shared__ uint32_t stage[kBlock / 32][32 * W];
  const TileRec t = tiles[blockIdx.x];
  const int lane = threadIdx.x & 31;
  uint32_t *sm = stage[threadIdx.x >> 5];
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
  // warp-staged loads: 32 boxes as 11 coalesced word loads, all issued before
  // the first is stored (a store that waits on its load would serialise them)
  const uint32_t *src = reinterpret_cast<const uint32_t *>(boxes + t.begin);
  for (int i0 = threadIdx.x - lane; i0 < t.count; i0 += kBlock) {
    const int n = min(32, t.count - i0);
    if (n == 32) {
      uint32_t v[W];
#pragma unroll
      for (int w = 0; w < W; ++w) v[w] = src[int64_t(i0) * W + w * 32 + lane];
#pragma unroll
      for (int w = 0; w < W; ++w) sm[w * 32 + lane] = v[w];
    } else {
      for (int w = lane; w < n * W; w += 32) sm[w] = src[int64_t(i0) * W + w];
    }
    __syncwarp();
    if (lane < n) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float l = __uint_as_float(sm[lane * W + 1 + k]), h = __uint_as_float(sm[lane * W + 4 + k]);
        nan |= (l != l) | (h != h);
        inverted |= l > h;
        const float dl = l - c[k], dh = h - c[k];
        s1[k] += dl + dh;
        s2[k] += dl * dl + dh * dh;
        lo[k] = min(lo[k], float_key(l));
        hi[k] = max(hi[k], float_key(h));
      }
    }
    __syncwarp();
  }
  __shared__ double dred[kBlock / 32][6];
  SceneRecord &r = scenes[t.scene];
  const double mom[6] = {double(s1[0]), double(s1[1]), double(s1[2]), double(s2[0]), double(s2[1]), double(s2[2])};
  double tot[6];
  block_sums(mom, tot, dred);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // sum(l + h) = S1 + 2 n c; sum(l^2 + h^2) = S2 + 2 c S1 + 2 n c^2
    if (threadIdx.x == 0) {
      const double a = tot[k], q = tot[3 + k];
      const double ck = c[k], n = double(t.count);
      atomicAdd(&r.s1[k], a + 2.0 * n * ck);
      atomicAdd(&r.s2[k], q + 2.0 * ck * a + 2.0 * n * ck * ck);
    }
    const uint32_t l = __reduce_min_sync(kFullMask, lo[k]);
    const uint32_t h = __reduce_max_sync(kFullMask, hi[k]);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&r.lo_key[k], l);
      atomicMax(&r.hi_key[k], h);
    }
  }
  if (__any_sync(kFullMask, inverted) && (threadIdx.x & 31) == 0) atomicOr(&r.inverted, 1);
  if (__any_sync(kFullMask, nan) && (threadIdx.x & 31) == 0) atomicOr(&hdr->flags, kFlagNaN);
}

__device__ int grid_side(float L, float h) {
  if (!(L > 0.f) || !(h > 0.f) || !isfinite(L)) return 1;
  const float s = ceilf(L / h);
  return s > float(kMaxGridSide) ? kMaxGridSide : (s < 1.f ? 1 : int(s));
}

__device__ __forceinline__ int level_side(int base, int level) {
  const int s = (base + (1 << level) - 1) >> level;
  return s < 1 ? 1 : s;
}

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
  r.base_nb = nb;
  r.base_nc = nc;
  GridParams &g = r.grid;
  g.axis = axis;
  g.ob = lob;
  g.oc = loc;
  g.Lb = Lb;
  g.Lc = Lc;
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

__device__ __forceinline__ float inv_side(int n, float L) { return n > 1 ? float(n) / L : 0.f; }

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

// ---- 3. replicas per grid level, per scene ------------------------------------------
__global__ void __launch_bounds__(kBlock)
batch_levels_kernel(const stq_aabb *__restrict__ boxes, const TileRec *__restrict__ tiles,
                    SceneRecord *scenes, const BatchHeader *hdr) {
  if (int(blockIdx.x) >= hdr->n_tiles) return;
  const TileRec t = tiles[blockIdx.x];
  SceneRecord &r = scenes[t.scene];
  const GridParams g = r.grid;
  int nbl[kGridLevels], ncl[kGridLevels];
  float ibl[kGridLevels], icl[kGridLevels];
#pragma unroll
  for (int l = 0; l < kGridLevels; ++l) {
    nbl[l] = level_side(r.base_nb, l);
    ncl[l] = level_side(r.base_nc, l);
    ibl[l] = inv_side(nbl[l], g.Lb);
    icl[l] = inv_side(ncl[l], g.Lc);
  }
  // a thread sees at most kTileBoxes / kBlock = 16 boxes of at most 2048^2
  // cells each: 32-bit sums per thread, 64-bit per block
  static_assert(uint64_t(kTileBoxes / kBlock) * kMaxGridSide * kMaxGridSide < (uint64_t(1) << 32),
                "per-thread level sums");
  unsigned reps[kGridLevels] = {};
  for (int i = threadIdx.x; i < t.count; i += kBlock) {
    const stq_aabb &x = boxes[t.begin + i];
#pragma unroll
    for (int l = 0; l < kGridLevels; ++l) {
      const Range q = cell_range(x, g.axis, g.ob, ibl[l], nbl[l], g.oc, icl[l], ncl[l]);
      reps[l] += unsigned(q.b1 - q.b0 + 1) * unsigned(q.c1 - q.c0 + 1);
    }
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
      int level = kGridLevels;  // none fits: one cell
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
      g.level = level;
      g.nb = level < kGridLevels ? level_side(r.base_nb, level) : 1;
      g.nc = level < kGridLevels ? level_side(r.base_nc, level) : 1;
      g.ib = inv_side(g.nb, g.Lb);
      g.ic = inv_side(g.nc, g.Lc);
      if (g.ib == 0.f) g.nb = 1;
      if (g.ic == 0.f) g.nc = 1;
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
// to the capacity), from the cell ranges by box index that the box-key kernel
// wrote
__device__ __forceinline__ uint32_t cells_count(uint2 r) {
  return ((r.x >> 11 & 2047u) - (r.x & 2047u) + 1u) * ((r.y >> 11 & 2047u) - (r.y & 2047u) + 1u);
}

__global__ void __launch_bounds__(kBlock)
batch_count_kernel(const uint32_t *__restrict__ order, const uint2 *__restrict__ box_cells,
                   const BatchHeader *hdr, uint32_t *__restrict__ counts, long long box_cap) {
  const long long N = hdr->n_boxes;
  for (long long p = blockIdx.x * (long long)kBlock + threadIdx.x; p < N; p += (long long)gridDim.x * kBlock)
    counts[p] = cells_count(box_cells[order[p]]);
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
    const int nc = scenes[sc].grid.nc;
    const unsigned long long cb0 = cell_base[sc];
    // the box's cell range and type (8 bytes, by box index) and its sort key,
    // instead of the 44-byte box
    const uint2 r = box_cells[bi];
    const int b0 = int(r.x & 2047u), b1 = int(r.x >> 11 & 2047u);
    const int c0 = int(r.y & 2047u), c1 = int(r.y >> 11 & 2047u);
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

// Sort keys of the boxes: the order-preserving image of the minimum on the
// scene's sweep axis, with the box index as value.
__global__ void __launch_bounds__(kBlock)
batch_box_keys_kernel(const stq_aabb *__restrict__ boxes, const TileRec *__restrict__ tiles,
                      const SceneRecord *__restrict__ scenes, const BatchHeader *hdr,
                      uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, uint2 *__restrict__ box_cells) {
  if (int(blockIdx.x) >= hdr->n_tiles) return;
  const TileRec t = tiles[blockIdx.x];
  const GridParams g = scenes[t.scene].grid;
  for (int i = threadIdx.x; i < t.count; i += kBlock) {
    const long long bi = t.begin + i;
    const stq_aabb &x = boxes[bi];
    keys[bi] = float_key(x.min[g.axis]);
    vals[bi] = uint32_t(bi);
    // the box's cell range and type, by box index, while the box is read in
    // order (cell coordinates are below kMaxGridSide: 11 bits)
    static_assert(kMaxGridSide <= 2048, "11-bit cell coordinates");
    const Range q = cell_range(x, g.axis, g.ob, g.ib, g.nb, g.oc, g.ic, g.nc);
    const unsigned type = unsigned(type_of(x.vertex_ids[1], x.vertex_ids[2]));
    box_cells[bi] = make_uint2(unsigned(q.b0) | unsigned(q.b1) << 11 | type << 22,
                               unsigned(q.c0) | unsigned(q.c1) << 11);
  }
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
    cell_floor[cell] = make_float2(cb > 0 ? cell_lower_bound(cb, g.ob, g.ib) : -INFINITY,
                                   cc > 0 ? cell_lower_bound(cc, g.oc, g.ic) : -INFINITY);
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
    const int fb = cell_coord(x.min[b], g.ob, g.ib, g.nb) == cb;
    const int fc = cell_coord(x.min[c], g.oc, g.ic, g.nc) == cc;
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
  batch_levels_kernel<<<unsigned(b.tile_cap), kBlock, 0, s>>>(b.boxes, b.tiles, b.scenes, b.hdr);
  batch_choose_kernel<<<1, 1024, 0, s>>>(b.box_off, b.scenes, b.cell_base, b.hdr);
  return cudaGetLastError();
}

cudaError_t launch_batch_box_keys(cudaStream_t s, const BatchBuffers &b) {
  batch_box_keys_kernel<<<unsigned(b.tile_cap), kBlock, 0, s>>>(b.boxes, b.tiles, b.scenes, b.hdr, b.box_keys,
                                                                b.box_vals, b.box_cells);
  return cudaGetLastError();
}

cudaError_t launch_batch_counts(cudaStream_t s, const BatchBuffers &b, int64_t n) {
  batch_count_kernel<<<blocks_for(std::max<int64_t>(n, b.box_cap)), kBlock, 0, s>>>(b.order, b.box_cells, b.hdr,
                                                                                  b.counts, b.box_cap);
  return cudaGetLastError();
}

cudaError_t launch_batch_emit(cudaStream_t s, const BatchBuffers &b, int64_t n, int num_sms) {
  batch_emit_kernel<<<blocks_for(n), kBlock, 0, s>>>(b.box_cells, b.sorted_keys, b.order, b.box_off, b.scenes,
                                                     b.cell_base, b.hdr,
                                              b.offsets, b.keys, b.vals, b.rep_cap, b.seg_cap);
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
  gather_cells_kernel<<<blocks_for(rep_cap), kBlock, 0, s>>>(boxes, keys, order, hdr, cell_base,
                                                             scenes, seg_scan, scene.xmin, scene.xmax,
                                                             cell_floor, scene.syz, scene.sv,
                                                             scene.sflag, scene.sfloor, scene.partner,
                                                             scene.run_end);
  return cudaGetLastError();
}

}  // namespace stq
