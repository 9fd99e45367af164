// boxes.cu - swept-box construction, sweep-axis choice, sort-key preparation
// and the sorted-scene gather.
//
// Build with IEEE float semantics (no --use_fast_math, -ftz=false): the box
// builder subtracts the smallest denormal and must not flush it.
#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {

namespace {

constexpr int kBuildBlock = 256;

// Min/max over the trajectory points of one primitive, per coordinate, in
// fp64; the reference rounds that extreme to float, moves it one ulp outward
// and widens it by nextafter_up(inflation_radius)
// (src/aabb.cu:193-304; equal, by monotonicity of each step, to the CPU
// builder's per-vertex rounding then union, src/cpu/aabb.cpp:23-95).
__device__ __forceinline__ void finish_box(const double lo[3], const double hi[3],
                                           float r_up, stq_aabb &b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.min[k] = __fsub_rn(ref_next_down(__double2float_rn(lo[k])), r_up);
    b.max[k] = __fadd_rn(ref_next_up(__double2float_rn(hi[k])), r_up);
  }
}

__device__ __forceinline__ void load_point(const double *V, int64_t i, double p[3]) {
  p[0] = V[3 * i];
  p[1] = V[3 * i + 1];
  p[2] = V[3 * i + 2];
}

__device__ __forceinline__ void include_point(const double p[3], double lo[3], double hi[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = p[k] < lo[k] ? p[k] : lo[k];
    hi[k] = hi[k] < p[k] ? p[k] : hi[k];
  }
}

// One thread per output box; boxes in id order: vertices, edges, faces
// (constructBoxes, src/io.cu:15-28). vertexIds as src/aabb.cu:243, 210, 285.
__global__ void __launch_bounds__(kBuildBlock)
build_boxes_kernel(const double *__restrict__ V0, const double *__restrict__ V1,
                   int64_t nV, const int32_t *__restrict__ E, int64_t nE,
                   const int32_t *__restrict__ F, int64_t nF, float r_up,
                   stq_aabb *__restrict__ out, int *flags) {
  const int64_t N = nV + nE + nF;
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < N;
       t += int64_t(gridDim.x) * blockDim.x) {
    stq_aabb b;
    double lo[3], hi[3], p[3];
    int idx[3];
    int npts;
    if (t < nV) {
      idx[0] = int(t);
      npts = 1;
      b.ref_id = int(t);
      b.vertex_ids[0] = int(t);
      b.vertex_ids[1] = int(-t - 1);
      b.vertex_ids[2] = int(-t - 1);
    } else if (t < nV + nE) {
      const int64_t e = t - nV;
      idx[0] = E[2 * e];
      idx[1] = E[2 * e + 1];
      npts = 2;
      b.ref_id = int(e);
      b.vertex_ids[0] = idx[0];
      b.vertex_ids[1] = idx[1];
      b.vertex_ids[2] = -idx[0] - 1;
    } else {
      const int64_t f = t - nV - nE;
      idx[0] = F[3 * f];
      idx[1] = F[3 * f + 1];
      idx[2] = F[3 * f + 2];
      npts = 3;
      b.ref_id = int(f);
      b.vertex_ids[0] = idx[0];
      b.vertex_ids[1] = idx[1];
      b.vertex_ids[2] = idx[2];
    }
    b.id = int(t);
    bool ok = true;
    for (int q = 0; q < npts; ++q)
      if (idx[q] < 0 || idx[q] >= nV) ok = false;
    if (!ok) {
      atomicOr(flags, kFlagBadIndex);
      for (int k = 0; k < 3; ++k) b.min[k] = b.max[k] = __int_as_float(0x7fc00000);
      out[t] = b;
      continue;
    }
    load_point(V0, idx[0], p);
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = p[k];
    load_point(V1, idx[0], p);
    include_point(p, lo, hi);
    for (int q = 1; q < npts; ++q) {
      load_point(V0, idx[q], p);
      include_point(p, lo, hi);
      load_point(V1, idx[q], p);
      include_point(p, lo, hi);
    }
    finish_box(lo, hi, r_up, b);
    out[t] = b;
  }
}

// ---- sweep-axis choice --------------------------------------------------------
// The reference's calc_mean / calc_variance (src/sweep.cu:93-123) accumulate
// the mean and the variance of the box corners with float atomics. Here each
// block reduces fp64 partial sums of (min + max) and (min^2 + max^2) per axis
// in a fixed order; one block combines them and picks the axis of largest
// variance, preferring x, then y, on ties (src/simulation.cu:630-635).
constexpr int kAxisBlock = 256;
constexpr int kAxisMaxBlocks = 1024;

__global__ void __launch_bounds__(kAxisBlock)
axis_partials_kernel(const stq_aabb *__restrict__ boxes, int64_t n,
                     double *__restrict__ partials) {
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const stq_aabb &b = boxes[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double lo = b.min[k], hi = b.max[k];
      acc[k] += lo + hi;
      acc[3 + k] += lo * lo + hi * hi;
    }
  }
  __shared__ double red[kAxisBlock / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFullMask, v, o);
    if (lane == 0) red[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0;
    for (int w = 0; w < kAxisBlock / 32; ++w) v += red[w][threadIdx.x];
    partials[blockIdx.x * 6 + threadIdx.x] = v;
  }
}

__global__ void axis_final_kernel(const double *__restrict__ partials, int nblocks,
                                  int64_t n, int *d_axis) {
  if (threadIdx.x != 0) return;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int k = 0; k < 6; ++k) s[k] += partials[b * 6 + k];
  double var[3];
  const double m = n > 0 ? 2.0 * double(n) : 1.0;
  for (int k = 0; k < 3; ++k) {
    const double mean = s[k] / m;
    var[k] = s[3 + k] - m * mean * mean;
  }
  int axis = 0;
  if (var[1] > var[axis]) axis = 1;
  if (var[2] > var[axis]) axis = 2;
  *d_axis = axis;
}

// ---- sort keys (create_ds, src/sweep.cu:125-161, first half) ------------------
__global__ void __launch_bounds__(256)
prep_keys_kernel(const stq_aabb *__restrict__ boxes, int64_t n,
                 const int *__restrict__ d_axis, uint32_t *__restrict__ keys,
                 uint32_t *__restrict__ vals, int *flags) {
  const int axis = *d_axis;
  bool nan = false;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const stq_aabb &b = boxes[i];
    const float lo = b.min[axis];
#pragma unroll
    for (int k = 0; k < 3; ++k) nan |= (b.min[k] != b.min[k]) | (b.max[k] != b.max[k]);
    keys[i] = float_key(lo);
    vals[i] = uint32_t(i);
  }
  if (__any_sync(kFullMask, nan) && (threadIdx.x & 31) == 0) atomicOr(flags, kFlagNaN);
}

// ---- sorted scene (create_ds, second half; the MiniBox of src/aabb.cuh:75-97
// split into 16-byte-aligned bounds and ids) -----------------------------------
__global__ void __launch_bounds__(256)
gather_kernel(const stq_aabb *__restrict__ boxes, const uint32_t *__restrict__ order,
              int64_t n, const int *__restrict__ d_axis, float2 *__restrict__ sx,
              float4 *__restrict__ syz, int4 *__restrict__ sv) {
  const int a = *d_axis;
  const int b = a == 0 ? 1 : 0;
  const int c = a == 2 ? 1 : 2;
  const int64_t total = n + 1 + kSortedPad;
  for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < total;
       k += int64_t(gridDim.x) * blockDim.x) {
    if (k < n) {
      const stq_aabb &x = boxes[order[k]];
      sx[k] = make_float2(x.min[a], x.max[a]);
      syz[k] = make_float4(x.min[b], x.min[c], x.max[b], x.max[c]);
      sv[k] = make_int4(x.vertex_ids[0], x.vertex_ids[1], x.vertex_ids[2], x.id);
    } else {  // sentinel and padding: NaN never passes the x-overlap test
      const float q = __int_as_float(0x7fc00000);
      sx[k] = make_float2(q, q);
      syz[k] = make_float4(q, q, q, q);
      sv[k] = make_int4(0, 0, 0, -1);
    }
  }
}


// ---- cells mode: statistics, grid policy, replicas -----------------------------
constexpr int kStatsBlock = 256;
constexpr int kStatsMaxBlocks = 1024;
constexpr int kHistBias = 40;  // bucket = binary exponent of the extent + 40

__device__ __forceinline__ float key_float(uint32_t k) {
  const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(b);
}

__global__ void stats_init_kernel(SceneStats *st) {
  for (int i = threadIdx.x; i < 3; i += blockDim.x) {
    st->lo_key[i] = 0xffffffffu;
    st->hi_key[i] = 0u;
  }
  for (int i = threadIdx.x; i < 3 * 64; i += blockDim.x) (&st->hist[0][0])[i] = 0u;
  if (threadIdx.x == 0) st->inverted = 0;
}

// One pass: fp64 partial sums for the variance (per block, fixed order),
// order-preserving min/max of the bounds, a log2 histogram of the extents
// (every 8th box), inverted-box and NaN flags.
__global__ void __launch_bounds__(kStatsBlock)
scene_stats_kernel(const stq_aabb *__restrict__ boxes, int64_t n, double *__restrict__ partials,
                   SceneStats *st, int *flags) {
  __shared__ unsigned sh_hist[3][64];
  for (int i = threadIdx.x; i < 3 * 64; i += kStatsBlock) (&sh_hist[0][0])[i] = 0u;
  __syncthreads();
  double acc[6] = {0, 0, 0, 0, 0, 0};
  uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  bool inverted = false, nan = false;
  for (int64_t i = blockIdx.x * int64_t(kStatsBlock) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * kStatsBlock) {
    const stq_aabb &b = boxes[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float l = b.min[k], h = b.max[k];
      nan |= (l != l) | (h != h);
      inverted |= l > h;
      acc[k] += double(l) + double(h);
      acc[3 + k] += double(l) * double(l) + double(h) * double(h);
      lo[k] = min(lo[k], float_key(l));
      hi[k] = max(hi[k], float_key(h));
      if ((i & 7) == 0) {
        const float ext = h - l;
        int bucket = 0;
        if (ext > 0.f) {
          int e;
          frexpf(ext, &e);
          bucket = min(63, max(1, e + kHistBias));
        }
        atomicAdd(&sh_hist[k][bucket], 1u);
      }
    }
  }
  __shared__ double red[kStatsBlock / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFullMask, v, o);
    if (lane == 0) red[warp][k] = v;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint32_t l = __reduce_min_sync(kFullMask, lo[k]);
    const uint32_t h = __reduce_max_sync(kFullMask, hi[k]);
    if (lane == 0) {
      atomicMin(&st->lo_key[k], l);
      atomicMax(&st->hi_key[k], h);
    }
  }
  if (__any_sync(kFullMask, inverted) && lane == 0) atomicOr(&st->inverted, 1);
  if (__any_sync(kFullMask, nan) && lane == 0) atomicOr(flags, kFlagNaN);
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0;
    for (int w = 0; w < kStatsBlock / 32; ++w) v += red[w][threadIdx.x];
    partials[blockIdx.x * 6 + threadIdx.x] = v;
  }
  for (int i = threadIdx.x; i < 3 * 64; i += kStatsBlock) {
    const unsigned c = (&sh_hist[0][0])[i];
    if (c) atomicAdd(&(&st->hist[0][0])[i], c);
  }
}

__device__ float median_extent(const unsigned *hist) {
  unsigned total = 0;
  for (int b = 0; b < 64; ++b) total += hist[b];
  unsigned run = 0;
  for (int b = 0; b < 64; ++b) {
    run += hist[b];
    if (2 * run >= total && total > 0) return b == 0 ? 0.f : 0.75f * exp2f(float(b - kHistBias));
  }
  return 0.f;
}

__device__ int grid_side(float L, float h) {
  if (!(L > 0.f) || !(h > 0.f) || !isfinite(L)) return 1;
  const float s = ceilf(L / h);
  return s > 2048.f ? 2048 : (s < 1.f ? 1 : int(s));
}

// Axis choice (max variance unless fixed) and the cell grid policy: cell side
// = scale x median box extent on each non-sweep axis, at most 2048 cells per
// axis and at most max(1, n / 4) cells in all.
__global__ void grid_policy_kernel(const double *__restrict__ partials, int nblocks, int64_t n,
                                   const SceneStats *__restrict__ st, int axis_mode, int cells_opt,
                                   float scale, GridParams *g, int *d_axis) {
  if (threadIdx.x != 0) return;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int k = 0; k < 6; ++k) s[k] += partials[b * 6 + k];
  int axis = axis_mode;
  if (axis < 0) {
    double var[3];
    const double m = n > 0 ? 2.0 * double(n) : 1.0;
    for (int k = 0; k < 3; ++k) {
      const double mean = s[k] / m;
      var[k] = s[3 + k] - m * mean * mean;
    }
    axis = 0;
    if (var[1] > var[axis]) axis = 1;
    if (var[2] > var[axis]) axis = 2;
  }
  *d_axis = axis;
  const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
  const float lob = key_float(st->lo_key[b]), hib = key_float(st->hi_key[b]);
  const float loc = key_float(st->lo_key[c]), hic = key_float(st->hi_key[c]);
  int nb = 1, nc = 1;
  if (cells_opt != 1 && !st->inverted && n > 1) {
    if (cells_opt > 1) {
      nb = nc = cells_opt;
    } else {
      const float Lb = hib - lob, Lc = hic - loc;
      float wb = median_extent(st->hist[b]), wc = median_extent(st->hist[c]);
      if (!(wb > 0.f)) wb = Lb / 1024.f;
      if (!(wc > 0.f)) wc = Lc / 1024.f;
      nb = grid_side(Lb, scale * wb);
      nc = grid_side(Lc, scale * wc);
      const int64_t max_cells = max(int64_t(1), min(int64_t(1) << 20, n / 4));
      while (int64_t(nb) * nc > max_cells) {
        if (nb >= nc) nb = (nb + 1) / 2;
        else nc = (nc + 1) / 2;
      }
    }
  }
  const float Lb = hib - lob, Lc = hic - loc;
  g->axis = axis;
  g->nb = nb;
  g->nc = nc;
  g->ncells = nb * nc;
  int bits = 0;
  while ((1 << bits) < nb * nc) ++bits;
  g->cell_bits = bits;
  g->inverted = st->inverted;
  g->ob = lob;
  g->oc = loc;
  g->ib = (nb > 1 && Lb > 0.f && isfinite(Lb)) ? float(nb) / Lb : 0.f;
  g->ic = (nc > 1 && Lc > 0.f && isfinite(Lc)) ? float(nc) / Lc : 0.f;
  if (g->ib == 0.f) g->nb = 1;
  if (g->ic == 0.f) g->nc = 1;
  g->ncells = g->nb * g->nc;
  bits = 0;
  while ((1 << bits) < g->ncells) ++bits;
  g->cell_bits = bits;
}

struct CellRange {
  int b0, b1, c0, c1;
};

__device__ __forceinline__ CellRange cell_range(const stq_aabb &x, const GridParams &g) {
  const int b = g.axis == 0 ? 1 : 0, c = g.axis == 2 ? 1 : 2;
  CellRange r;
  r.b0 = cell_coord(x.min[b], g.ob, g.ib, g.nb);
  r.b1 = cell_coord(x.max[b], g.ob, g.ib, g.nb);
  r.c0 = cell_coord(x.min[c], g.oc, g.ic, g.nc);
  r.c1 = cell_coord(x.max[c], g.oc, g.ic, g.nc);
  return r;
}

__global__ void __launch_bounds__(256)
replica_count_kernel(const stq_aabb *__restrict__ boxes, int64_t n,
                     const GridParams *__restrict__ grid, uint32_t *__restrict__ counts) {
  const GridParams g = *grid;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const CellRange r = cell_range(boxes[i], g);
    counts[i] = uint32_t(r.b1 - r.b0 + 1) * uint32_t(r.c1 - r.c0 + 1);
  }
}

__global__ void __launch_bounds__(256)
replica_emit_kernel(const stq_aabb *__restrict__ boxes, int64_t n,
                    const GridParams *__restrict__ grid, const uint32_t *__restrict__ offsets,
                    unsigned long long *__restrict__ keys, uint32_t *__restrict__ vals) {
  const GridParams g = *grid;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const stq_aabb &x = boxes[i];
    const CellRange r = cell_range(x, g);
    const unsigned long long xk = float_key(x.min[g.axis]);
    uint32_t o = offsets[i];
    for (int cb = r.b0; cb <= r.b1; ++cb)
      for (int cc = r.c0; cc <= r.c1; ++cc) {
        keys[o] = (static_cast<unsigned long long>(cb * g.nc + cc) << 32) | xk;
        vals[o] = uint32_t(i);
        ++o;
      }
  }
}

__global__ void __launch_bounds__(256)
fill_sentinels_kernel(float2 *__restrict__ sx, int64_t slots) {
  const float q = __int_as_float(0x7fc00000);
  for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < slots;
       k += int64_t(gridDim.x) * blockDim.x)
    sx[k] = make_float2(q, q);
}

// Sorted replica p of cell c goes to position p + c: every cell is followed
// by one NaN slot (prefilled), which ends every x-run at the cell boundary.
__global__ void __launch_bounds__(256)
gather_cells_kernel(const stq_aabb *__restrict__ boxes, const unsigned long long *__restrict__ keys,
                    const uint32_t *__restrict__ order, int64_t R,
                    const GridParams *__restrict__ grid, float2 *__restrict__ sx,
                    float4 *__restrict__ syz, int4 *__restrict__ sv, int *__restrict__ scell) {
  const int a = grid->axis;
  const int b = a == 0 ? 1 : 0;
  const int c = a == 2 ? 1 : 2;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < R;
       p += int64_t(gridDim.x) * blockDim.x) {
    const int cell = int(keys[p] >> 32);
    const stq_aabb &x = boxes[order[p]];
    const int64_t k = p + cell;
    sx[k] = make_float2(x.min[a], x.max[a]);
    syz[k] = make_float4(x.min[b], x.min[c], x.max[b], x.max[c]);
    sv[k] = make_int4(x.vertex_ids[0], x.vertex_ids[1], x.vertex_ids[2], x.id);
    scell[k] = cell;
  }
}

int grid_for(int64_t n, int block, int cap = 152 * 32) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return int(g);
}

}  // namespace

cudaError_t launch_build_boxes(cudaStream_t s, const double *V0, const double *V1,
                               int64_t nV, const int32_t *E, int64_t nE,
                               const int32_t *F, int64_t nF, float r_up,
                               stq_aabb *out, int *flags) {
  const int64_t N = nV + nE + nF;
  if (N == 0) return cudaSuccess;
  build_boxes_kernel<<<grid_for(N, kBuildBlock), kBuildBlock, 0, s>>>(
      V0, V1, nV, E, nE, F, nF, r_up, out, flags);
  return cudaGetLastError();
}

int axis_partial_blocks(int64_t n) {
  int64_t b = (n + kAxisBlock * 8 - 1) / (kAxisBlock * 8);
  if (b < 1) b = 1;
  if (b > kAxisMaxBlocks) b = kAxisMaxBlocks;
  return int(b);
}

cudaError_t launch_axis_select(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               double *partials, int nblocks, int *d_axis) {
  axis_partials_kernel<<<nblocks, kAxisBlock, 0, s>>>(boxes, n, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  axis_final_kernel<<<1, 32, 0, s>>>(partials, nblocks, n, d_axis);
  return cudaGetLastError();
}

cudaError_t launch_prep_keys(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                             const int *d_axis, uint32_t *keys, uint32_t *vals,
                             int *flags) {
  if (n == 0) return cudaSuccess;
  prep_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(boxes, n, d_axis, keys, vals, flags);
  return cudaGetLastError();
}

cudaError_t launch_gather(cudaStream_t s, const stq_aabb *boxes,
                          const uint32_t *order, int64_t n, const int *d_axis,
                          SortedScene scene) {
  const int64_t total = n + 1 + kSortedPad;
  gather_kernel<<<grid_for(total, 256), 256, 0, s>>>(boxes, order, n, d_axis, scene.sx,
                                                     scene.syz, scene.sv);
  return cudaGetLastError();
}

size_t stats_partials_bytes(int64_t n) {
  (void)n;
  return sizeof(double) * 6 * kStatsMaxBlocks;
}

cudaError_t launch_scene_stats(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               double *partials, SceneStats *stats, int *flags) {
  stats_init_kernel<<<1, 256, 0, s>>>(stats);
  int64_t nb = (n + kStatsBlock * 8 - 1) / (kStatsBlock * 8);
  nb = nb < 1 ? 1 : (nb > kStatsMaxBlocks ? kStatsMaxBlocks : nb);
  scene_stats_kernel<<<unsigned(nb), kStatsBlock, 0, s>>>(boxes, n, partials, stats, flags);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // the policy kernel reads the block count from here
  return cudaSuccess;
}

int stats_blocks(int64_t n) {
  int64_t nb = (n + kStatsBlock * 8 - 1) / (kStatsBlock * 8);
  return int(nb < 1 ? 1 : (nb > kStatsMaxBlocks ? kStatsMaxBlocks : nb));
}

cudaError_t launch_grid_policy(cudaStream_t s, const double *partials, int64_t n,
                               const SceneStats *stats, int axis_mode, int cells_opt,
                               float scale, GridParams *grid, int *d_axis) {
  grid_policy_kernel<<<1, 32, 0, s>>>(partials, stats_blocks(n), n, stats, axis_mode, cells_opt,
                                      scale, grid, d_axis);
  return cudaGetLastError();
}

cudaError_t launch_replica_count(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                                 const GridParams *grid, uint32_t *counts) {
  if (n == 0) return cudaSuccess;
  replica_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(boxes, n, grid, counts);
  return cudaGetLastError();
}

cudaError_t launch_replica_emit(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                                const GridParams *grid, const uint32_t *offsets,
                                unsigned long long *keys, uint32_t *vals) {
  if (n == 0) return cudaSuccess;
  replica_emit_kernel<<<grid_for(n, 256), 256, 0, s>>>(boxes, n, grid, offsets, keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_fill_sentinels(cudaStream_t s, float2 *sx, int64_t slots) {
  fill_sentinels_kernel<<<grid_for(slots, 256), 256, 0, s>>>(sx, slots);
  return cudaGetLastError();
}

cudaError_t launch_gather_cells(cudaStream_t s, const stq_aabb *boxes,
                                const unsigned long long *keys, const uint32_t *order,
                                int64_t R, const GridParams *grid, SortedScene scene) {
  if (R == 0) return cudaSuccess;
  gather_cells_kernel<<<grid_for(R, 256), 256, 0, s>>>(boxes, keys, order, R, grid, scene.sx,
                                                       scene.syz, scene.sv, scene.scell);
  return cudaGetLastError();
}

}  // namespace stq
