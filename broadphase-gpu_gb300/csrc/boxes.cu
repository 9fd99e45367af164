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

}  // namespace stq
