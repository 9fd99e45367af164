// boxes.cu - swept-box construction from vertex trajectories, for one scene
// or for a batch of scenes.
//
// Build with IEEE float semantics (no --use_fast_math, -ftz=false): the box
// builder subtracts the smallest denormal and must not flush it.
#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {

namespace {

constexpr int kBuildBlock = 256;

// Min/max over the trajectory points of one primitive, per coordinate; the
// reference takes the extreme in fp64, rounds it to float, moves it one ulp
// outward and widens it by nextafter_up(inflation_radius) (src/aabb.cu:193-304).
// Rounding to float is monotone (overflow goes to +-inf, NaN stays NaN), so
// rounding every point first and taking the extreme in float gives the same
// bits (the CPU builder's order, src/cpu/aabb.cpp:23-95). fp64 work is slow on
// this part, conversions included, so the positions are rounded once per
// vertex (round_points_kernel) rather than once per box that uses them: a face
// box would convert 18 coordinates, an edge box 12.
__device__ __forceinline__ void load_point(const double *V, int64_t i, float p[3]) {
  p[0] = __double2float_rn(V[3 * i]);
  p[1] = __double2float_rn(V[3 * i + 1]);
  p[2] = __double2float_rn(V[3 * i + 2]);
}

// Rounded positions of vertex i: (x0, y0, z0, x1) and (y1, z1, -, -).
__device__ __forceinline__ void load_rounded(const float4 *P, int64_t i, float p0[3], float p1[3]) {
  const float4 a = P[2 * i], b = P[2 * i + 1];
  p0[0] = a.x;
  p0[1] = a.y;
  p0[2] = a.z;
  p1[0] = a.w;
  p1[1] = b.x;
  p1[2] = b.y;
}

// P[2v], P[2v + 1] <- vertex v's t0 and t1 positions rounded to float.
__global__ void __launch_bounds__(256)
round_points_kernel(const double *__restrict__ V0, const double *__restrict__ V1, int64_t nV,
                    float4 *__restrict__ P) {
  for (int64_t v = blockIdx.x * 256ll + threadIdx.x; v < nV; v += int64_t(gridDim.x) * 256) {
    float a[3], b[3];
    load_point(V0, v, a);
    load_point(V1, v, b);
    P[2 * v] = make_float4(a[0], a[1], a[2], b[0]);
    P[2 * v + 1] = make_float4(b[1], b[2], 0.f, 0.f);
  }
}

// Batched: the scenes' vertices are consecutive, voff[S] of them (at most vert_cap).
__global__ void __launch_bounds__(256)
batch_round_points_kernel(const double *__restrict__ V0, const double *__restrict__ V1,
                          const long long *__restrict__ voff, const BatchHeader *hdr, int64_t vert_cap,
                          float4 *__restrict__ P) {
  const long long n = voff[hdr->n_scenes];
  const int64_t nV = n < vert_cap ? n : vert_cap;
  for (int64_t v = blockIdx.x * 256ll + threadIdx.x; v < nV; v += int64_t(gridDim.x) * 256) {
    float a[3], b[3];
    load_point(V0, v, a);
    load_point(V1, v, b);
    P[2 * v] = make_float4(a[0], a[1], a[2], b[0]);
    P[2 * v + 1] = make_float4(b[1], b[2], 0.f, 0.f);
  }
}

__device__ __forceinline__ void include_point(const float p[3], float lo[3], float hi[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = p[k] < lo[k] ? p[k] : lo[k];
    hi[k] = hi[k] < p[k] ? p[k] : hi[k];
  }
}

// One box t of a scene with nV vertices, nE edges, nF faces: boxes in id
// order vertices, edges, faces (constructBoxes, src/io.cu:15-28); vertexIds
// as src/aabb.cu:243, 210, 285.
// Points from P (rounded once per vertex) when P is given, else from V0/V1.
__device__ __forceinline__ stq_aabb build_one(const double *__restrict__ V0,
                                              const double *__restrict__ V1, const float4 *__restrict__ P,
                                              int64_t nV, const int32_t *__restrict__ E, int64_t nE,
                                              const int32_t *__restrict__ F, int64_t t, int id,
                                              float r_up, int *flags) {
  stq_aabb b;
  float lo[3], hi[3], p[3];
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
  b.id = id;
  bool ok = true;
  for (int q = 0; q < npts; ++q)
    if (idx[q] < 0 || idx[q] >= nV) ok = false;
  if (!ok) {
    atomicOr(flags, kFlagBadIndex);
    for (int k = 0; k < 3; ++k) b.min[k] = b.max[k] = __int_as_float(0x7fc00000);
    return b;
  }
  if (P) {
    float p1[3];
    load_rounded(P, idx[0], p, p1);
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = p[k];
    include_point(p1, lo, hi);
    for (int q = 1; q < npts; ++q) {
      load_rounded(P, idx[q], p, p1);
      include_point(p, lo, hi);
      include_point(p1, lo, hi);
    }
  } else {
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
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.min[k] = __fsub_rn(ref_next_down(lo[k]), r_up);
    b.max[k] = __fadd_rn(ref_next_up(hi[k]), r_up);
  }
  return b;
}

constexpr int kBoxWords = int(sizeof(stq_aabb) / 4);  // 11
static_assert(sizeof(stq_aabb) == 44, "44-byte boxes");

// The warp's boxes out[base, base + count), lane l holding box base + l, go
// through shared memory and out as consecutive 4-byte words: 11 coalesced
// stores per 32 boxes instead of 11 strided stores per box.
__device__ __forceinline__ void store_boxes(const stq_aabb &b, bool have, int64_t base, int count,
                                            stq_aabb *__restrict__ out, uint32_t *sm, int lane) {
  if (have) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(&b);
#pragma unroll
    for (int f = 0; f < kBoxWords; ++f) sm[lane * kBoxWords + f] = w[f];
  }
  __syncwarp();
  uint32_t *dst = reinterpret_cast<uint32_t *>(out + base);
  if (count == 32) {  // all shared-memory reads before the first store
    uint32_t v[kBoxWords];
#pragma unroll
    for (int f = 0; f < kBoxWords; ++f) v[f] = sm[f * 32 + lane];
#pragma unroll
    for (int f = 0; f < kBoxWords; ++f) dst[f * 32 + lane] = v[f];
  } else {
    for (int i = lane; i < count * kBoxWords; i += 32) dst[i] = sm[i];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kBuildBlock)
build_boxes_kernel(const double *__restrict__ V0, const double *__restrict__ V1,
                   int64_t nV, const int32_t *__restrict__ E, int64_t nE,
                   const int32_t *__restrict__ F, int64_t nF, float r_up,
                   stq_aabb *__restrict__ out, int *flags, const float4 *__restrict__ P) {
  __shared__ uint32_t stage[kBuildBlock / 32][32 * kBoxWords];
  const int lane = threadIdx.x & 31;
  const int64_t N = nV + nE + nF;
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) - lane; base < N; base += step) {
    const int64_t t = base + lane;
    stq_aabb b;
    if (t < N) b = build_one(V0, V1, P, nV, E, nE, F, t, int(t), r_up, flags);
    store_boxes(b, t < N, base, int(N - base < 32 ? N - base : 32), out, stage[threadIdx.x >> 5], lane);
  }
}

// Batched: box t belongs to the scene s with box_off[s] <= t < box_off[s+1];
// its id is the batch index t, its vertex ids are local to scene s.
__global__ void __launch_bounds__(kBuildBlock)
batch_build_kernel(const double *__restrict__ V0, const double *__restrict__ V1,
                   const long long *__restrict__ voff, const int32_t *__restrict__ E,
                   const long long *__restrict__ eoff, const int32_t *__restrict__ F,
                   const long long *__restrict__ foff, const long long *__restrict__ box_off,
                   BatchHeader *hdr, float r_up, stq_aabb *__restrict__ out,
                   const float4 *__restrict__ P) {
  __shared__ uint32_t stage[kBuildBlock / 32][32 * kBoxWords];
  const int lane = threadIdx.x & 31;
  const int n_scenes = hdr->n_scenes;
  const int64_t n_boxes = hdr->n_boxes;
  int *flags = &hdr->flags;
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) - lane; base < n_boxes;
       base += step) {
    const int64_t t = base + lane;
    stq_aabb b;
    if (t < n_boxes) {
      int lo = 0, hi = n_scenes - 1;  // last scene with box_off[s] <= t
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (box_off[mid] <= t) lo = mid;
        else hi = mid - 1;
      }
      const int s = lo;
      const int64_t v0 = voff[s], e0 = eoff[s], f0 = foff[s];
      b = build_one(V0 + 3 * v0, V1 + 3 * v0, P + 2 * v0, voff[s + 1] - v0, E + 2 * e0, eoff[s + 1] - e0,
                    F + 3 * f0, t - box_off[s], int(t), r_up, flags);
    }
    store_boxes(b, t < n_boxes, base, int(n_boxes - base < 32 ? n_boxes - base : 32), out, stage[threadIdx.x >> 5],
                lane);
  }
}

// Serving: scene s's mesh lives in its own allocation (MeshRef); the box id
// is the batch index, vertex ids are local to the scene.
__global__ void __launch_bounds__(kBuildBlock)
batch_build_refs_kernel(const MeshRef *__restrict__ refs, const long long *__restrict__ box_off,
                        BatchHeader *hdr, float r_up, stq_aabb *__restrict__ out) {
  __shared__ uint32_t stage[kBuildBlock / 32][32 * kBoxWords];
  const int lane = threadIdx.x & 31;
  const int n_scenes = hdr->n_scenes;
  const int64_t n_boxes = hdr->n_boxes;
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) - lane; base < n_boxes;
       base += step) {
    const int64_t t = base + lane;
    stq_aabb b;
    if (t < n_boxes) {
      int lo = 0, hi = n_scenes - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (box_off[mid] <= t) lo = mid;
        else hi = mid - 1;
      }
      const MeshRef &m = refs[lo];
      b = build_one(m.V0, m.V1, nullptr, m.nV, m.E, m.nE, m.F, t - box_off[lo], int(t), r_up, &hdr->flags);
    }
    store_boxes(b, t < n_boxes, base, int(n_boxes - base < 32 ? n_boxes - base : 32), out, stage[threadIdx.x >> 5],
                lane);
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
                               stq_aabb *out, int *flags, float4 *points) {
  const int64_t N = nV + nE + nF;
  if (N == 0) return cudaSuccess;
  if (nV > 0) round_points_kernel<<<grid_for(nV, 256), 256, 0, s>>>(V0, V1, nV, points);
  build_boxes_kernel<<<grid_for(N, kBuildBlock), kBuildBlock, 0, s>>>(
      V0, V1, nV, E, nE, F, nF, r_up, out, flags, nV > 0 ? points : nullptr);
  return cudaGetLastError();
}

cudaError_t launch_batch_build(cudaStream_t s, const double *V0, const double *V1,
                               const long long *voff, const int32_t *E, const long long *eoff,
                               const int32_t *F, const long long *foff, const long long *box_off,
                               BatchHeader *hdr, int64_t box_cap, float r_up, stq_aabb *out,
                               float4 *points, int64_t vert_cap) {
  batch_round_points_kernel<<<grid_for(vert_cap, 256), 256, 0, s>>>(V0, V1, voff, hdr, vert_cap, points);
  batch_build_kernel<<<grid_for(box_cap, kBuildBlock), kBuildBlock, 0, s>>>(
      V0, V1, voff, E, eoff, F, foff, box_off, hdr, r_up, out, points);
  return cudaGetLastError();
}

cudaError_t launch_batch_build_refs(cudaStream_t s, const MeshRef *refs, const long long *box_off,
                                    BatchHeader *hdr, int64_t box_cap, float r_up, stq_aabb *out) {
  batch_build_refs_kernel<<<grid_for(box_cap, kBuildBlock), kBuildBlock, 0, s>>>(refs, box_off, hdr,
                                                                                 r_up, out);
  return cudaGetLastError();
}

}  // namespace stq
