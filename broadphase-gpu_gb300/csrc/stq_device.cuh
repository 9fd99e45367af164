// stq_device.cuh - device-side primitives shared by the STQ kernels.
//
// Box layout, the exact outward rounding of the box builder, the order-
// preserving sort key, and the pair predicates of the reference
// (Ahdhn/broadphase-gpu src/aabb.cu:12-40, src/collision.cu:24-48).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/stq_abi.h"

namespace stq {

static_assert(sizeof(stq_aabb) == 44, "stq_aabb must match stq::gpu::Aabb (44 B)");
static_assert(offsetof(stq_aabb, min) == 4 && offsetof(stq_aabb, max) == 16 &&
                  offsetof(stq_aabb, vertex_ids) == 28 && offsetof(stq_aabb, ref_id) == 40,
              "stq_aabb field offsets must match stq::gpu::Aabb");

constexpr unsigned kFullMask = 0xffffffffu;
// Padding after the last sentinel of a sorted scene, so that a lane group of
// up to 32 lanes may read past a run end without leaving the allocation.
constexpr int kSortedPad = 256;

// ---- IEEE next float, as the reference calls it -----------------------------
// nextafter_up(x) = nextafterf(x, x + FLT_MAX) and nextafter_down(x) =
// nextafterf(x, x - FLT_MAX) (src/aabb.cu:56-61, src/cpu/aabb.cpp:16-21).
// For finite x that is the adjacent float toward +inf / -inf; for infinite x
// the direction argument equals x and x is returned. Written on the bit
// pattern from the IEEE 754 definition of adjacent floats.
__host__ __device__ inline float ref_next_up(float x) {
  if (x != x) return x;                            // NaN
  if (x == INFINITY || x == -INFINITY) return x;   // y == x
  uint32_t b;
  memcpy(&b, &x, 4);
  if ((b & 0x7fffffffu) == 0) b = 1u;              // +-0 -> +min denormal
  else if (b & 0x80000000u) b -= 1u;               // negative: toward zero
  else b += 1u;                                    // positive: away from zero
  float r;
  memcpy(&r, &b, 4);
  return r;
}

__host__ __device__ inline float ref_next_down(float x) {
  if (x != x) return x;
  if (x == INFINITY || x == -INFINITY) return x;
  uint32_t b;
  memcpy(&b, &x, 4);
  if ((b & 0x7fffffffu) == 0) b = 0x80000001u;     // +-0 -> -min denormal
  else if (b & 0x80000000u) b += 1u;               // negative: away from zero
  else b -= 1u;                                    // positive: toward zero
  float r;
  memcpy(&r, &b, 4);
  return r;
}

// ---- order-preserving float -> uint32 key -----------------------------------
// Key order is float '<' order with -0 and +0 equal (both map to the key of
// +0), so key equality is float equality and bound searches on keys agree
// with the float tests of the sweep; NaN is rejected before sorting.
__device__ __forceinline__ uint32_t float_key(float f) {
  uint32_t b = __float_as_uint(f);
  if (b == 0x80000000u) b = 0u;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Box type from the signs of vertexIds (src/aabb.cu:12-31): vertex 0, edge
// 1, face 2.
__device__ __forceinline__ int type_of(int v1, int v2) {
  return v2 >= 0 ? 2 : (v1 >= 0 ? 1 : 0);
}

// Cell coordinate of a bound: clamp(floor((v - origin) * inv), 0, n - 1),
// with round-to-nearest float steps. Each step is monotone non-decreasing in
// v, so a <= b implies cell(a) <= cell(b): a point inside a box's range has
// its cell inside the box's cell range.
__device__ __forceinline__ int cell_coord(float v, float origin, float inv, int n) {
  float t = __fmul_rn(__fsub_rn(v, origin), inv);
  t = fminf(fmaxf(t, 0.f), float(n - 1));
  return int(t);
}

// Lower bound of cell C (1 <= C <= n - 1) on one axis: the smallest float v
// with cell_coord(v, origin, inv, n) >= C, i.e. with (v - origin) * inv >= C
// in the same round-to-nearest steps. That test is monotone in v, so a binary
// search over the floats in order (ordered bit patterns from -inf to +inf,
// -0 just below +0; no NaN lies between) finds v exactly in 32 steps. For a
// box of a replica in cell C, "C is the cell of the box's minimum" is then
// "minimum >= the lower bound of C": the cell of the minimum is at most C.
__device__ __forceinline__ float cell_lower_bound(int C, float origin, float inv) {
  auto ordered = [](float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  };
  auto from_ordered = [](uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
  };
  const float fc = float(C);
  uint32_t lo = ordered(-INFINITY), hi = ordered(INFINITY);  // test fails at lo, holds at hi
  while (hi - lo > 1u) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (__fmul_rn(__fsub_rn(from_ordered(mid), origin), inv) >= fc) hi = mid;
    else lo = mid;
  }
  return from_ordered(hi);
}

// ---- box type and pair filter ------------------------------------------------
// Type from the signs of vertexIds (src/aabb.cu:12-31): vertex {v,-v-1,-v-1}
// -> 0, edge {e0,e1,-e0-1} -> 1, face {f0,f1,f2} -> 2.
__device__ __forceinline__ int box_type(int v1, int v2) {
  return v2 >= 0 ? 2 : (v1 >= 0 ? 1 : 0);
}

// is_valid_pair (src/aabb.cu:33-40): V-F, F-V or E-E, i.e. types sum to 2.
__device__ __forceinline__ bool valid_pair(const int4 &a, const int4 &b) {
  return box_type(a.y, a.z) + box_type(b.y, b.z) == 2;
}

// covertex (src/collision.cu:44-48): any of the 9 id pairs equal.
__device__ __forceinline__ bool covertex(const int4 &a, const int4 &b) {
  return a.x == b.x || a.x == b.y || a.x == b.z || a.y == b.x || a.y == b.y ||
         a.y == b.z || a.z == b.x || a.z == b.y || a.z == b.z;
}

// does_collide(MiniBox) (src/collision.cu:38-42): inclusive overlap on the two
// non-sweep axes. Layout (min_b, min_c, max_b, max_c).
__device__ __forceinline__ bool overlap_bc(const float4 &a, const float4 &b) {
  return a.z >= b.x && a.x <= b.z && a.w >= b.y && a.y <= b.w;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace stq
