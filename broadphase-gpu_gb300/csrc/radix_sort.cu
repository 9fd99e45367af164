// radix_sort.cu - stable LSD radix sort on the device.
//
// Replaces the comparison sort of the reference (thrust::sort_by_key with
// sort_aabb_x, src/simulation.cu:645-649, 277-293). Keys are the order-
// preserving uint32 images of the sweep-axis minima; values are box indices.
// Each pass is reduce-then-scan, with no inter-block waiting:
//   upsweep   per-tile digit histogram          (reads keys)
//   scan      per-digit exclusive scan over tiles, then over digit totals
//   downsweep stable in-tile ranking (warp match_any + per-warp counters),
//             staging in shared memory by digit, coalesced scatter
#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {

namespace {

constexpr int kSortBlock = 256;
constexpr int kSortWarps = kSortBlock / 32;

template <typename K> struct TileShape {
  static constexpr int items = 8;  // 16 for 4-byte keys needs 89 registers: 2 blocks per SM
  static constexpr int tile = kSortBlock * items;
};
static_assert(TileShape<uint32_t>::tile == kRadixTile && TileShape<unsigned long long>::tile == kRadixTile,
              "radix tile of the workspace sizing");

int64_t num_tiles(int64_t n, int tile) { return (n + tile - 1) / tile; }

// A pass whose digit is 0 in every key: d_hi counts the distinct values of
// the keys' bits from begin_bit up, rel = shift - begin_bit.
__device__ __forceinline__ bool pass_is_identity(const unsigned int *d_hi, int rel) {
  if (!d_hi) return false;
  const unsigned int hi = *d_hi;
  return rel >= 32 || hi <= 1u || ((hi - 1u) >> rel) == 0u;
}

template <typename K, int BITS>
__global__ void __launch_bounds__(kSortBlock)
upsweep_kernel(const K *__restrict__ keys, int64_t n, int shift,
               uint32_t *__restrict__ hist, int64_t ntiles, const unsigned int *d_n, bool match,
               const unsigned int *d_hi, int rel) {
  if (pass_is_identity(d_hi, rel)) return;  // the scatter copies the keys through
  if (d_n && int64_t(*d_n) < n) n = *d_n;
  constexpr int BINS = 1 << BITS;
  constexpr int TILE = TileShape<K>::tile;
  constexpr int ITEMS = TILE / kSortBlock;
  __shared__ uint32_t h[kSortWarps][BINS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kSortWarps * BINS; i += kSortBlock) (&h[0][0])[i] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * TILE;
  int d[ITEMS];  // all loads first
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const int64_t idx = base + int64_t(i) * kSortBlock + threadIdx.x;
    d[i] = idx < n ? int((keys[idx] >> shift) & (BINS - 1)) : BINS;
  }
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    // a warp whose digits are all equal adds once; a digit that repeats
    // within warps (the top byte of float keys: sign and exponent) is
    // counted per distinct value; other digits by one shared atomic each
    const int d0 = __shfl_sync(kFullMask, d[i], 0);
    if (__all_sync(kFullMask, d[i] == d0)) {
      if (lane == 0 && d0 < BINS) atomicAdd(&h[warp][d0], 32u);
    } else if (match) {
      const unsigned peers = __match_any_sync(kFullMask, d[i]);
      if (d[i] < BINS && lane == __ffs(peers) - 1) atomicAdd(&h[warp][d[i]], __popc(peers));
    } else if (d[i] < BINS) {
      atomicAdd(&h[warp][d[i]], 1u);
    }
  }
  __syncthreads();
  for (int dg = threadIdx.x; dg < BINS; dg += kSortBlock) {
    uint32_t t = 0;
    for (int w = 0; w < kSortWarps; ++w) t += h[w][dg];
    hist[int64_t(dg) * ntiles + blockIdx.x] = t;
  }
}

// Block-wide exclusive scan of one value per thread (kSortBlock threads).
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total, uint32_t *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFullMask, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) scratch[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kSortWarps ? scratch[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFullMask, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kSortWarps) scratch[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t warp_base = warp > 0 ? scratch[warp - 1] : 0;
  *total = scratch[kSortWarps - 1];
  __syncthreads();
  return warp_base + x - v;
}

// Exclusive scan of in[b, b + 2048) (clipped to n) into out, starting from
// carry, by one block with 8 entries per thread: coalesced loads into shared
// memory, each thread scans 8 consecutive entries (padded indices: no bank
// conflicts), one block scan. Returns the chunk's total (in every thread).
constexpr int kChunkPer = 8, kChunk = kSortBlock * kChunkPer;
__device__ uint32_t scan_chunk(const uint32_t *in, uint32_t *out, int64_t b, int64_t n, uint32_t carry) {
  __shared__ uint32_t buf[kChunk + kChunk / 32];
  __shared__ uint32_t scratch[32];
  auto at = [](int x) { return x + (x >> 5); };
#pragma unroll
  for (int i = 0; i < kChunkPer; ++i) {
    const int x = i * kSortBlock + threadIdx.x;
    buf[at(x)] = b + x < n ? in[b + x] : 0u;
  }
  __syncthreads();
  uint32_t v[kChunkPer], sum = 0;
#pragma unroll
  for (int i = 0; i < kChunkPer; ++i) {
    v[i] = buf[at(threadIdx.x * kChunkPer + i)];
    sum += v[i];
  }
  uint32_t tot;
  uint32_t run = carry + block_exclusive_scan(sum, &tot, scratch);
#pragma unroll
  for (int i = 0; i < kChunkPer; ++i) {
    buf[at(threadIdx.x * kChunkPer + i)] = run;
    run += v[i];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kChunkPer; ++i) {
    const int x = i * kSortBlock + threadIdx.x;
    if (b + x < n) out[b + x] = buf[at(x)];
  }
  __syncthreads();  // the next chunk overwrites buf
  return tot;
}

// Exclusive scan of row[0..n) in place by one block; returns the total.
__device__ uint32_t block_scan_row(uint32_t *row, int64_t n) {
  uint32_t carry = 0;
  for (int64_t b = 0; b < n; b += kChunk) carry += scan_chunk(row, row, b, n, carry);
  return carry;
}

// One block per digit: exclusive scan of hist[d][0..ntiles) in place.
__global__ void __launch_bounds__(kSortBlock)
scan_rows_kernel(uint32_t *__restrict__ hist, int64_t ntiles,
                 uint32_t *__restrict__ totals) {
  const uint32_t total = block_scan_row(hist + int64_t(blockIdx.x) * ntiles, ntiles);
  if (threadIdx.x == 0) totals[blockIdx.x] = total;
}

template <int BINS>
__global__ void __launch_bounds__(kSortBlock)
scan_totals_kernel(uint32_t *__restrict__ totals) {
  __shared__ uint32_t scratch[32];
  const uint32_t v = threadIdx.x < BINS ? totals[threadIdx.x] : 0;
  uint32_t tot;
  const uint32_t ex = block_exclusive_scan(v, &tot, scratch);
  if (threadIdx.x < BINS) totals[threadIdx.x] = ex;
}

template <typename K, int BITS, bool VALS>
__global__ void __launch_bounds__(kSortBlock)
downsweep_kernel(const K *__restrict__ kin, K *__restrict__ kout,
                 const uint32_t *__restrict__ vin, uint32_t *__restrict__ vout,
                 int64_t n, int shift, const uint32_t *__restrict__ tile_off,
                 const uint32_t *__restrict__ digit_base, int64_t ntiles,
                 const unsigned int *d_n, const unsigned int *d_hi, int rel) {
  if (d_n && int64_t(*d_n) < n) n = *d_n;
  constexpr int BINS = 1 << BITS;
  constexpr int ITEMS = TileShape<K>::items;
  constexpr int TILE = TileShape<K>::tile;
  if (pass_is_identity(d_hi, rel)) {
    // every key's digit is 0: the stable pass is the identity; copy the tile
    const int64_t t0 = int64_t(blockIdx.x) * TILE;
    for (int64_t i = t0 + threadIdx.x; i < n && i < t0 + TILE; i += kSortBlock) {
      kout[i] = kin[i];
      if (VALS) vout[i] = vin[i];
    }
    return;
  }
  __shared__ uint32_t cnt[kSortWarps][BINS + 1];
  __shared__ uint32_t tile_prefix[BINS];
  __shared__ uint32_t gbase[BINS];
  __shared__ uint32_t scratch[32];
  __shared__ K stage[TILE];
  __shared__ uint32_t vstage[VALS ? TILE : 1];
  __shared__ uint8_t stage_d[TILE];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile_start = int64_t(blockIdx.x) * TILE;
  const int64_t wstart = tile_start + int64_t(warp) * 32 * ITEMS;
  for (int i = threadIdx.x; i < kSortWarps * (BINS + 1); i += kSortBlock) (&cnt[0][0])[i] = 0;
  __syncthreads();

  K key[ITEMS];
  uint32_t val[ITEMS];
  int dig[ITEMS];
  uint32_t rank[ITEMS];
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const int64_t idx = wstart + it * 32 + lane;
    if (idx < n) {
      key[it] = kin[idx];
      if (VALS) val[it] = vin[idx];
      dig[it] = int((key[it] >> shift) & (BINS - 1));
    } else {
      dig[it] = BINS;  // dummy bin: counted, never written
    }
  }
  // Stable in-warp ranking: items in input order, lanes in input order.
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    const unsigned peers = __match_any_sync(kFullMask, dig[it]);
    const uint32_t base = cnt[warp][dig[it]];
    __syncwarp();
    if (lane == __ffs(peers) - 1) cnt[warp][dig[it]] = base + __popc(peers);
    __syncwarp();
    rank[it] = base + __popc(peers & lanemask_lt());
  }
  __syncthreads();
  // Per digit: exclusive prefix over warps and the digit's tile total.
  uint32_t dtotal = 0;
  if (threadIdx.x < BINS) {
    uint32_t run = 0;
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = cnt[w][threadIdx.x];
      cnt[w][threadIdx.x] = run;
      run += c;
    }
    dtotal = run;
  }
  __syncthreads();
  uint32_t tot;
  const uint32_t ex = block_exclusive_scan(dtotal, &tot, scratch);
  if (threadIdx.x < BINS) {
    tile_prefix[threadIdx.x] = ex;
    gbase[threadIdx.x] =
        digit_base[threadIdx.x] + tile_off[int64_t(threadIdx.x) * ntiles + blockIdx.x];
  }
  __syncthreads();
  // Stage keys and values in tile-sorted order, then write both out digit run
  // by run (one destination per staged element).
#pragma unroll
  for (int it = 0; it < ITEMS; ++it) {
    if (dig[it] < BINS) {
      const int pos = int(tile_prefix[dig[it]] + cnt[warp][dig[it]] + rank[it]);
      stage[pos] = key[it];
      if (VALS) vstage[pos] = val[it];
      stage_d[pos] = uint8_t(dig[it]);
    }
  }
  __syncthreads();
  const int count = int(n - tile_start < TILE ? (n > tile_start ? n - tile_start : 0) : TILE);
  for (int p = threadIdx.x; p < count; p += kSortBlock) {
    const int d = stage_d[p];
    const uint32_t o = gbase[d] + (p - tile_prefix[d]);
    kout[o] = stage[p];
    if (VALS) vout[o] = vstage[p];
  }
}

template <typename K, int BITS, bool VALS>
cudaError_t sort_impl(cudaStream_t s, K *kbuf[2], uint32_t *vbuf[2], int64_t n,
                      int begin_bit, int end_bit, void *workspace, int *which,
                      int64_t *launches, const unsigned int *d_n = nullptr,
                      const unsigned int *d_hi = nullptr) {
  constexpr int BINS = 1 << BITS;
  constexpr int TILE = TileShape<K>::tile;
  *which = 0;
  if (n <= 1) return cudaSuccess;
  const int64_t ntiles = num_tiles(n, TILE);
  uint32_t *hist = static_cast<uint32_t *>(workspace);
  uint32_t *totals = hist + int64_t(BINS) * ntiles;
  int cur = 0;
  for (int shift = begin_bit; shift < end_bit; shift += BITS) {
    // the top digit of 4-byte keys (float sign and exponent) repeats within warps
    const bool match = sizeof(K) == 4 && shift + BITS >= 32;
    upsweep_kernel<K, BITS><<<unsigned(ntiles), kSortBlock, 0, s>>>(kbuf[cur], n, shift,
                                                                     hist, ntiles, d_n, match, d_hi,
                                                                     shift - begin_bit);
    scan_rows_kernel<<<BINS, kSortBlock, 0, s>>>(hist, ntiles, totals);
    scan_totals_kernel<BINS><<<1, kSortBlock, 0, s>>>(totals);
    downsweep_kernel<K, BITS, VALS><<<unsigned(ntiles), kSortBlock, 0, s>>>(
        kbuf[cur], kbuf[cur ^ 1], VALS ? vbuf[cur] : nullptr,
        VALS ? vbuf[cur ^ 1] : nullptr, n, shift, hist, totals, ntiles, d_n, d_hi, shift - begin_bit);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (launches) *launches += 4;
    cur ^= 1;
  }
  *which = cur;
  return cudaSuccess;
}

}  // namespace

size_t radix_workspace_bytes(int64_t n, int key_bytes, int bits) {
  const int tile = key_bytes == 4 ? TileShape<uint32_t>::tile : TileShape<unsigned long long>::tile;
  const int64_t ntiles = num_tiles(n > 0 ? n : 1, tile);
  return sizeof(uint32_t) * (size_t(1 << bits) * ntiles + (1 << bits)) + 256;
}

cudaError_t radix_sort_u32(cudaStream_t s, uint32_t *kbuf[2], uint32_t *vbuf[2],
                           int64_t n, int bits, void *workspace, int *which,
                           int64_t *launches, const unsigned int *d_n) {
  if (bits == 4)
    return sort_impl<uint32_t, 4, true>(s, kbuf, vbuf, n, 0, 32, workspace, which, launches, d_n);
  return sort_impl<uint32_t, 8, true>(s, kbuf, vbuf, n, 0, 32, workspace, which, launches, d_n);
}

cudaError_t radix_sort_u64(cudaStream_t s, unsigned long long *kbuf[2], int64_t n,
                           int begin_bit, int end_bit, void *workspace, int *which,
                           int64_t *launches) {
  return sort_impl<unsigned long long, 8, false>(s, kbuf, nullptr, n, begin_bit, end_bit,
                                                 workspace, which, launches);
}

cudaError_t radix_sort_u64_vals(cudaStream_t s, unsigned long long *kbuf[2], uint32_t *vbuf[2],
                                int64_t n, int begin_bit, int end_bit, void *workspace,
                                int *which, int64_t *launches, const unsigned int *d_n,
                                int bits, const unsigned int *d_hi) {
  if (bits == 4)
    return sort_impl<unsigned long long, 4, true>(s, kbuf, vbuf, n, begin_bit, end_bit,
                                                  workspace, which, launches, d_n, d_hi);
  return sort_impl<unsigned long long, 8, true>(s, kbuf, vbuf, n, begin_bit, end_bit,
                                                workspace, which, launches, d_n, d_hi);
}

// ---- exclusive scan of uint32 counts (reduce-then-scan, no waiting) -------------
namespace {

constexpr int kScanItems = 8;
constexpr int kScanTile = kSortBlock * kScanItems;

__global__ void __launch_bounds__(kSortBlock)
scan_reduce_kernel(const uint32_t *__restrict__ in, int64_t n, uint32_t *__restrict__ sums) {
  __shared__ uint32_t scratch[32];
  const int64_t base = int64_t(blockIdx.x) * kScanTile + threadIdx.x;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)  // coalesced; a sum needs no order
    if (base + i * kSortBlock < n) s += in[base + i * kSortBlock];
  uint32_t tot;
  block_exclusive_scan(s, &tot, scratch);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kSortBlock)
scan_sums_kernel(uint32_t *__restrict__ sums, int64_t ntiles, uint32_t *__restrict__ total) {
  const uint32_t t = block_scan_row(sums, ntiles);
  if (threadIdx.x == 0) *total = t;
}

__global__ void __launch_bounds__(kSortBlock)
scan_apply_kernel(const uint32_t *__restrict__ in, int64_t n, const uint32_t *__restrict__ sums,
                  uint32_t *__restrict__ out) {
  static_assert(kScanTile == kChunk, "one chunk per scan tile");
  scan_chunk(in, out, int64_t(blockIdx.x) * kScanTile, n, sums[blockIdx.x]);
}

}  // namespace

size_t scan_workspace_bytes(int64_t n) {
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  return sizeof(uint32_t) * size_t(ntiles + 1);
}

cudaError_t exclusive_scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n,
                               void *workspace, uint32_t *d_total, int64_t *launches) {
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  uint32_t *sums = static_cast<uint32_t *>(workspace);
  if (n > 0) scan_reduce_kernel<<<unsigned(ntiles), kSortBlock, 0, s>>>(in, n, sums);
  scan_sums_kernel<<<1, kSortBlock, 0, s>>>(sums, ntiles, d_total);
  if (n > 0) scan_apply_kernel<<<unsigned(ntiles), kSortBlock, 0, s>>>(in, n, sums, out);
  if (launches) *launches += n > 0 ? 3 : 1;
  return cudaGetLastError();
}

}  // namespace stq
