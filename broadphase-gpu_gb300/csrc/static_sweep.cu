// static_sweep.cu - the one entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a broad
// phase: simulation steps that run under a memory budget reserved up front
// (an out-of-memory error in the middle of a step is not recoverable for
// them), hosts whose own pooling allocator owns the device memory and forbids
// the CUDA runtime's, and real-time loops that cannot take the device-wide
// synchronisation cudaFree may cause. stq_sweep_static serves them: it sorts
// and sweeps one scene of at most STQ_STATIC_MAX_BOXES boxes using only the
// file-scope scratch array below, which every GPU that loads this library
// holds until the process exits. The caller passes the boxes and the pair
// buffer.
#include <mutex>

#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {
namespace {

constexpr int64_t kMax = STQ_STATIC_MAX_BOXES;
constexpr int64_t kSlots = kMax + 1 + kSortedPad;

// Byte layout of the scratch array (offsets are multiples of 256).
constexpr size_t up256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kOffKeys0 = 0;
constexpr size_t kOffKeys1 = kOffKeys0 + up256(sizeof(uint32_t) * kMax);
constexpr size_t kOffVals0 = kOffKeys1 + up256(sizeof(uint32_t) * kMax);
constexpr size_t kOffVals1 = kOffVals0 + up256(sizeof(uint32_t) * kMax);
constexpr size_t kOffSortWs = kOffVals1 + up256(sizeof(uint32_t) * kMax);
constexpr size_t kSortWsBytes = sizeof(uint32_t) * (256 * ((kMax + kRadixTile - 1) / kRadixTile) + 256) + 256;
constexpr size_t kOffXmin = kOffSortWs + up256(kSortWsBytes);
constexpr size_t kOffXmax = kOffXmin + up256(sizeof(float) * kSlots);
constexpr size_t kOffSyz = kOffXmax + up256(sizeof(float) * kSlots);
constexpr size_t kOffSv = kOffSyz + up256(sizeof(float4) * kSlots);
constexpr size_t kOffFlag = kOffSv + up256(sizeof(int4) * kSlots);
constexpr size_t kOffFloor = kOffFlag + up256(sizeof(int) * kSlots);
constexpr size_t kOffPartner = kOffFloor + up256(sizeof(float2) * kSlots);
constexpr size_t kOffHdr = kOffPartner + up256(sizeof(int) * kSlots);
constexpr size_t kOffScenePairs = kOffHdr + up256(sizeof(BatchHeader));
constexpr size_t kScratchBytes = kOffScenePairs + up256(sizeof(unsigned long long));

// The scratch of every stq_sweep_static call on this device (about 4.5 MB).
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// Writes the scene's sizes into the header (zeroed by the host before this
// launch, so the NaN flag that any block may set is never cleared after it),
// the sort keys and the box indices.
__global__ void static_keys_kernel(const stq_aabb *__restrict__ boxes, int n, int axis,
                                   unsigned char *scratch) {
  BatchHeader *hdr = reinterpret_cast<BatchHeader *>(scratch + kOffHdr);
  uint32_t *keys = reinterpret_cast<uint32_t *>(scratch + kOffKeys0);
  uint32_t *vals = reinterpret_cast<uint32_t *>(scratch + kOffVals0);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    hdr->n_boxes = n;
    hdr->n_scenes = 1;
    hdr->replicas = unsigned(n);
    hdr->cells = 1;
    hdr->length = unsigned(n);
  }
  bool nan = false;
  if (i < n) {
    const stq_aabb &b = boxes[i];
    for (int k = 0; k < 3; ++k) nan |= (b.min[k] != b.min[k]) | (b.max[k] != b.max[k]);
    keys[i] = float_key(b.min[axis]);
    vals[i] = uint32_t(i);
  }
  if (__any_sync(kFullMask, nan) && (threadIdx.x & 31) == 0) atomicOr(&hdr->flags, kFlagNaN);
}

// Sorted positions 0..n-1 (one cell), then the NaN sentinel and the padding.
__global__ void static_gather_kernel(const stq_aabb *__restrict__ boxes, int n, int axis,
                                     const uint32_t *__restrict__ order, unsigned char *scratch) {
  float *xmin = reinterpret_cast<float *>(scratch + kOffXmin);
  float *xmax = reinterpret_cast<float *>(scratch + kOffXmax);
  float4 *syz = reinterpret_cast<float4 *>(scratch + kOffSyz);
  int4 *sv = reinterpret_cast<int4 *>(scratch + kOffSv);
  int *sflag = reinterpret_cast<int *>(scratch + kOffFlag);
  float2 *sfloor = reinterpret_cast<float2 *>(scratch + kOffFloor);
  int *partner = reinterpret_cast<int *>(scratch + kOffPartner);
  const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const stq_aabb &x = boxes[order[k]];
    xmin[k] = x.min[axis];
    xmax[k] = x.max[axis];
    syz[k] = make_float4(x.min[b], x.min[c], x.max[b], x.max[c]);
    sv[k] = make_int4(x.vertex_ids[0], x.vertex_ids[1], x.vertex_ids[2], x.id);
    sflag[k] = 3;  // one cell: every box is in its first cell on both axes
    sfloor[k] = make_float2(-INFINITY, -INFINITY);
    partner[k] = k + 1;  // one list: candidates follow in sort order
  } else if (k < n + 1 + kSortedPad) {
    const float q = __int_as_float(0x7fc00000);
    xmin[k] = q;
    xmax[k] = q;
    partner[k] = k;
  }
}

std::mutex g_mutex;
void *g_scratch_ptr[256] = {};  // per device, set at the first call on it

}  // namespace
}  // namespace stq

extern "C" int stq_sweep_static(const stq_aabb *d_boxes, int64_t n, int axis, stq_pair *d_pairs,
                                int64_t capacity, int64_t *count, int64_t *total, void *stream) {
  using namespace stq;
  if (!count || n < 0) return STQ_ERR_INVALID_ARG;
  if (n > kMax) return STQ_ERR_CAPACITY;  // larger scenes need stq_sweep
  if (axis < 0 || axis > 2 || capacity < 0 || (n > 0 && !d_boxes) || (capacity > 0 && !d_pairs))
    return STQ_ERR_INVALID_ARG;
  *count = 0;
  if (total) *total = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return STQ_ERR_CUDA;
  unsigned char *scratch = nullptr;
  {
    // host code must not use g_static_scratch's address directly: look it up
    // once per device, with that device current
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev] &&
        cudaGetSymbolAddress(&g_scratch_ptr[dev], g_static_scratch) != cudaSuccess) {
      g_scratch_ptr[dev] = nullptr;
      return STQ_ERR_CUDA;
    }
    scratch = static_cast<unsigned char *>(g_scratch_ptr[dev]);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int ni = int(n);
  const int blocks = (ni + 1 + int(kSortedPad) + 255) / 256;
  // the header and the scene's pair counter start at zero (the array keeps
  // the last call's contents); a memset on the stream, not an allocation
  if (cudaMemsetAsync(scratch + kOffHdr, 0, kScratchBytes - kOffHdr, s) != cudaSuccess) return STQ_ERR_CUDA;
  static_keys_kernel<<<(ni + 255) / 256 > 0 ? (ni + 255) / 256 : 1, 256, 0, s>>>(d_boxes, ni, axis,
                                                                                   scratch);
  uint32_t *kb[2] = {reinterpret_cast<uint32_t *>(scratch + kOffKeys0),
                     reinterpret_cast<uint32_t *>(scratch + kOffKeys1)};
  uint32_t *vb[2] = {reinterpret_cast<uint32_t *>(scratch + kOffVals0),
                     reinterpret_cast<uint32_t *>(scratch + kOffVals1)};
  int which = 0;
  if (radix_sort_u32(s, kb, vb, n, 8, scratch + kOffSortWs, &which, nullptr) != cudaSuccess)
    return STQ_ERR_CUDA;
  static_gather_kernel<<<blocks, 256, 0, s>>>(d_boxes, ni, axis, vb[which], scratch);
  SweepParams p;
  p.xmin = reinterpret_cast<const float *>(scratch + kOffXmin);
  p.xmax = reinterpret_cast<const float *>(scratch + kOffXmax);
  p.syz = reinterpret_cast<const float4 *>(scratch + kOffSyz);
  p.sv = reinterpret_cast<const int4 *>(scratch + kOffSv);
  p.sflag = reinterpret_cast<const int *>(scratch + kOffFlag);
  p.sfloor = reinterpret_cast<const float2 *>(scratch + kOffFloor);
  p.partner = reinterpret_cast<const int *>(scratch + kOffPartner);
  p.run_end = nullptr;  // run ends are not computed here; the sweep takes the queue shape
  p.begin = 0;
  p.end = ni;
  p.chunk = 32;
  p.pairs = d_pairs;
  p.capacity = capacity;
  BatchHeader *hdr = reinterpret_cast<BatchHeader *>(scratch + kOffHdr);
  p.count = &hdr->pairs;
  p.work = &hdr->work;
  p.box_counts = nullptr;
  p.scene_pairs = reinterpret_cast<unsigned long long *>(scratch + kOffScenePairs);
  p.hdr = hdr;
  p.stats = nullptr;
  p.typed = 0;  // one list of all box types
  p.run_cap = 0;  // no warp pass: it would need a list of handed-over runs
  p.long_list = nullptr;
  p.long_items = nullptr;
  p.long_work = nullptr;
  int num_sms = 152;
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (launch_sweep(s, p, SweepTuning(), false, num_sms) != cudaSuccess) return STQ_ERR_CUDA;
  BatchHeader h;
  if (cudaMemcpyAsync(&h, hdr, sizeof(BatchHeader), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return STQ_ERR_CUDA;
  if (h.flags & kFlagNaN) return STQ_ERR_INVALID_INPUT;
  const int64_t found = int64_t(h.pairs);
  if (total) *total = found;
  *count = found < capacity ? found : capacity;
  return found <= capacity ? STQ_OK : STQ_OVERFLOW;
}
