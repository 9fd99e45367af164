// sweep.cu - the sweep-and-tiniest-queue pass, pair compaction, the
// overflow prefix selection and the all-pairs checker.
//
// Reference: twostage_queue (src/sweep.cu:226-279) with its shared Queue
// (src/queue.cuh:9-38, src/queue.cu:75-115), does_collide / covertex /
// is_valid_pair (src/collision.cu:38-48, src/aabb.cu:33-40) and add_overlap
// (src/collision.cu:50-74).
//
// GB300 design. A start box k's candidates are its x-run
// j = partner[k], partner[k]+1, ... up to the first j whose min exceeds k's
// max (a NaN sentinel ends every list); partner[k] is k+1 for an edge, and the
// first face (for a vertex) or vertex (for a face) of the same cell's list at
// or after k's min. Two shapes walk the runs:
//   - queue (stq_sweep_lane_kernel, stq_sweep_kernel): each warp owns a
//     shared-memory ring of pending start boxes (the "tiniest queue"); a lane,
//     or a group of G lanes, takes one start box from the ring and walks its
//     run, and takes the next pending box when the run ends, so a long run
//     never stalls the others;
//   - flat (stq_sweep_flat_kernel, the default): the gather has found every
//     run's end (run_end), so a warp lays the runs of 32 consecutive start
//     positions end to end and tests one candidate per lane and step.
// Runs longer than a cap go to a warp pass (stq_long_run_kernel). Refill,
// hand-out and pair output use __ballot_sync/__popc compaction: no
// shared-memory atomics, and one global atomic per 32 or more pairs.
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "stq_device.cuh"
#include "stq_internal.h"

namespace stq {

namespace {

// Appends the warp's n staged pairs with one atomic; pairs past the capacity
// are counted but not written.
__device__ __forceinline__ void flush_staged(const int2 *st, int n, int lane, const SweepParams &p) {
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(p.count, (unsigned long long)n);
  base = __shfl_sync(kFullMask, base, 0);
  int2 *out = reinterpret_cast<int2 *>(p.pairs);
  for (int i = lane; i < n; i += 32)
    if (base + i < (unsigned long long)p.capacity) out[base + i] = st[i];
  __syncwarp();
}

template <int G, int Q, int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK)
stq_sweep_kernel(const SweepParams p) {
  static_assert(32 % G == 0, "lane group must divide the warp");
  // the refill tops the ring up to one entry per group: Q >= 32 / G
  static_assert((Q & (Q - 1)) == 0 && Q >= 16 && Q >= 32 / G, "queue depth: power of two >= 16 and >= groups");
  constexpr int E = 32 / G;  // lane groups per warp
  constexpr int STAGE = 64;  // pairs staged per warp before one global append
  __shared__ int ring[BLOCK / 32][Q];
  __shared__ int2 stage[COUNT ? 1 : BLOCK / 32][COUNT ? 1 : STAGE];

  const int lane = threadIdx.x & 31;
  const int gl = lane % G;              // lane within group
  const int grp = lane / G;             // group within warp
  const unsigned grp_mask = G == 32 ? kFullMask : (((1u << G) - 1u) << (grp * G));
  const unsigned upto_me = grp_mask & (lane == 31 ? kFullMask : ((2u << lane) - 1u));
  const unsigned leaders_below = (grp * G) == 0 ? 0u : ((1u << (grp * G)) - 1u);
  int *q = ring[threadIdx.x >> 5];

  // warp-uniform queue and work state
  int qhead = 0, qsize = 0;
  int next_k = 0, chunk_end = 0;
  bool more = true;
  // lane-group state (identical in the G lanes of a group)
  int k = -1, j0 = 0, acc = 0, taken = 0;
  float kmax = 0.f;
  float4 kb = make_float4(0.f, 0.f, 0.f, 0.f);
  int4 kv = make_int4(0, 0, 0, 0);
  float2 kfl = make_float2(0.f, 0.f);  // first-cell rule of the current start box
  const int end = min(p.end, int(p.hdr->length));
  const int span = end - p.begin;
  int kf = 0;  // scene of the current start box (above the first-cell bits)
  unsigned tested = 0;  // candidates this lane tested (statistics)
  // warp-uniform: staged pairs, and pairs of the current scene not yet added
  // to its counter
  int staged = 0;
  int wscene = 0;
  unsigned long long wpairs = 0;
  const bool multi = p.hdr->n_scenes > 1;  // per-scene counts need the scene of each hit
  int2 *st = stage[COUNT ? 0 : (threadIdx.x >> 5)];

  while (true) {
    // 1. Refill the ring with start boxes that have at least one candidate.
    while (qsize < E && more) {
      if (next_k >= chunk_end) {
        int c = 0;
        if (lane == 0) c = atomicAdd(p.work, p.chunk);
        c = __shfl_sync(kFullMask, c, 0);
        if (c >= span) {
          more = false;
          break;
        }
        next_k = p.begin + c;
        chunk_end = min(next_k + p.chunk, end);
      }
      const int take = min(32, min(Q - qsize, chunk_end - next_k));
      const int kk = next_k + lane;
      bool push = false;
      if (lane < take) push = p.xmin[p.partner[kk]] <= p.xmax[kk];
      const unsigned m = __ballot_sync(kFullMask, push);
      if (push) q[(qhead + qsize + __popc(m & lanemask_lt())) & (Q - 1)] = kk;
      qsize += __popc(m);
      next_k += take;
    }
    __syncwarp();
    // 2. Idle groups take pending start boxes, in ring order.
    const bool idle = k < 0;
    const unsigned needm = __ballot_sync(kFullMask, idle && gl == 0);
    const int ntake = min(__popc(needm), qsize);
    if (idle) {
      const int r = __popc(needm & leaders_below);
      if (r < ntake) {
        k = q[(qhead + r) & (Q - 1)];
        j0 = p.partner[k];
        kmax = p.xmax[k];
        kb = p.syz[k];
        kv = p.sv[k];
        kfl = p.sfloor[k];
        acc = 0;
        taken = 0;
        kf = multi ? p.sflag[k] : 0;
      }
    }
    qhead = (qhead + ntake) & (Q - 1);
    qsize -= ntake;
    __syncwarp();
    const bool active = k >= 0;
    if (__ballot_sync(kFullMask, active) == 0) {
      if (!more && qsize == 0) break;
      continue;
    }
    // 3. Test G consecutive candidates per group. Valid lanes form the
    //    prefix of the group before the first x-test failure.
    const int j = j0 + gl;
    const bool xok = active && p.xmin[j] <= kmax;
    const unsigned failm = __ballot_sync(kFullMask, active && !xok);
    const bool valid = active && (failm & upto_me) == 0;
    bool hit = false;
    int lo_id = 0, hi_id = 0;
    if (valid) {
      ++tested;
      const float4 b = p.syz[j];
      // a pair found in several cells is emitted only in the cell of its
      // reference point: on b and on c, one of the two replicas must be its
      // box's first cell (the candidate's: minimum >= the cell's lower bound)
      if (overlap_bc(kb, b) && b.x >= kfl.x && b.y >= kfl.y) {  // ids only for these
        const int4 bv = p.sv[j];
        hit = (p.typed || valid_pair(kv, bv)) && !covertex(kv, bv);
        lo_id = min(kv.w, bv.w);
        hi_id = max(kv.w, bv.w);
      }
    }
    // 4. Emit: compact the step's hits into the warp's staging buffer; append
    //    it to the pair list with one global atomic per 32 or more pairs.
    const unsigned hm = __ballot_sync(kFullMask, hit);
    const int ghits = __popc(hm & grp_mask);
    if (COUNT) {
      acc += ghits;
    } else if (hm) {
      if (hit) st[staged + __popc(hm & lanemask_lt())] = make_int2(lo_id, hi_id);
      staged += __popc(hm);
      // per-scene counts: one register while the warp stays in one scene
      if (!multi) {
        wpairs += __popc(hm);
      } else {
        const int lead = __shfl_sync(kFullMask, kf >> 2, __ffs(hm) - 1);
        if (__all_sync(kFullMask, !hit || (kf >> 2) == lead)) {
          if (lead != wscene) {
            if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
            wscene = lead;
            wpairs = 0;
          }
          wpairs += __popc(hm);
        } else if (gl == 0 && ghits) {
          atomicAdd(&p.scene_pairs[kf >> 2], (unsigned long long)ghits);
        }
      }
      if (staged >= 32) {
        __syncwarp();
        flush_staged(st, staged, lane, p);
        staged = 0;
      }
    }
    // 5. A group whose G lanes all passed continues; otherwise its run ended.
    const unsigned vm = __ballot_sync(kFullMask, valid);
    if (active) {
      if ((vm & grp_mask) == grp_mask) {
        j0 += G;
        taken += G;
        if (p.run_cap && taken >= p.run_cap) {  // a long run: the warp pass takes the rest
          if (gl == 0) {
            p.long_list[atomicAdd(p.long_items, 1u)] = make_int2(k, j0);
            if (COUNT) p.box_counts[k - p.begin] = acc;
          }
          k = -1;
        }
      } else {
        if (COUNT && gl == 0) p.box_counts[k - p.begin] = acc;
        k = -1;
      }
    }
  }
  if (!COUNT) {
    __syncwarp();
    if (staged) flush_staged(st, staged, lane, p);
    if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
    const unsigned t = __reduce_add_sync(kFullMask, tested);
    if (lane == 0 && p.stats) atomicAdd(p.stats, (unsigned long long)t);
  }
}

// One start box per lane. A lane walks its own run, U consecutive candidates
// per step: the U minima are loaded together (U independent loads in flight
// per lane), the valid ones are the prefix before the first x-test failure
// (lane-local: no ballot), and a lane whose run ended takes the next pending
// box from the warp's ring. Otherwise as stq_sweep_kernel: ring refill by
// ballot compaction, lazy vertex-id loads, per-warp staging of pairs.
template <int U, int Q, int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK)
stq_sweep_lane_kernel(const SweepParams p) {
  static_assert(U == 1 || U == 2 || U == 4 || U == 8, "candidates per lane step: 1, 2, 4 or 8");
  static_assert((Q & (Q - 1)) == 0 && Q >= 32, "queue depth: power of two >= 32");
  constexpr int STAGE = 32 * (U + 1);  // < 32 left over + at most 32 * U new pairs
  // A ring entry carries the partner the refill read for its start box, so a
  // take starts the candidate loads without a dependent global load; where
  // that would pass 48 KB of shared memory the entry is the start box alone.
  constexpr bool kWide = (BLOCK / 32) * (Q * 8 + STAGE * 8) <= 48 * 1024;
  using Entry = typename std::conditional<kWide, int2, int>::type;
  __shared__ Entry ring[BLOCK / 32][Q];
  __shared__ int2 stage[COUNT ? 1 : BLOCK / 32][COUNT ? 1 : STAGE];

  const int lane = threadIdx.x & 31;
  const unsigned below = lanemask_lt();
  Entry *q = ring[threadIdx.x >> 5];
  int2 *st = stage[COUNT ? 0 : (threadIdx.x >> 5)];

  int qhead = 0, qsize = 0;
  int next_k = 0, chunk_end = 0;
  bool more = true;
  int k = -1, j = 0, acc = 0, kf = 0, taken = 0;
  float kmax = 0.f;
  float4 kb = make_float4(0.f, 0.f, 0.f, 0.f);
  int4 kv = make_int4(0, 0, 0, 0);
  float2 kfl = make_float2(0.f, 0.f);  // first-cell rule of the start box
  const int end = min(p.end, int(p.hdr->length));
  const int span = end - p.begin;
  unsigned tested = 0;
  int staged = 0;
  int wscene = 0;
  unsigned long long wpairs = 0;
  const bool multi = p.hdr->n_scenes > 1;

  while (true) {
    // 1. Refill the ring with start boxes that have at least one candidate.
    while (qsize < 32 && more) {
      if (next_k >= chunk_end) {
        int c = 0;
        if (lane == 0) c = atomicAdd(p.work, p.chunk);
        c = __shfl_sync(kFullMask, c, 0);
        if (c >= span) {
          more = false;
          break;
        }
        next_k = p.begin + c;
        chunk_end = min(next_k + p.chunk, end);
      }
      const int take = min(32, min(Q - qsize, chunk_end - next_k));
      const int kk = next_k + lane;
      bool push = false;
      int pk = 0;
      if (lane < take) {
        pk = p.partner[kk];
        push = p.xmin[pk] <= p.xmax[kk];
      }
      const unsigned m = __ballot_sync(kFullMask, push);
      if (push) {
        Entry &slot = q[(qhead + qsize + __popc(m & below)) & (Q - 1)];
        if constexpr (kWide) slot = make_int2(kk, pk);
        else slot = kk;
      }
      qsize += __popc(m);
      next_k += take;
    }
    __syncwarp();
    // 2. Idle lanes take pending start boxes, in ring order.
    const unsigned needm = __ballot_sync(kFullMask, k < 0);
    const int ntake = min(__popc(needm), qsize);
    if (k < 0) {
      const int r = __popc(needm & below);
      if (r < ntake) {
        const Entry e = q[(qhead + r) & (Q - 1)];
        if constexpr (kWide) {
          k = e.x;
          j = e.y;
        } else {
          k = e;
          j = p.partner[k];
        }
        kmax = p.xmax[k];
        kb = p.syz[k];
        kv = p.sv[k];
        kfl = p.sfloor[k];
        kf = multi ? p.sflag[k] : 0;
        acc = 0;
        taken = 0;
      }
    }
    qhead = (qhead + ntake) & (Q - 1);
    qsize -= ntake;
    __syncwarp();
    const bool active = k >= 0;
    if (__ballot_sync(kFullMask, active) == 0) {
      if (!more && qsize == 0) break;
      continue;
    }
    // 3. U candidates of the lane's run: the valid ones are the prefix before
    //    the first x-test failure (a NaN sentinel ends every list).
    float xm[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xm[u] = active ? p.xmin[j + u] : 0.f;
    int nvalid = 0;
    if (active) {
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (nvalid == u && xm[u] <= kmax) ++nvalid;
    }
    tested += unsigned(nvalid);
    // hits as bits; a hit's id is loaded again on output (an L1 hit) rather
    // than kept in registers for the whole step
    unsigned hits = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u < nvalid) {
        const float4 b = p.syz[j + u];
        if (overlap_bc(kb, b) && b.x >= kfl.x && b.y >= kfl.y) {  // and the first-cell rule
          const int4 bv = p.sv[j + u];
          if ((p.typed || valid_pair(kv, bv)) && !covertex(kv, bv)) hits |= 1u << u;
        }
      }
    }
    // 4. Emit the step's hits through the warp's staging buffer.
    const int nh = __popc(hits);
    if (COUNT) {
      acc += nh;
    } else {
      const unsigned anym = __ballot_sync(kFullMask, nh > 0);
      if (anym) {
        int total = 0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const bool hit = (hits >> u) & 1u;
          const unsigned hm = __ballot_sync(kFullMask, hit);
          if (hit) {
            const int id = p.sv[j + u].w;
            st[staged + __popc(hm & below)] = make_int2(min(kv.w, id), max(kv.w, id));
          }
          staged += __popc(hm);
          total += __popc(hm);
        }
        // per-scene counts: one register while the warp stays in one scene
        if (!multi) {
          wpairs += unsigned(total);
        } else {
          const int lead = __shfl_sync(kFullMask, kf >> 2, __ffs(anym) - 1);
          if (__all_sync(kFullMask, nh == 0 || (kf >> 2) == lead)) {
            if (lead != wscene) {
              if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
              wscene = lead;
              wpairs = 0;
            }
            wpairs += unsigned(total);
          } else if (nh) {
            atomicAdd(&p.scene_pairs[kf >> 2], (unsigned long long)nh);
          }
        }
        if (staged >= 32) {
          __syncwarp();
          flush_staged(st, staged, lane, p);
          staged = 0;
        }
      }
    }
    // 5. A lane whose U candidates all passed continues; otherwise its run ended.
    if (active) {
      if (nvalid == U) {
        j += U;
        taken += U;
        if (p.run_cap && taken >= p.run_cap) {  // a long run: the warp pass takes the rest
          p.long_list[atomicAdd(p.long_items, 1u)] = make_int2(k, j);
          if (COUNT) p.box_counts[k - p.begin] = acc;
          k = -1;
        }
      } else {
        if (COUNT) p.box_counts[k - p.begin] = acc;
        k = -1;
      }
    }
  }
  if (!COUNT) {
    __syncwarp();
    if (staged) flush_staged(st, staged, lane, p);
    if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
    const unsigned t = __reduce_add_sync(kFullMask, tested);
    if (lane == 0 && p.stats) atomicAdd(p.stats, (unsigned long long)t);
  }
}

// Flat shape. A warp takes 32 consecutive start positions; each one's run on
// the sweep axis is [partner, run_end), both found by the gather (runs longer
// than run_cap are cut there and the rest goes to the warp pass). The runs of
// the starts that have candidates are laid end to end, and the warp walks
// that flat sequence 32 candidates per step, one per lane: lane l of the step
// at `base` takes flat candidate f = base + l, whose start is the last one
// whose run begins at or before f (a bit mask of the run beginnings inside the
// step, one OR-reduction, and a population count). Consecutive lanes read
// consecutive positions of a run, and every lane works except in the last
// step of the 32 starts.
// Two passes per warp. The filter tests the y/z overlap and the first-cell
// rule on the candidate's (min_b, min_c, max_b, max_c) record, V steps with
// their loads issued together, and compacts the candidates that pass into a
// per-warp shared-memory queue. Once 32 are queued, the check takes them one
// per lane: the vertex ids of both boxes, is_valid_pair and covertex, and the
// hits go through the staging buffer as in the other shapes. The starts'
// records sit in shared memory, so the queue is drained before the next 32
// starts replace them.
struct FlatStart {
  float4 kb;   // start box (min_b, min_c, max_b, max_c)
  float2 kfl;  // first-cell rule
  int joff;    // position of flat candidate f is joff + f
  int kf;      // first-cell bits and scene
  int4 kv;     // vertex ids and id
};
static_assert(sizeof(FlatStart) == 48, "FlatStart: three 16-byte words");

template <int BLOCK, int V>
__global__ void __launch_bounds__(BLOCK)
stq_sweep_flat_kernel(const SweepParams p) {
  constexpr int STAGE = 64;  // < 32 left over + at most 32 new pairs per check
  constexpr int QUEUE = 32 * (V + 1);  // < 32 left over + at most 32 * V per filter round
  __shared__ FlatStart recs[BLOCK / 32][32];
  __shared__ int2 stage[BLOCK / 32][STAGE];
  __shared__ int2 queue[BLOCK / 32][QUEUE];  // (start record, candidate position)

  const int lane = threadIdx.x & 31;
  const unsigned below = lanemask_lt();
  const unsigned upto = below | (1u << lane);
  FlatStart *rec = recs[threadIdx.x >> 5];
  int2 *st = stage[threadIdx.x >> 5];
  int2 *qu = queue[threadIdx.x >> 5];

  const int end = min(p.end, int(p.hdr->length));
  const int span = end - p.begin;
  const bool multi = p.hdr->n_scenes > 1;
  int next_k = 0, chunk_end = 0;
  unsigned long long tested = 0;  // warp-uniform
  int staged = 0, queued = 0;
  int wscene = 0;
  unsigned long long wpairs = 0;

  // the check of n <= 32 queued candidates (the last n entries)
  auto check = [&](int n) {
    bool hit = false;
    int2 pr = make_int2(0, 0);
    int kf = 0;
    if (lane < n) {
      const int2 e = qu[queued - n + lane];
      const int4 bv = p.sv[e.y];
      const int4 kv = rec[e.x].kv;
      if (multi) kf = rec[e.x].kf;
      hit = (p.typed || valid_pair(kv, bv)) && !covertex(kv, bv);
      pr = make_int2(min(kv.w, bv.w), max(kv.w, bv.w));
    }
    queued -= n;
    const unsigned hm = __ballot_sync(kFullMask, hit);
    if (hm) {
      if (hit) st[staged + __popc(hm & below)] = pr;
      staged += __popc(hm);
      if (!multi) {
        wpairs += __popc(hm);
      } else {
        const int lead = __shfl_sync(kFullMask, kf >> 2, __ffs(hm) - 1);
        if (__all_sync(kFullMask, !hit || (kf >> 2) == lead)) {
          if (lead != wscene) {
            if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
            wscene = lead;
            wpairs = 0;
          }
          wpairs += __popc(hm);
        } else if (hit) {
          atomicAdd(&p.scene_pairs[kf >> 2], 1ull);
        }
      }
      if (staged >= 32) {
        __syncwarp();
        flush_staged(st, staged, lane, p);
        staged = 0;
      }
    }
  };

  while (true) {
    if (next_k >= chunk_end) {
      int c = 0;
      if (lane == 0) c = atomicAdd(p.work, p.chunk);
      c = __shfl_sync(kFullMask, c, 0);
      if (c >= span) break;
      next_k = p.begin + c;
      chunk_end = min(next_k + p.chunk, end);
    }
    const int take = min(32, chunk_end - next_k);
    const int k = next_k + lane;
    next_k += take;
    // 1. Runs: the candidates before the first minimum above the start's
    //    maximum (a sentinel position has an empty run).
    int len = 0, j = 0;
    if (lane < take) {
      j = p.partner[k];
      len = max(p.run_end[k] - j, 0);
      if (p.run_cap && len > p.run_cap) {  // a long run: the warp pass takes the rest
        p.long_list[atomicAdd(p.long_items, 1u)] = make_int2(k, j + p.run_cap);
        len = p.run_cap;
      }
    }
    const unsigned nz = __ballot_sync(kFullMask, len > 0);
    if (nz == 0) continue;
    // 2. Lay the runs end to end: exclusive prefix of the lengths; the starts
    //    with candidates keep their records in shared memory, in lane order.
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += v;
    }
    const int excl = incl - len;
    const int total = __shfl_sync(kFullMask, incl, 31);
    if (len > 0) {
      FlatStart r;
      r.kb = p.syz[k];
      r.kfl = p.sfloor[k];
      r.joff = j - excl;
      r.kf = multi ? p.sflag[k] : 0;
      r.kv = p.sv[k];
      rec[__popc(nz & below)] = r;
    }
    __syncwarp();
    tested += unsigned(total);
    // a run that begins inside the step at `base` marks bit (excl - base)
    const unsigned my_begin = len > 0 ? unsigned(excl) : 0xffffffffu;
    // 3. The filter over the flat candidates, V steps of 32 at a time.
    int begun = 0;  // starts whose run began before the current step
    for (int base = 0; base < total; base += 32 * V) {
      int si[V], jj[V];
      float4 kfj[V];  // (rule b, rule c, joff, -) of each lane's start
      float4 b[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const unsigned d = my_begin - unsigned(base + 32 * v);
        const unsigned heads = __reduce_or_sync(kFullMask, d < 32u ? (1u << d) : 0u);
        si[v] = begun + __popc(heads & upto) - 1;
        begun += __popc(heads);
        const int f = base + 32 * v + lane;
        kfj[v] = *reinterpret_cast<const float4 *>(&rec[si[v]].kfl);
        jj[v] = f < total ? __float_as_int(kfj[v].z) + f : -1;
      }
#pragma unroll
      for (int v = 0; v < V; ++v)
        if (jj[v] >= 0) b[v] = p.syz[jj[v]];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        bool pass = false;
        if (jj[v] >= 0) {
          const float4 kb = rec[si[v]].kb;
          // the first-cell rule as in the other shapes
          pass = overlap_bc(kb, b[v]) && b[v].x >= kfj[v].x && b[v].y >= kfj[v].y;
        }
        const unsigned pm = __ballot_sync(kFullMask, pass);
        if (pass) qu[queued + __popc(pm & below)] = make_int2(si[v], jj[v]);
        queued += __popc(pm);
      }
      __syncwarp();
      // 4. The check, 32 queued candidates at a time.
      while (queued >= 32) {
        check(32);
        __syncwarp();
      }
    }
    if (queued) check(queued);
    __syncwarp();  // the records are rewritten by the next 32 starts
  }
  __syncwarp();
  if (staged) flush_staged(st, staged, lane, p);
  if (lane == 0 && wpairs) atomicAdd(&p.scene_pairs[wscene], wpairs);
  if (lane == 0 && p.stats) atomicAdd(p.stats, tested);
}

// The warp pass over the runs the lane sweep handed over (runs longer than
// SweepParams::run_cap, which would keep one lane or group busy long after the
// others finished). One warp per run; each step tests 32 * U consecutive
// candidates, lane l taking j + 32u + l; the valid ones are those before the
// first x-test failure in position order (the padding after the last list
// covers the reads past it). All pairs of a run belong to its start box's scene.
template <int U, bool COUNT>
__global__ void __launch_bounds__(256)
stq_long_run_kernel(const SweepParams p) {
  constexpr int STAGE = 32 * (U + 1);
  __shared__ int2 stage[COUNT ? 1 : 8][COUNT ? 1 : STAGE];
  const int lane = threadIdx.x & 31;
  const unsigned below = lanemask_lt();
  int2 *st = stage[COUNT ? 0 : (threadIdx.x >> 5)];
  const unsigned n_items = *p.long_items;
  if (n_items == 0) return;
  int staged = 0;
  unsigned tested = 0;
  while (true) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(p.long_work, 1u);
    item = __shfl_sync(kFullMask, item, 0);
    if (item >= n_items) break;
    const int2 it = p.long_list[item];
    const int k = it.x;
    int j = it.y;
    const float kmax = p.xmax[k];
    const float4 kb = p.syz[k];
    const int4 kv = p.sv[k];
    const float2 kfl = p.sfloor[k];
    const int kf = p.sflag[k];
    unsigned run_hits = 0;  // warp-uniform (emit) or this lane's (count mode)
    while (true) {
      float xm[U];
#pragma unroll
      for (int u = 0; u < U; ++u) xm[u] = p.xmin[j + 32 * u + lane];
      int first = 32 * U;  // offset of the first x-test failure
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const unsigned fm = __ballot_sync(kFullMask, !(xm[u] <= kmax));
        if (first == 32 * U && fm) first = 32 * u + __ffs(fm) - 1;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int off = 32 * u + lane;
        bool hit = false;
        int2 pr = make_int2(0, 0);
        if (off < first) {
          ++tested;
          const float4 b = p.syz[j + off];
          if (overlap_bc(kb, b) && b.x >= kfl.x && b.y >= kfl.y) {  // and the first-cell rule
            const int4 bv = p.sv[j + off];
            hit = (p.typed || valid_pair(kv, bv)) && !covertex(kv, bv);
            pr = make_int2(min(kv.w, bv.w), max(kv.w, bv.w));
          }
        }
        if (COUNT) {
          run_hits += hit ? 1u : 0u;
        } else {
          const unsigned hm = __ballot_sync(kFullMask, hit);
          if (hit) st[staged + __popc(hm & below)] = pr;
          staged += __popc(hm);
          run_hits += unsigned(__popc(hm));
        }
      }
      if (!COUNT && staged >= 32) {
        __syncwarp();
        flush_staged(st, staged, lane, p);
        staged = 0;
      }
      if (first < 32 * U) break;
      j += 32 * U;
    }
    if (COUNT) {
      const unsigned total = __reduce_add_sync(kFullMask, run_hits);
      if (lane == 0 && total) atomicAdd(&p.box_counts[k - p.begin], int(total));
    } else if (lane == 0 && run_hits) {
      atomicAdd(&p.scene_pairs[kf >> 2], (unsigned long long)run_hits);
    }
  }
  if (!COUNT) {
    __syncwarp();
    if (staged) flush_staged(st, staged, lane, p);
    const unsigned t = __reduce_add_sync(kFullMask, tested);
    if (lane == 0 && p.stats) atomicAdd(p.stats, (unsigned long long)t);
  }
}

// Resident blocks per SM of a sweep kernel, queried once per kernel and
// device: the query costs host time on every launch otherwise, and the host
// calls launch one sweep per window back to back.
template <typename Kern>
cudaError_t resident_blocks(Kern kern, int block, int *per_sm) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> known;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const auto key = std::make_pair(reinterpret_cast<const void *>(kern), dev);
  std::lock_guard<std::mutex> lock(mu);
  auto it = known.find(key);
  if (it == known.end()) {
    int v = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, block, 0);
    if (e != cudaSuccess) return e;
    it = known.emplace(key, v).first;
  }
  *per_sm = it->second;
  return cudaSuccess;
}

template <typename Kern>
cudaError_t launch_persistent(Kern kern, int block, cudaStream_t s, const SweepParams &p, int num_sms) {
  int per_sm = 0;
  cudaError_t e = resident_blocks(kern, block, &per_sm);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  // persistent grid: all resident blocks, capped by the available work
  const int64_t warps_needed = (int64_t(p.end - p.begin) + p.chunk - 1) / p.chunk;
  int64_t blocks = int64_t(num_sms) * per_sm;
  const int64_t max_useful = (warps_needed + block / 32 - 1) / (block / 32);
  if (blocks > max_useful) blocks = max_useful;
  if (blocks < 1) blocks = 1;
  kern<<<unsigned(blocks), block, 0, s>>>(p);
  return cudaGetLastError();
}

template <int G, int Q, int BLOCK, bool COUNT>
cudaError_t launch_variant(cudaStream_t s, const SweepParams &p, int num_sms) {
  return launch_persistent(stq_sweep_kernel<G, Q, BLOCK, COUNT>, BLOCK, s, p, num_sms);
}

template <int G, int Q>
cudaError_t launch_gq(cudaStream_t s, const SweepParams &p, int block, int sms) {
  switch (block) {
    case 128: return launch_variant<G, Q, 128, false>(s, p, sms);
    case 512: return launch_variant<G, Q, 512, false>(s, p, sms);
    default: return launch_variant<G, Q, 256, false>(s, p, sms);
  }
}

template <int G>
cudaError_t launch_g(cudaStream_t s, const SweepParams &p, const SweepTuning &t, int sms) {
  switch (t.queue) {
    case 16:  // at least one entry per lane group
      if constexpr (G >= 2) return launch_gq<G, 16>(s, p, t.block, sms);
      else return launch_gq<G, 32>(s, p, t.block, sms);
    case 32: return launch_gq<G, 32>(s, p, t.block, sms);
    case 128: return launch_gq<G, 128>(s, p, t.block, sms);
    default: return launch_gq<G, 64>(s, p, t.block, sms);
  }
}

template <int U, int Q>
cudaError_t launch_uq(cudaStream_t s, const SweepParams &p, int block, int sms) {
  switch (block) {
    case 128: return launch_persistent(stq_sweep_lane_kernel<U, Q, 128, false>, 128, s, p, sms);
    case 512: return launch_persistent(stq_sweep_lane_kernel<U, Q, 512, false>, 512, s, p, sms);
    default: return launch_persistent(stq_sweep_lane_kernel<U, Q, 256, false>, 256, s, p, sms);
  }
}

template <int U>
cudaError_t launch_u(cudaStream_t s, const SweepParams &p, const SweepTuning &t, int sms) {
  switch (t.queue) {
    case 16:  // one start box per lane refills to 32 entries: the ring holds at least 32
    case 32: return launch_uq<U, 32>(s, p, t.block, sms);
    case 128: return launch_uq<U, 128>(s, p, t.block, sms);
    default: return launch_uq<U, 64>(s, p, t.block, sms);
  }
}

// The flat shape's blocks are 128 or 256 threads (512 would pass the 48 KB of
// static shared memory a block may hold).
template <int V>
cudaError_t launch_flat(cudaStream_t s, const SweepParams &p, int block, int sms) {
  if (block == 128) return launch_persistent(stq_sweep_flat_kernel<128, V>, 128, s, p, sms);
  return launch_persistent(stq_sweep_flat_kernel<256, V>, 256, s, p, sms);
}

// ---- overflow: longest prefix of start boxes whose pairs fit ------------------
constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

__global__ void __launch_bounds__(kScanBlock)
tile_sums_kernel(const int32_t *__restrict__ c, int64_t m, long long *__restrict__ sums) {
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  long long s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    const int64_t idx = base + int64_t(i) * kScanBlock + threadIdx.x;
    if (idx < m) s += c[idx];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFullMask, s, o);
  __shared__ long long red[kScanBlock / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int w = 0; w < kScanBlock / 32; ++w) t += red[w];
    sums[blockIdx.x] = t;
  }
}

// Single thread: exclusive scan of the tile sums and the last tile whose
// start is within capacity. Tiles are few (m / 2048).
__global__ void tile_select_kernel(long long *__restrict__ sums, int64_t ntiles,
                                   long long capacity, long long *__restrict__ sel) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long run = 0;
  int64_t last = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const long long v = sums[t];
    sums[t] = run;
    if (run <= capacity) last = t;
    run += v;
  }
  sel[0] = last;
}

// Within the selected tile: the longest prefix whose inclusive sum fits.
__global__ void __launch_bounds__(kScanBlock)
prefix_in_tile_kernel(const int32_t *__restrict__ c, int64_t m,
                      const long long *__restrict__ sums, const long long *__restrict__ sel,
                      long long capacity, DevScalars *scalars) {
  const int64_t t = sel[0];
  const int64_t base = t * kScanTile;
  if (threadIdx.x == 0) {
    long long run = sums[t];
    int64_t prefix = base;
    for (int64_t i = base; i < m && i < base + kScanTile; ++i) {
      run += c[i];
      if (run > capacity) break;
      prefix = i + 1;
    }
    scalars->prefix = prefix;
  }
}

// ---- all-pairs checker (get_collision_pairs, src/collision.cu:91-154) ---------
constexpr int kBruteTile = 128;

__global__ void __launch_bounds__(kBruteTile)
brute_force_kernel(const stq_aabb *__restrict__ boxes, int64_t n,
                   stq_pair *__restrict__ pairs, long long capacity,
                   unsigned long long *count) {
  __shared__ stq_aabb tile[kBruteTile];
  const int64_t i = int64_t(blockIdx.x) * kBruteTile + threadIdx.x;
  stq_aabb a;
  if (i < n) a = boxes[i];
  for (int64_t t0 = int64_t(blockIdx.y) * kBruteTile; t0 < n; t0 += int64_t(gridDim.y) * kBruteTile) {
    __syncthreads();
    if (t0 + threadIdx.x < n) tile[threadIdx.x] = boxes[t0 + threadIdx.x];
    __syncthreads();
    if (i >= n) continue;
    for (int q = 0; q < kBruteTile && t0 + q < n; ++q) {
      const int64_t jj = t0 + q;
      if (jj <= i) continue;
      const stq_aabb &b = tile[q];
      bool ov = true;
      for (int k = 0; k < 3; ++k) ov = ov && a.max[k] >= b.min[k] && a.min[k] <= b.max[k];
      const int4 av = make_int4(a.vertex_ids[0], a.vertex_ids[1], a.vertex_ids[2], a.id);
      const int4 bv = make_int4(b.vertex_ids[0], b.vertex_ids[1], b.vertex_ids[2], b.id);
      if (ov && valid_pair(av, bv) && !covertex(av, bv)) {
        const unsigned long long idx = atomicAdd(count, 1ull);
        if (idx < (unsigned long long)capacity)
          reinterpret_cast<int2 *>(pairs)[idx] = make_int2(min(a.id, b.id), max(a.id, b.id));
      }
    }
  }
}

__global__ void pairs_keys_kernel(stq_pair *pairs, int64_t n, unsigned long long *keys,
                                  bool to_keys) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    if (to_keys) {
      keys[i] = (static_cast<unsigned long long>(uint32_t(pairs[i].first)) << 32) |
                uint32_t(pairs[i].second);
    } else {
      pairs[i].first = int32_t(keys[i] >> 32);
      pairs[i].second = int32_t(keys[i] & 0xffffffffu);
    }
  }
}

}  // namespace

static cudaError_t launch_long_runs(cudaStream_t s, const SweepParams &p, bool count_mode, int num_sms) {
  if (!p.run_cap) return cudaSuccess;
  if (count_mode) stq_long_run_kernel<4, true><<<unsigned(num_sms * 2), 256, 0, s>>>(p);
  else stq_long_run_kernel<4, false><<<unsigned(num_sms * 2), 256, 0, s>>>(p);
  return cudaGetLastError();
}

static cudaError_t launch_sweep_lanes(cudaStream_t s, const SweepParams &p, const SweepTuning &t,
                                      bool count_mode, int num_sms);

cudaError_t launch_sweep(cudaStream_t s, const SweepParams &p, const SweepTuning &t,
                         bool count_mode, int num_sms) {
  if (p.end <= p.begin) return cudaSuccess;
  cudaError_t e = launch_sweep_lanes(s, p, t, count_mode, num_sms);
  if (e != cudaSuccess) return e;
  return launch_long_runs(s, p, count_mode, num_sms);
}

static cudaError_t launch_sweep_lanes(cudaStream_t s, const SweepParams &p, const SweepTuning &t,
                                      bool count_mode, int num_sms) {
  if (count_mode)  // per-start-box counts do not depend on the tuning
    return launch_variant<8, 64, 256, true>(s, p, num_sms);
  if (t.shape == kShapeFlat && p.run_end) {
    switch (t.per_lane) {  // filter steps per round
      case 2: return launch_flat<2>(s, p, t.block, num_sms);
      default: return launch_flat<4>(s, p, t.block, num_sms);
    }
  }
  if (t.lanes == 1) {  // one start box per lane
    switch (t.per_lane) {
      case 1: return launch_u<1>(s, p, t, num_sms);
      case 2: return launch_u<2>(s, p, t, num_sms);
      case 8: return launch_u<8>(s, p, t, num_sms);
      default: return launch_u<4>(s, p, t, num_sms);
    }
  }
  switch (t.lanes) {
    case 2: return launch_g<2>(s, p, t, num_sms);
    case 4: return launch_g<4>(s, p, t, num_sms);
    case 16: return launch_g<16>(s, p, t, num_sms);
    case 32: return launch_g<32>(s, p, t, num_sms);
    default: return launch_g<8>(s, p, t, num_sms);
  }
}

size_t prefix_workspace_bytes(int64_t m) {
  const int64_t ntiles = (m + kScanTile - 1) / kScanTile;
  return sizeof(long long) * (ntiles + 2);
}

cudaError_t launch_prefix_select(cudaStream_t s, const int32_t *box_counts, int64_t m,
                                 long long capacity, void *workspace, DevScalars *scalars,
                                 int64_t *launches) {
  const int64_t ntiles = (m + kScanTile - 1) / kScanTile;
  long long *sums = static_cast<long long *>(workspace);
  long long *sel = sums + ntiles + 1;
  tile_sums_kernel<<<unsigned(ntiles), kScanBlock, 0, s>>>(box_counts, m, sums);
  tile_select_kernel<<<1, 32, 0, s>>>(sums, ntiles, capacity, sel);
  prefix_in_tile_kernel<<<1, kScanBlock, 0, s>>>(box_counts, m, sums, sel, capacity, scalars);
  if (launches) *launches += 3;
  return cudaGetLastError();
}

cudaError_t launch_brute_force(cudaStream_t s, const stq_aabb *boxes, int64_t n,
                               stq_pair *pairs, long long capacity,
                               unsigned long long *count) {
  if (n < 2) return cudaSuccess;
  const int64_t tiles = (n + kBruteTile - 1) / kBruteTile;
  dim3 grid(unsigned(tiles), unsigned(tiles < 64 ? tiles : 64));
  brute_force_kernel<<<grid, kBruteTile, 0, s>>>(boxes, n, pairs, capacity, count);
  return cudaGetLastError();
}

cudaError_t launch_pairs_to_keys(cudaStream_t s, const stq_pair *pairs, int64_t n,
                                 unsigned long long *keys, bool to_keys) {
  if (n == 0) return cudaSuccess;
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  pairs_keys_kernel<<<unsigned(g), 256, 0, s>>>(const_cast<stq_pair *>(pairs), n, keys, to_keys);
  return cudaGetLastError();
}

}  // namespace stq
