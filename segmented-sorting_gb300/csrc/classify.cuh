// Segment classification and the pieces the cooperative long-segment kernel
// shares with the host: the workspace views, the counters, the bounded grid
// barrier and the mapping of a job's instance to its buffers.
//
// Classify replaces the reference's length binning bb_bin
// (src/bb_segsort/bb_bin.h:23,31-139): instead of 13 power-of-two bins and a
// device-to-host copy of their counts (bb_bin.h:46), it writes a half-tile ->
// first-segment map that the tile sort reads directly, and two device-side
// lists of the segments longer than the tile capacity: those longer than the
// radix threshold for the LSD radix passes, the others for the merge passes.
// Two forms write the same map and lists: one thread per segment boundary
// (problems of long segments on average), or one warp-cooperative search per
// half-tile (short segments, and batches).
#pragma once

#include "segsort_common.cuh"

namespace segsort {

constexpr int kBarrierSpinLimit = 1 << 24;  // ~2 s with the back-off below

enum : int {
  kCtrJobs = 0,       // segments for the merge passes found by classify
  kCtrItems = 2,      // merge items of all jobs
  kCtrPasses = 3,     // most merge passes of any job
  kCtrBarCount = 6,   // grid barrier: arrivals
  kCtrBarGen = 7,     // grid barrier: generation
  kCtrRJobs = 8,      // segments for the radix passes found by classify
  kCtrRTiles = 9,     // radix tiles of all radix jobs
  kCtrRDigits = 10,   // OR over radix jobs of their digits that vary
  kCtrFallback = 11,  // tile chunks the bucket sort left to the comparison sort
  kCtrListTicket = 12,  // next listed chunk a comparison-sort CTA takes
  kCtrWords = 16,
};

struct TileChunk;  // tile_sort.cuh

// Device views of the workspace.
template <typename K>
struct LargeWs {
  uint32_t *ctr;          // [kCtrWords]
  int4 *jobs;             // [max_jobs] merge segments: {begin, end, segment or 0, instance}
  int32_t *item_prefix;   // [max_jobs + 1] merge items before each job
  int32_t *half_first;    // [halves + 1] first segment starting at or after h * CAP/2
  int32_t *item_job;      // [max_items] job of each merge item
  uint32_t *split;        // [max_items] merge-path split of each item's first output
  int4 *item_desc;        // [2 * max_items] item descriptors of the current pass
  K *tmp_keys;            // [n]
  uint32_t *tmp_vals;     // [n]
  int4 *rjobs;            // [max_rjobs] radix segments: {begin, end, segment or 0, instance}
  int32_t *rtile_prefix;  // [max_rjobs + 1] radix tiles before each radix job
  int4 *rtile_desc;       // [max_rtiles] radix tiles: {first position, length, job, index in job}
  uint32_t *rdigits;      // [max_rjobs] digits of the job's keys that vary (bit d: digit d)
  uint32_t *rhist;        // [max_rjobs][digits][256] digit counts, then bucket starts
  unsigned long long *rlook;  // [max_rtiles][256] look-back words of the radix tiles
  TileChunk *fallback;    // [max_fallback] chunks for the comparison sort (bucket route)
  int64_t max_fallback;
  int32_t max_jobs;
  int32_t max_rjobs;
  int64_t max_items;
  int64_t halves;
  int64_t max_rtiles;
  int64_t radix_min;      // segments longer than this take the radix passes
  // 1: first stage of the MSD route (radix_sort.cuh): the radix segments that
  // qualify run one pass on their top varying digit, the others all their
  // passes; the long-segment kernel then returns before the merge passes.
  int32_t msd_stage;
  int32_t tile_cap;       // keys per tile of the tile sort
  int64_t lsd_min;        // MSD stage: a segment that does not qualify and is not longer than
                          // this is left to the second stage's merge passes
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}

// ---------------------------------------------------------------------------
// Classify: one thread per segment boundary s in [0, nseg].
//  * half_first[h] = s for every half-tile h with off(s-1) < h*half <= off(s)
//    (off(-1) = -inf, off(nseg) = +inf): the first segment starting in or
//    after half-tile h, so the tile sort needs no search over the offsets;
//  * segments longer than cap become jobs of the merge passes, or of the
//    radix passes when longer than ws.radix_min (warp-aggregated atomic
//    appends), tagged with the instance they belong to.
// Every lane of the warp calls it; `valid` is false for lanes past the end.
template <typename K>
__device__ __forceinline__ void classify_boundary(const Offsets &off, int64_t s, bool valid,
                                                  int64_t cap, int64_t half, int32_t *half_first,
                                                  int64_t halves, const LargeWs<K> &ws,
                                                  int32_t inst) {
  const int lane = threadIdx.x & 31;
  int64_t len = 0, cur = 0;
  if (valid && s <= off.nseg) {
    cur = s < off.nseg ? off(s) : 0;
    const int64_t h_lo = s == 0 ? 0 : off(s - 1) / half + 1;
    const int64_t h_hi = s == off.nseg ? halves : min(cur / half, halves);
    for (int64_t h = h_lo; h <= h_hi; ++h) half_first[h] = static_cast<int32_t>(s);
    if (s < off.nseg) len = off(s + 1) - cur;
    if (off.flags != nullptr && s < off.nseg && (off.flags[s] & kSegSkip)) len = 0;  // sorted
  }
  const bool rlarge = len > ws.radix_min;
  const bool large = len > cap && !rlarge;
  const int4 job = make_int4(static_cast<int32_t>(cur), static_cast<int32_t>(cur + len),
                            static_cast<int32_t>(s), inst);
  const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, large);
  if (ballot != 0) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&ws.ctr[kCtrJobs], __popc(ballot));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    const uint32_t j = base + __popc(ballot & lanemask_lt());
    if (large && j < static_cast<uint32_t>(ws.max_jobs)) ws.jobs[j] = job;
  }
  const uint32_t rballot = __ballot_sync(0xFFFFFFFFu, rlarge);
  if (rballot != 0) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&ws.ctr[kCtrRJobs], __popc(rballot));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    const uint32_t j = base + __popc(rballot & lanemask_lt());
    if (rlarge && j < static_cast<uint32_t>(ws.max_rjobs)) ws.rjobs[j] = job;
  }
}

// Appends long segment seg (from beg to end) to the merge or the radix job
// list; nothing for a segment its flags mark as already sorted.
template <typename K>
__device__ __forceinline__ void add_long_job(const LargeWs<K> &ws, const Offsets &off,
                                             int64_t seg, int64_t beg, int64_t end,
                                             int32_t inst) {
  if (off.flags != nullptr && (off.flags[seg] & kSegSkip)) return;
  const int4 job = make_int4(static_cast<int32_t>(beg), static_cast<int32_t>(end),
                             static_cast<int32_t>(seg), inst);
  const bool radix = end - beg > ws.radix_min;
  const uint32_t j = atomicAdd(&ws.ctr[radix ? kCtrRJobs : kCtrJobs], 1u);
  if (j < static_cast<uint32_t>(radix ? ws.max_rjobs : ws.max_jobs))
    (radix ? ws.rjobs : ws.jobs)[j] = job;
}

template <typename K>
__global__ void __launch_bounds__(256)
large_classify_kernel(Offsets off, int64_t cap, int64_t half, LargeWs<K> ws) {
  pdl_trigger();  // the tile kernel may launch under this one (it waits for it)
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  classify_boundary<K>(off, s, true, cap, half, ws.half_first, ws.halves, ws, 0);
}

// The first segment s in [0, nseg] with off(s) >= x, counting off(nseg) as
// +inf (offsets are non-decreasing).  Called by a whole warp; every round
// probes 32 points of the remaining interval, so a search over 2^23 segments
// takes 5 rounds of loads.
__device__ __forceinline__ int64_t warp_lower_bound(const Offsets &off, int64_t x) {
  const int lane = threadIdx.x & 31;
  int64_t lo = 0, hi = off.nseg;  // the answer lies in [lo, hi]
  while (hi > lo) {
    const int64_t span = hi - lo;
    const bool small = span <= 32;
    // Probes lie in [lo, hi), so they read offsets below nseg only.
    const int64_t p = small ? lo + lane : lo + (span * (lane + 1)) / 33;
    const bool ge = (small && lane >= span) ? true : off(p) >= x;
    const int c = __popc(~__ballot_sync(0xFFFFFFFFu, ge));  // lanes below the first true one
    if (small) {
      lo += c;
      hi = lo;
    } else {
      const long long before = __shfl_sync(0xFFFFFFFFu, static_cast<long long>(p), c > 0 ? c - 1 : 0);
      const long long at = __shfl_sync(0xFFFFFFFFu, static_cast<long long>(p), c < 32 ? c : 31);
      const int64_t nlo = c > 0 ? before + 1 : lo;
      const int64_t nhi = c < 32 ? at : hi;
      lo = nlo;
      hi = nhi;
    }
  }
  return lo;
}

// Classify by half-tiles (one problem): half_first[h] -- the lower bound of
// h * half in the offsets, the same map classify_boundary writes -- for h in
// [0, halves], and the one segment that can be long among those starting in
// half-tile h: the last one, half_first[h + 1] - 1.  A segment longer than
// cap >= half runs past the end of the half-tile it starts in, so no other
// segment starts after it there, and every long segment is found once, by
// the half-tile it starts in.  Work grows with the number of half-tiles, not
// segments.  A CTA of kClassifyWarps + 1 warps handles kClassifyWarps
// entries, one search per warp: the extra warp finds the next CTA's first
// entry, which the CTA's last job check needs.
constexpr int kClassifyWarps = 8;

template <typename K>
__global__ void __launch_bounds__((kClassifyWarps + 1) * 32)
large_classify_halves_kernel(Offsets off, int64_t cap, int64_t half, LargeWs<K> ws) {
  pdl_trigger();  // the tile kernel may launch under this one (it waits for it)
  __shared__ int64_t lb_s[kClassifyWarps + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t h = static_cast<int64_t>(blockIdx.x) * kClassifyWarps + w;
  if (h <= ws.halves) {
    const int64_t a = warp_lower_bound(off, h * half);
    if (lane == 0) {
      lb_s[w] = a;
      if (w < kClassifyWarps) ws.half_first[h] = static_cast<int32_t>(a);
    }
  }
  __syncthreads();
  if (w < kClassifyWarps && h < ws.halves && lane == 0) {
    const int64_t a = lb_s[w], b = lb_s[w + 1];
    if (b > a) {
      const int64_t beg = off(b - 1), end = off(b);
      if (end - beg > cap) add_long_job(ws, off, b - 1, beg, end, 0);
    }
  }
}

// Batched form of the half-tile classify: global entry g is entry
// g - half_base of the instance that owns it (each instance owns
// 2 * tiles + 1 entries).  Entry h + 1 of the job check belongs to the same
// instance as entry h, since h < 2 * tiles.
template <typename K>
__global__ void __launch_bounds__((kClassifyWarps + 1) * 32)
large_classify_halves_batch_kernel(const BatchInst *__restrict__ tab, int32_t count,
                                   int64_t entries, int64_t cap, int64_t half, LargeWs<K> ws) {
  __shared__ int64_t lb_s[kClassifyWarps + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t g = static_cast<int64_t>(blockIdx.x) * kClassifyWarps + w;
  int32_t i = 0;
  int64_t h = 0, halves = 0;
  if (g < entries) {
    i = find_instance(tab, count, g, &BatchInst::half_base);
    const BatchInst &I = tab[i];
    h = g - I.half_base;
    halves = 2 * ((I.n + cap - 1) / cap);
    const int64_t a = warp_lower_bound(I.offsets_view(), h * half);
    if (lane == 0) {
      lb_s[w] = a;
      if (w < kClassifyWarps) ws.half_first[g] = static_cast<int32_t>(a);
    }
  }
  __syncthreads();
  if (w < kClassifyWarps && g < entries && h < halves && lane == 0) {
    const int64_t a = lb_s[w], b = lb_s[w + 1];
    if (b > a) {
      const Offsets off = tab[i].offsets_view();
      const int64_t beg = off(b - 1), end = off(b);
      if (end - beg > cap) add_long_job(ws, off, b - 1, beg, end, i);
    }
  }
}

// ---------------------------------------------------------------------------
// Where the long-segment kernel finds an instance's keys and values: the
// caller's buffers and the instance's region of the temporary buffers, both
// indexed by instance-local positions.
template <typename K>
struct SideBuffers {
  K *keys;
  uint32_t *vals;
  K *tmp_keys;
  uint32_t *tmp_vals;
};

// One problem: every job belongs to it.
template <typename K>
struct SingleSpace {
  K *keys;
  uint32_t *vals;
  K *tmp_keys;
  uint32_t *tmp_vals;
  __device__ __forceinline__ SideBuffers<K> operator()(int32_t) const {
    return {keys, vals, tmp_keys, tmp_vals};
  }
};

// A batch: jobs carry their instance, whose buffers come from the table.
template <typename K>
struct BatchSpace {
  const BatchInst *tab;
  K *tmp_keys;
  uint32_t *tmp_vals;
  __device__ __forceinline__ SideBuffers<K> operator()(int32_t i) const {
    const BatchInst &I = tab[i];
    return {static_cast<K *>(I.keys), I.vals, tmp_keys + I.tmp_base,
            tmp_vals ? tmp_vals + I.tmp_base : nullptr};
  }
};

// ---------------------------------------------------------------------------
// Grid barrier for a cooperative launch (all CTAs resident), bounded: a CTA
// that waits longer than spin_limit back-offs raises kStatusTimeout and goes
// on, so a lost arrival can corrupt the result but never hang the GPU.
__device__ __forceinline__ void grid_barrier(uint32_t *ctr, int spin_limit = kBarrierSpinLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = ld_volatile(ctr + kCtrBarGen);
    __threadfence();
    const uint32_t arrived = atomicAdd(ctr + kCtrBarCount, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(ctr + kCtrBarCount, 0u);
      __threadfence();
      atomicAdd(ctr + kCtrBarGen, 1u);
    } else {
      int spins = 0;
      while (ld_volatile(ctr + kCtrBarGen) == gen) {
        if (++spins > spin_limit) {
          raise_status(kStatusTimeout);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

}  // namespace segsort
