// Long-segment path: segments longer than the tile capacity CAP.
//
// A most-significant-digit split turns every long segment into 256 buckets
// with one stable scatter, and the tile-sort core (sort_chunk) then sorts the
// buckets in shared memory.  Per element that is one read of the keys for the
// histograms, one read+write of keys and values for the scatter and one for
// the bucket sort (36 bytes for 32-bit key/value pairs), against 4 scatter
// passes (68 bytes) for a least-significant-digit radix sort.  The scatter
// uses the highest byte that varies inside the segment (constant leading
// bytes are skipped), and a bucket still longer than CAP becomes a segment of
// the next level, split on the next byte.  Every level consumes a byte, so
// there are at most sizeof(key) levels; a bucket left with no bytes holds
// equal keys and is already in stable order.
//
// The scatter is the "onesweep" pass: each 4096-key chunk ranks its keys by
// digit in shared memory (peer lanes from one ballot per digit bit, counts from
// leader atomics, which keeps equal digits in input order), learns its global
// digit offsets from the chunks
// before it in the same segment through decoupled look-back, and writes runs
// of equal digits to their places.
//
// Everything after the classify kernel runs in one cooperative kernel
// (large_sort_kernel): all CTAs are resident, phases are separated by a
// bounded grid barrier, and a call without long segments costs one launch
// that returns at once.  Every wait on another CTA is bounded; a wait that
// gives up raises kStatusTimeout and the kernel carries on, so a lost wait
// can corrupt the result but never hang the GPU.
//
// It replaces the reference's large-segment driver gen_grid_kern_r2049
// (src/bb_segsort/bb_comput_l.h:1155-1284: a 2048-key block sort followed by
// log2(len/2048) global merge passes, with several synchronous device-to-host
// copies) and CUB's one-CTA-per-segment radix sort
// (lib/cub/device/dispatch/dispatch_radix_sort.cuh:323).
#pragma once

#include "segsort_common.cuh"
#include "tile_sort.cuh"

namespace segsort {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kLThreads = 512;  // CTA size; threads [0, kRadix) own one digit each in the digit loops
constexpr int kLWarps = kLThreads / 32;

// Keys per thread and per chunk of the scatter: 8192 keys for 32-bit keys,
// 4096 for 64-bit keys.
template <typename K>
struct PassShape {
  static constexpr int kItems = sizeof(K) == 4 ? 16 : 8;
  static constexpr int kChunk = kLThreads * kItems;
};

constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagInclusive = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr int kLookbackSpinLimit = 1 << 20;  // ~0.1 s with the back-off below
constexpr int kBarrierSpinLimit = 1 << 24;   // ~2 s

enum : int {
  kCtrJobs = 0,          // +0 / +1: job counts of the two job lists
  kCtrChunks = 2,        // scatter chunks of the current level
  kCtrPass = 3,          // scatter chunk tickets
  kCtrBuckets = 4,       // bucket-chunk entries of the current level
  kCtrBucketTicket = 5,  // bucket-chunk tickets
  kCtrBarCount = 6,      // grid barrier: arrivals
  kCtrBarGen = 7,        // grid barrier: generation
  kCtrWords = 16,
};

enum : int { kEntrySort = 0, kEntryCopy = 1, kEntryDirect = 2 };
constexpr int32_t kDigitUnset = -2;  // digit[] before the scatter wrote it
constexpr int32_t kDigitNone = -1;   // no remaining byte varies: keys are equal

// Device views of the workspace.
template <typename K>
struct LargeWs {
  uint32_t *ctr;          // [kCtrWords]
  int4 *jobs[2];          // job lists: {begin, end, bytes left to sort, 0}
  int32_t *chunk_prefix;  // [max_jobs + 1] scatter chunks before each job
  uint32_t *hist;         // [max_jobs][passes][kRadix]
  int32_t *bstart;        // [max_jobs][kRadix + 1] bucket starts, relative to the job
  int32_t *digit;         // [max_jobs] byte the job was split on
  uint32_t *status;       // [max_chunks][kRadix] look-back words
  int4 *desc;             // [max_chunks] chunk begin, job end, job index, job begin
  int4 *entries;          // [max_entries] {job, d0, d1, sort}, {begin, len, 0, copy} or
                          // {begin, len, 0, direct}
  int32_t *half_first;    // [halves + 1] first segment starting at or after h * CAP/2
  K *tmp_keys;            // [n]
  uint32_t *tmp_vals;     // [n]
  int32_t max_jobs;
  int32_t passes;         // bytes of the order bits
  int64_t max_chunks;
  int64_t max_entries;
  int64_t halves;
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Lanes of the warp holding the same 8-bit digit as this lane, among the
// lanes in `active` (bit-plane ballots: one ballot per digit bit).
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, uint32_t active) {
  uint32_t peers = active;
#pragma unroll
  for (int b = 0; b < kRadixBits; ++b) {
    const uint32_t bit = (d >> b) & 1u;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
    peers &= bal ^ (bit - 1u);  // bal where the bit is set, ~bal where it is clear
  }
  return peers;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ int32_t ld_volatile(const int32_t *p) {
  return *reinterpret_cast<const volatile int32_t *>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t *>(p) = v;
}

// ---------------------------------------------------------------------------
// Classify: one thread per segment boundary s in [0, nseg].
//  * half_first[h] = s for every half-tile h with off(s-1) < h*half <= off(s)
//    (off(-1) = -inf, off(nseg) = +inf): the first segment starting in or
//    after half-tile h, so the tile sort needs no search over the offsets;
//  * segments longer than cap become jobs of the first level (warp-aggregated
//    atomic append), tagged with the instance they belong to.
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
  }
  const bool large = len > cap;
  const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, large);
  if (ballot == 0) return;
  uint32_t base = 0;
  if (lane == 0) base = atomicAdd(&ws.ctr[kCtrJobs], __popc(ballot));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  const uint32_t j = base + __popc(ballot & lanemask_lt());
  if (large && j < static_cast<uint32_t>(ws.max_jobs))
    ws.jobs[0][j] = make_int4(static_cast<int32_t>(cur), static_cast<int32_t>(cur + len),
                              ws.passes, inst);
}

template <typename K>
__global__ void __launch_bounds__(256)
large_classify_kernel(Offsets off, int64_t cap, int64_t half, LargeWs<K> ws) {
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  classify_boundary<K>(off, s, true, cap, half, ws.half_first, ws.halves, ws, 0);
}

// Batched form: thread g classifies boundary g - bound_base of the instance
// that owns it; `bounds` is the batch's total of nseg + 1 over its instances.
template <typename K>
__global__ void __launch_bounds__(256)
large_classify_batch_kernel(const BatchInst *__restrict__ tab, int32_t count, int64_t bounds,
                            int64_t cap, int64_t half, LargeWs<K> ws) {
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool valid = g < bounds;
  const int32_t i = find_instance(tab, count, valid ? g : 0, &BatchInst::bound_base);
  const BatchInst &I = tab[i];
  const int64_t tiles = (I.n + cap - 1) / cap;
  classify_boundary<K>(I.offsets_view(), g - I.bound_base, valid, cap, half,
                       ws.half_first + I.half_base, 2 * tiles, ws, i);
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
// Grid barrier for a cooperative launch (all CTAs resident), bounded.
__device__ __forceinline__ void grid_barrier(uint32_t *ctr) {
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
        if (++spins > kBarrierSpinLimit) {
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

// Block-wide exclusive sum of one value per thread (kLThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t *warp_tmp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tmp[warp] = x;
  __syncthreads();
  uint32_t wsum = 0;
#pragma unroll
  for (int w = 0; w < kLWarps; ++w) wsum += (w < warp) ? warp_tmp[w] : 0u;
  __syncthreads();
  return wsum + x - v;
}

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

// Shared-memory sizes of the kernel's phases (one dynamic buffer, reused).
template <typename K, bool PAIRS, typename Cfg>
struct LargeSmem {
  static constexpr int kChunk = PassShape<K>::kChunk;
  // Histogram tables shared by groups of warps: 8 for 32-bit keys, 4 for
  // 64-bit keys (32 KB either way).
  static constexpr int kHistTables = sizeof(typename KeyOrder<K>::Bits) == 4 ? 8 : 4;
  static constexpr size_t kHist = kHistTables * sizeof(typename KeyOrder<K>::Bits) * kRadix * 4;
  static constexpr size_t kScatter = kLWarps * kRadix * 4   // per-warp digit counts
                                     + 2 * kRadix * 4       // chunk offsets, deltas
                                     + kChunk * sizeof(K)   // staged keys
                                     + (PAIRS ? kChunk * 4 : 0);
  static constexpr size_t kPlan = kLWarps * (kRadix + 1) * 4;
  static constexpr size_t kBytes = cmax(cmax(Cfg::kSmemBytes, kScatter), cmax(kHist, kPlan));
};

// ---------------------------------------------------------------------------
// Space (SingleSpace or BatchSpace) maps a job's instance to its buffers.
template <typename K, bool PAIRS, typename Cfg, typename Space>
__global__ void __launch_bounds__(kLThreads, 1)
large_sort_kernel(Space sp, LargeWs<K> ws) {
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  constexpr int kItems = PassShape<K>::kItems;
  constexpr int kChunk = PassShape<K>::kChunk;
  constexpr int kMaxLevels = sizeof(Bits);
  constexpr int CAP = Cfg::CAP;
  static_assert(Cfg::NT == kLThreads, "the bucket sort runs with the kernel's CTA shape");

  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t hb[CAP / 32];
  __shared__ int warp_s[kLWarps];
  __shared__ uint32_t warp_tmp[kLWarps];
  __shared__ int64_t tk_s;
  __shared__ uint64_t carry_s;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t G = gridDim.x;
  const int passes = ws.passes;
  const uint32_t lt = lanemask_lt();

  if (ld_volatile(&ws.ctr[kCtrJobs]) == 0) return;  // no long segments: one short launch

  for (int level = 0; level < kMaxLevels; ++level) {
    const int cur = level & 1;
    const int64_t nj = min(static_cast<int64_t>(ld_volatile(&ws.ctr[kCtrJobs + cur])),
                           static_cast<int64_t>(ws.max_jobs));
    if (nj == 0) break;
    const int4 *jobs = ws.jobs[cur];
    int4 *next_jobs = ws.jobs[cur ^ 1];
    // Level parity: even levels scatter the caller's buffers into tmp, odd
    // levels tmp into the caller's buffers.

    // ---- P1: chunk prefix (CTA 0); reset per-level counters and arrays --------
    if (blockIdx.x == 0) {
      if (tid == 0) carry_s = 0;
      __syncthreads();
      const uint64_t capc = static_cast<uint64_t>(ws.max_chunks);
      for (int64_t base = 0; base < nj; base += kLThreads) {
        const int64_t j = base + tid;
        uint32_t v = 0;
        if (j < nj) {
          const int4 jb = jobs[j];
          const int64_t len = jb.y > jb.x ? jb.y - jb.x : 0;
          // Level-0 jobs that fit the bucket sort are sorted directly.
          v = (level == 0 && len <= CAP) ? 0u : static_cast<uint32_t>((len + kChunk - 1) / kChunk);
        }
        const uint32_t ex = block_exclusive_sum(v, warp_tmp);
        const uint64_t e64 = carry_s + ex;
        if (j < nj) ws.chunk_prefix[j] = static_cast<int32_t>(e64 < capc ? e64 : capc);
        __syncthreads();
        if (tid == kLThreads - 1) carry_s = e64 + v;
        __syncthreads();
      }
      if (tid == 0) {
        const uint64_t total = carry_s < capc ? carry_s : capc;
        ws.chunk_prefix[nj] = static_cast<int32_t>(total);
        ws.ctr[kCtrChunks] = static_cast<uint32_t>(total);
        ws.ctr[kCtrPass] = 0;
        ws.ctr[kCtrBuckets] = 0;
        ws.ctr[kCtrBucketTicket] = 0;
        ws.ctr[kCtrJobs + (cur ^ 1)] = 0;
      }
    }
    {
      const int64_t words = nj * passes * kRadix / 4;
      uint4 *h4 = reinterpret_cast<uint4 *>(ws.hist);
      for (int64_t i = blockIdx.x * kLThreads + tid; i < words; i += G * kLThreads)
        h4[i] = make_uint4(0, 0, 0, 0);
      for (int64_t j = blockIdx.x * kLThreads + tid; j < nj; j += G * kLThreads)
        ws.digit[j] = kDigitUnset;
    }
    grid_barrier(ws.ctr);
    const int64_t total = ld_volatile(&ws.ctr[kCtrChunks]);

    // ---- P1b: chunk descriptors, zeroed look-back words -------------------------
    for (int64_t j = blockIdx.x; j < nj; j += G) {
      const int4 jb = jobs[j];
      const int64_t p0 = ws.chunk_prefix[j], p1 = ws.chunk_prefix[j + 1];
      for (int64_t c = tid; c < p1 - p0; c += kLThreads)
        ws.desc[p0 + c] = make_int4(static_cast<int32_t>(jb.x + c * kChunk), jb.y,
                                    static_cast<int32_t>(j), jb.x);
    }
    {
      uint4 *s4 = reinterpret_cast<uint4 *>(ws.status);
      for (int64_t i = blockIdx.x * kLThreads + tid; i < total * kRadix / 4; i += G * kLThreads)
        s4[i] = make_uint4(0, 0, 0, 0);
    }
    grid_barrier(ws.ctr);

    // ---- P2: digit histograms of every byte still to sort -----------------------
    {
      constexpr int kTables = LargeSmem<K, PAIRS, Cfg>::kHistTables;
      uint32_t *h = reinterpret_cast<uint32_t *>(smem);
      uint32_t *mine = h + (warp % kTables) * passes * kRadix;
      for (int64_t t = blockIdx.x; t < total; t += G) {
        for (int i = tid; i < kTables * passes * kRadix; i += kLThreads) h[i] = 0;
        __syncthreads();
        const int4 dsc = ws.desc[t];
        const int64_t cb = dsc.x, e = dsc.y;
        const int32_t j = dsc.z;
        const int4 jb = jobs[j];
        const int bytes = min(jb.z, passes);
        const SideBuffers<K> B = sp(jb.w);
        const K *src_k = cur == 0 ? B.keys : B.tmp_keys;
        const int clen = static_cast<int>(min(static_cast<int64_t>(kChunk), e - cb));
        Bits xs[kItems];
#pragma unroll
        for (int u = 0; u < kItems; ++u) {
          const int i = u * kLThreads + tid;
          xs[u] = i < clen ? Ord::to_bits(src_k[cb + i]) : Bits(0);
        }
#pragma unroll
        for (int u = 0; u < kItems; ++u) {
          const int i = u * kLThreads + tid;
          const bool valid = i < clen;
          const Bits x = xs[u];
          for (int q = 0; q < bytes; ++q) {
            const uint32_t d = static_cast<uint32_t>((x >> (q * kRadixBits)) & (kRadix - 1));
            // A whole warp on one digit (skewed keys) adds once.
            const uint32_t d_first = __shfl_sync(0xFFFFFFFFu, d, 0);
            if (__all_sync(0xFFFFFFFFu, valid && d == d_first)) {
              if (lane == 0) atomicAdd(&mine[q * kRadix + d_first], 32u);
            } else if (valid) {
              atomicAdd(&mine[q * kRadix + d], 1u);
            }
          }
        }
        __syncthreads();
        uint32_t *gh = ws.hist + static_cast<size_t>(j) * passes * kRadix;
        for (int i = tid; i < bytes * kRadix; i += kLThreads) {
          uint32_t v = 0;
#pragma unroll
          for (int tb = 0; tb < kTables; ++tb) v += h[tb * passes * kRadix + i];
          if (v) atomicAdd(&gh[i], v);
        }
        __syncthreads();
      }
    }
    grid_barrier(ws.ctr);

    // ---- P3: stable scatter by the highest varying byte ------------------------
    {
      uint32_t *whist = reinterpret_cast<uint32_t *>(smem);
      uint32_t *boff_s = whist + kLWarps * kRadix;
      int32_t *delta_s = reinterpret_cast<int32_t *>(boff_s + kRadix);
      K *ks = reinterpret_cast<K *>(delta_s + kRadix);
      uint32_t *vs = reinterpret_cast<uint32_t *>(ks + kChunk);
      // Thread 0 holds the next ticket and its descriptor, fetched while the
      // current chunk is being processed.
      int64_t next_t = 0;
      int4 next_d = make_int4(0, 0, 0, 0);
      if (tid == 0) {
        next_t = atomicAdd(&ws.ctr[kCtrPass], 1u);
        if (next_t < total) next_d = ws.desc[next_t];
      }
      __shared__ int4 dsc_s;
      while (true) {
        if (tid == 0) {
          tk_s = next_t;
          dsc_s = next_d;
        }
        for (int i = tid; i < kLWarps * kRadix; i += kLThreads) whist[i] = 0;
        __syncthreads();
        const int64_t t = tk_s;
        if (t >= total) break;
        const int4 dsc = dsc_s;
        if (tid == 0) {
          next_t = atomicAdd(&ws.ctr[kCtrPass], 1u);
          if (next_t < total) next_d = ws.desc[next_t];
        }
        const int64_t cb = dsc.x, e = dsc.y, b = dsc.w;
        const int32_t j = dsc.z;
        const int4 jb = jobs[j];
        const SideBuffers<K> B = sp(jb.w);
        const K *src_k = cur == 0 ? B.keys : B.tmp_keys;
        K *dst_k = cur == 0 ? B.tmp_keys : B.keys;
        const uint32_t *src_v = cur == 0 ? B.vals : B.tmp_vals;
        uint32_t *dst_v = cur == 0 ? B.tmp_vals : B.vals;
        const int64_t c = (cb - b) / kChunk;
        const int clen = static_cast<int>(min(static_cast<int64_t>(kChunk), e - cb));
        const uint32_t *jh = ws.hist + static_cast<size_t>(j) * passes * kRadix;
        // Highest byte with two or more non-empty digits.
        int D = kDigitNone;
        for (int q = min(jb.z, passes) - 1; q >= 0; --q) {
          if (__syncthreads_count(tid < kRadix && jh[q * kRadix + tid] != 0) > 1) {
            D = q;
            break;
          }
        }
        if (D == kDigitNone) {
          if (c == 0 && tid == 0) ws.digit[j] = kDigitNone;
          __syncthreads();
          continue;
        }
        const int shift = D * kRadixBits;

        K kv[kItems];
        uint32_t vv[kItems];
        uint32_t rank2[kItems / 2];
        const int wbase = warp * (kItems * 32);
#pragma unroll
        for (int q = 0; q < kItems; ++q) {
          const int i = wbase + q * 32 + lane;
          if (i < clen) {
            kv[q] = src_k[cb + i];
            if constexpr (PAIRS) vv[q] = src_v[cb + i];
          }
        }
#pragma unroll
        for (int q = 0; q < kItems; ++q) {
          const int i = wbase + q * 32 + lane;
          const bool valid = i < clen;
          const uint32_t d = valid ? static_cast<uint32_t>((Ord::to_bits(kv[q]) >> shift) & (kRadix - 1))
                                   : 0u;
          const uint32_t peers = digit_peers(d, __ballot_sync(0xFFFFFFFFu, valid));
          const int leader = valid ? 31 - __clz(peers) : 0;
          uint32_t before = 0;
          if (valid && lane == leader) before = atomicAdd(&whist[warp * kRadix + d], __popc(peers));
          before = __shfl_sync(0xFFFFFFFFu, before, leader);
          const uint32_t r = before + __popc(peers & lt);
          if (q & 1) rank2[q >> 1] |= r << 16; else rank2[q >> 1] = r;
        }
        __syncthreads();

        // Per digit (threads [0, kRadix)): warp prefixes, chunk total,
        // look-back, global offsets.
        const int d = tid;
        const bool owner = d < kRadix;
        uint32_t tot = 0, excl = 0, hcount = 0;
        if (owner) {
#pragma unroll
          for (int w = 0; w < kLWarps; ++w) {
            const uint32_t x = whist[w * kRadix + d];
            whist[w * kRadix + d] = tot;
            tot += x;
          }
          uint32_t *st = ws.status + static_cast<size_t>(t) * kRadix;
          if (c == 0) {
            st_volatile(st + d, kFlagInclusive | tot);
          } else {
            st_volatile(st + d, kFlagAggregate | tot);
            const int64_t q_first = t - c;  // the job's first chunk (always inclusive)
            int64_t q = t - 1;
            while (true) {
              if (q < q_first) {  // unreachable: chunk q_first publishes an inclusive value
                raise_status(kStatusTimeout);
                break;
              }
              const uint32_t *qs = ws.status + static_cast<size_t>(q) * kRadix;
              uint32_t v = ld_volatile(qs + d);
              int spins = 0;
              while ((v >> 30) == 0 && spins < kLookbackSpinLimit) {
                if (spins > 64) __nanosleep(64);
                ++spins;
                v = ld_volatile(qs + d);
              }
              if ((v >> 30) == 0) {
                raise_status(kStatusTimeout);
                break;
              }
              excl += v & kValueMask;
              if (v & kFlagInclusive) break;
              --q;
            }
            st_volatile(st + d, kFlagInclusive | ((excl + tot) & kValueMask));
          }
          hcount = jh[D * kRadix + d];
        }
        const uint32_t boff = block_exclusive_sum(tot, warp_tmp);
        const uint32_t dbase = block_exclusive_sum(hcount, warp_tmp);
        if (owner) {
          boff_s[d] = boff;
          delta_s[d] = static_cast<int32_t>(dbase + excl) - static_cast<int32_t>(boff);
          if (c == 0) {  // the job's bucket starts, for the planning phase
            int32_t *bs = ws.bstart + static_cast<size_t>(j) * (kRadix + 1);
            bs[d] = static_cast<int32_t>(dbase);
            if (d == kRadix - 1) bs[kRadix] = static_cast<int32_t>(dbase + hcount);
            if (d == 0) ws.digit[j] = D;
          }
        }
        __syncthreads();

#pragma unroll
        for (int q = 0; q < kItems; ++q) {
          const int i = wbase + q * 32 + lane;
          if (i < clen) {
            const uint32_t dg = static_cast<uint32_t>((Ord::to_bits(kv[q]) >> shift) & (kRadix - 1));
            const uint32_t pos = boff_s[dg] + whist[warp * kRadix + dg] +
                                 ((rank2[q >> 1] >> ((q & 1) * 16)) & 0xFFFFu);
            ks[pos] = kv[q];
            if constexpr (PAIRS) vs[pos] = vv[q];
          }
        }
        __syncthreads();
        for (int i = tid; i < clen; i += kLThreads) {
          const K k = ks[i];
          const uint32_t dg = static_cast<uint32_t>((Ord::to_bits(k) >> shift) & (kRadix - 1));
          const int64_t dst = b + i + delta_s[dg];
          // Always inside [b, e) for well-formed offsets; the check keeps
          // overlapping malformed segments from writing outside their range.
          if (dst >= b && dst < e) {
            dst_k[dst] = k;
            if constexpr (PAIRS) dst_v[dst] = vs[i];
          }
        }
        __syncthreads();
      }
    }
    grid_barrier(ws.ctr);

    // ---- P4: bucket planning, one warp per job ---------------------------------
    {
      int32_t *bs_s = reinterpret_cast<int32_t *>(smem) + warp * (kRadix + 1);
      for (int64_t j = static_cast<int64_t>(blockIdx.x) * kLWarps + warp; j < nj; j += G * kLWarps) {
        const int4 jb = jobs[j];
        if (level == 0 && jb.y - jb.x <= CAP) {  // fits the bucket sort: sorted in place
          if (lane == 0) {
            const uint32_t k = atomicAdd(&ws.ctr[kCtrBuckets], 1u);
            if (k < ws.max_entries) ws.entries[k] = make_int4(jb.x, jb.y - jb.x, jb.w, kEntryDirect);
          }
          continue;
        }
        const int32_t D = ld_volatile(ws.digit + j);
        if (D == kDigitUnset) continue;  // not scattered (malformed offsets only)
        if (D >= 0) {
          const int32_t *bs = ws.bstart + static_cast<size_t>(j) * (kRadix + 1);
          for (int i = lane; i <= kRadix; i += 32) bs_s[i] = bs[i];
        }
        __syncwarp();
        if (lane == 0) {
          const int64_t len = jb.y - jb.x;
          // Two walks over the buckets: count the entries and next-level jobs,
          // reserve their slots with one atomic each, then write them.
          uint32_t e_base = 0, n_base = 0;
          for (int walk = 0; walk < 2; ++walk) {
            uint32_t ne = 0, nn = 0;
            // Copy [a, a + l) from tmp to the caller's buffers in CAP pieces.
            auto copy = [&](int64_t a, int64_t l) {
              for (int64_t o = 0; o < l; o += CAP, ++ne)
                if (walk == 1 && e_base + ne < ws.max_entries)
                  ws.entries[e_base + ne] =
                      make_int4(static_cast<int32_t>(a + o),
                                static_cast<int32_t>(min(l - o, static_cast<int64_t>(CAP))), jb.w,
                                kEntryCopy);
            };
            if (D == kDigitNone) {
              // Equal keys: in order already, in this level's source buffer.
              if (cur == 1) copy(jb.x, len);
            } else {
              // Greedy packing in one linear scan: chunk [d0, d) holds acc
              // elements; empty buckets join whichever chunk they fall in.
              int d0 = 0;
              int64_t acc = 0;
              for (int d = 0; d < kRadix; ++d) {
                const int64_t s0 = bs_s[d];
                const int64_t size = min(static_cast<int64_t>(bs_s[d + 1]), len) - s0;
                if (size <= 0) continue;
                if (size > CAP) {  // bucket d alone is longer than CAP
                  if (acc > 0) {
                    if (walk == 1 && e_base + ne < ws.max_entries)
                      ws.entries[e_base + ne] = make_int4(static_cast<int32_t>(j), d0, d, kEntrySort);
                    ++ne;
                  }
                  if (D == 0) {
                    // No byte left: equal keys, in stable order in this level's output.
                    if (cur == 0) copy(jb.x + s0, size);
                  } else {
                    if (walk == 1 && n_base + nn < static_cast<uint32_t>(ws.max_jobs))
                      next_jobs[n_base + nn] = make_int4(static_cast<int32_t>(jb.x + s0),
                                                         static_cast<int32_t>(jb.x + s0 + size), D, jb.w);
                    ++nn;
                  }
                  d0 = d + 1;
                  acc = 0;
                } else if (acc + size > CAP) {
                  if (walk == 1 && e_base + ne < ws.max_entries)
                    ws.entries[e_base + ne] = make_int4(static_cast<int32_t>(j), d0, d, kEntrySort);
                  ++ne;
                  d0 = d;
                  acc = size;
                } else {
                  acc += size;
                }
              }
              if (acc > 0) {
                if (walk == 1 && e_base + ne < ws.max_entries)
                  ws.entries[e_base + ne] = make_int4(static_cast<int32_t>(j), d0, kRadix, kEntrySort);
                ++ne;
              }
            }
            if (walk == 0) {
              if (ne) e_base = atomicAdd(&ws.ctr[kCtrBuckets], ne);
              if (nn) n_base = atomicAdd(&ws.ctr[kCtrJobs + (cur ^ 1)], nn);
              if (ne == 0 && nn == 0) break;
            }
          }
        }
        __syncwarp();
      }
    }
    grid_barrier(ws.ctr);

    // ---- P5: bucket sort (this level's scatter output -> caller's buffers) -----
    {
      const int64_t nent =
          min(static_cast<int64_t>(ld_volatile(&ws.ctr[kCtrBuckets])), ws.max_entries);
      int64_t next_t = 0;
      int4 next_e = make_int4(0, 0, 0, 0);
      if (tid == 0) {
        next_t = atomicAdd(&ws.ctr[kCtrBucketTicket], 1u);
        if (next_t < nent) next_e = ws.entries[next_t];
      }
      __shared__ int4 ent_s;
      while (true) {
        if (tid == 0) {
          tk_s = next_t;
          ent_s = next_e;
        }
        __syncthreads();
        const int64_t t = tk_s;
        const int4 en = ent_s;
        __syncthreads();
        if (t >= nent) break;
        if (tid == 0) {
          next_t = atomicAdd(&ws.ctr[kCtrBucketTicket], 1u);
          if (next_t < nent) next_e = ws.entries[next_t];
        }
        if (en.w == kEntryDirect) {
          const SideBuffers<K> B = sp(en.z);
          const int64_t a = en.x;
          const int m = en.y;
          if (m > 0 && m <= CAP)
            sort_chunk<Cfg, PAIRS>(B.keys + a, PAIRS ? B.vals + a : nullptr, B.keys + a,
                                   PAIRS ? B.vals + a : nullptr, m, false, [](auto &&) {}, smem,
                                   hb, warp_s);
          continue;
        }
        if (en.w == kEntryCopy) {
          const SideBuffers<K> B = sp(en.z);
          const int64_t a = en.x;
          const int m = en.y;
          for (int i = tid; i < m; i += kLThreads) {
            B.keys[a + i] = B.tmp_keys[a + i];
            if constexpr (PAIRS) B.vals[a + i] = B.tmp_vals[a + i];
          }
          continue;
        }
        const int4 jb = jobs[en.x];
        const SideBuffers<K> B = sp(jb.w);
        K *dst_k = cur == 0 ? B.tmp_keys : B.keys;
        uint32_t *dst_v = cur == 0 ? B.tmp_vals : B.vals;
        const int32_t *bs = ws.bstart + static_cast<size_t>(en.x) * (kRadix + 1);
        const int d0 = en.y, d1 = en.z;
        const int64_t s0 = bs[d0];
        const int64_t a = jb.x + s0;
        const int64_t m = static_cast<int64_t>(bs[d1]) - s0;
        if (m <= 0 || m > CAP || a < jb.x || a + m > jb.y) continue;  // malformed only
        // The buckets of one job are ordered by their digit, the highest byte
        // that varies in the job, so sorting the chunk as one segment by the
        // whole key sorts every bucket in it.
        sort_chunk<Cfg, PAIRS>(dst_k + a, PAIRS ? dst_v + a : nullptr, B.keys + a,
                               PAIRS ? B.vals + a : nullptr, static_cast<int>(m), false,
                               [](auto &&) {},
                               smem, hb, warp_s);
      }
    }
    grid_barrier(ws.ctr);
  }
}

}  // namespace segsort
