// Long segments by LSD radix sort: segments longer than the radix threshold
// (LargeWs::radix_min, at least the tile capacity).
//
// Every such segment is sorted by its own least-significant-digit radix sort
// over the order bits of its keys, 8-bit digits, one stable counting pass per
// digit: 4 passes for 32-bit keys, 8 for 64-bit keys.  All segments share
// each pass, so a pass is one phase of the cooperative long-segment kernel
// over the tiles of every radix segment, and the segments never mix because
// each one's buckets are placed inside its own range.
//
//   setup    every CTA numbers the tiles of every segment (a prefix over
//            the jobs, kept in its shared memory when it fits); CTA 0 also
//            stores it; every CTA clears its share of the jobs' digit counts.
//   counts   one read of the keys: per tile, the counts of every digit
//            position (shared-memory histograms), added into the segment's.
//   starts   per segment and digit position, the exclusive prefix of the 256
//            counts (where each bucket starts) and whether the position
//            varies at all: a digit every key of the segment shares is not
//            sorted by (the pass would be the identity).
//   pass d   per tile (CTA b takes tiles b, b + G, ...; every CTA of the
//            cooperative grid is resident and a tile waits only on the tiles
//            before it, so the CTA holding the lowest unfinished tile always
//            makes progress; when every segment has the same number of tiles,
//            tile t is tile t / nj of segment t mod nj, so that the tiles in
//            flight at once spread over the segments and their look-back
//            chains stay short): the tile's keys and values arrive in a staging
//            buffer by bulk asynchronous copy, issued while the CTA was
//            finishing the tile before; the stable rank of every key among
//            the tile's keys of its digit (lanes with equal digits found by
//            eight ballots, per-warp counters, a block scan); the tile's
//            count of each digit published for the tiles after it; the tile
//            reordered by digit in shared memory, which frees the staging
//            buffer for the next tile's copy; the counts of the segment's
//            tiles before it collected by decoupled look-back, sixteen
//            predecessors per round; the tile written to the other buffer,
//            each digit's keys to consecutive addresses.
//   copy     segments that ran an odd number of passes end in the temporary
//            buffers and are copied back.
//
// A pass reads and writes every key and value of the segment once (16 bytes
// per 32-bit key/value pair), plus 4 bytes per key for the counts: 68 bytes
// per pair for 32-bit keys, against 16 bytes per pair per merge pass of the
// merge route (tile_sort.cuh runs, merge_sort.cuh passes), whose pass count
// grows with log2 of the length.
//
// Stability: within a tile the ranks follow the tile's element order (warp,
// then item, then lane), the look-back adds the earlier tiles of the segment
// and the bucket start the smaller digits, so every pass is a stable counting
// sort and the result is the stable sort of the segment: the order
// std::stable_sort gives (src/bb_segsort/main.cu:152-173).
//
// It replaces the reference's merge passes over global memory for segments
// longer than one block (src/bb_segsort/bb_comput_l.h:567-1102 kern_block_merge,
// driven log2(len / 2048) times from :1264-1272) and CUB's one-CTA-per-segment
// radix sort (src/radixseg.cu:115-124).
#pragma once

#include "segsort_common.cuh"
#include "tile_sort.cuh"
#include "tile_stream.cuh"
#include "classify.cuh"

namespace segsort {

constexpr int kRBits = 8;
constexpr int kRBuckets = 1 << kRBits;  // one bucket per thread of the block
constexpr int kRItems = 16;             // keys per thread in a radix tile
constexpr int kLookSpinLimit = 1 << 22;  // ~0.3 s with the back-off below
constexpr int kLookWindow = 16;          // predecessors read per look-back round
constexpr int kLookEagerSpins = 32;      // polls before the look-back backs off
// rdigits flag of a segment on the MSD route: its digit mask holds only its
// top varying digit (one pass); the pass count and buffer parity use the
// mask bits alone.
constexpr uint32_t kRDigitMsd = 1u << 16;
constexpr uint32_t kRDigitMask = kRDigitMsd - 1u;
// rdigits flag of a segment the MSD stage leaves unsorted (it does not
// qualify and is not longer than the LSD threshold): the second stage sorts
// it like any other segment.
constexpr uint32_t kRDigitDefer = 1u << 17;
// A segment takes the MSD route when at least this many digit positions vary
// (fewer LSD passes cost less than the MSD pass, its copy-back and the tile
// pass over the sub-buckets) ...
constexpr int kMsdMinDigits = 3;
// ... and no bucket of its top varying digit holds more than this many keys
// times the tile capacity (a larger sub-bucket takes the merge passes).
constexpr int kMsdMaxBucketTiles = 4;

template <typename K, bool PAIRS, int NT>
struct RadixShape {
  static_assert(NT == kRBuckets, "one thread per bucket");
  using Bits = typename KeyOrder<K>::Bits;
  static constexpr int D = static_cast<int>(sizeof(Bits));  // digit positions
  static constexpr int IPT = kRItems;
  static constexpr int TILE = NT * IPT;
  static constexpr int NW = NT / 32;
  static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
  // Shared memory: the staging buffers of the bulk copies (the tile's 16-byte
  // granules: up to 16 bytes more than the tile), the reordered tile (keys,
  // then values), per-warp digit counters, the output shift of each digit,
  // the tile slots and the mbarrier of the copies.
  static constexpr size_t kStageK = 0;
  static constexpr size_t kStageV = kStageK + up16(static_cast<size_t>(TILE) * sizeof(K) + 16);
  static constexpr size_t kKeys = kStageV + (PAIRS ? up16(static_cast<size_t>(TILE) * 4 + 16) : 0);
  static constexpr size_t kVals = kKeys + static_cast<size_t>(TILE) * sizeof(K);
  static constexpr size_t kWarpCnt = kVals + (PAIRS ? static_cast<size_t>(TILE) * 4 : 0);
  static constexpr size_t kShift = kWarpCnt + static_cast<size_t>(NW) * kRBuckets * 4;
  static constexpr size_t kSlots = kShift + kRBuckets * 4;
  static constexpr size_t kBar = kSlots + 64;
  static constexpr size_t kBytes = kBar + 16;
  // Jobs whose tile prefix a CTA keeps in shared memory during the setup and
  // count phases (in the staging and reorder buffers, free then).
  static constexpr int kLocalJobs = static_cast<int>((kWarpCnt - kStageK) / 4) - 1;
  static_assert(static_cast<size_t>(D) * kRBuckets <= static_cast<size_t>(NW) * kRBuckets,
                "the count phase's histograms fit the warp counters");
};

// A tile as thread 0 describes it to the CTA: its index, segment (job),
// first position and length within the instance, index within the
// segment, the tile number of its look-back words (segment-major, so that a
// tile's predecessors are the numbers just below), the buffer it is read
// from, whether its segment varies in the pass's digit.
struct RadixSlot {
  int64_t t;
  int32_t j, a, cnt, k, w, from_tmp, active;
  int32_t pad;
};

// Radix tiles of a segment of len keys.
template <int TILE>
__host__ __device__ __forceinline__ int64_t radix_tiles(int64_t len) {
  return (len + TILE - 1) / TILE;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// The radix job that owns tile t: the last j in [0, nj) with
// rtile_prefix[j] <= t (the prefix is strictly increasing: every radix job
// spans at least two tiles).  Called by a whole warp; every round probes 32
// points of the remaining interval, so 2^15 jobs take three rounds of loads.
__device__ __forceinline__ int32_t warp_find_rjob(const int32_t *prefix, int32_t nj, int64_t t) {
  const int lane = threadIdx.x & 31;
  int32_t lo = 0, hi = nj - 1;  // the answer lies in [lo, hi]; prefix[0] = 0 <= t
  while (lo < hi) {
    const int32_t span = hi - lo;
    if (span <= 32) {
      const bool ok = lane < span && prefix[lo + 1 + lane] <= t;
      return lo + __popc(__ballot_sync(0xFFFFFFFFu, ok));
    }
    // Probes strictly inside (lo, hi), non-decreasing with the lane.
    const int32_t p = lo + static_cast<int32_t>((static_cast<int64_t>(span) * (lane + 1)) / 33);
    const int c = __popc(__ballot_sync(0xFFFFFFFFu, prefix[p] <= t));
    const int32_t at_last = __shfl_sync(0xFFFFFFFFu, p, c > 0 ? c - 1 : 0);
    const int32_t at_next = __shfl_sync(0xFFFFFFFFu, p, c < 32 ? c : 31);
    if (c > 0) lo = at_last;
    if (c < 32) hi = at_next - 1;
  }
  return lo;
}

template <typename Bits>
__device__ __forceinline__ uint32_t radix_digit(Bits b, int d) {
  return static_cast<uint32_t>(b >> (kRBits * d)) & (kRBuckets - 1);
}

// Look-back word of one (tile, bucket) in pass d: high half the tag
// 2 * (d + 1) (the tile's own count) or 2 * (d + 1) + 1 (the count of the
// segment's tiles up to and including this one), low half the count.  Words
// of earlier passes carry smaller tags and read as "not yet published"; the
// count travels in the same 64-bit word as its tag, so no fence is needed.
__device__ __forceinline__ unsigned long long look_word(uint32_t tag, uint32_t count) {
  return (static_cast<unsigned long long>(tag) << 32) | count;
}

// Lanes of the warp whose 8-bit digit equals this lane's, among the lanes
// with valid set (a valid lane is always its own peer).  Eight ballots, one
// per digit bit: each keeps the lanes that agree with this lane on that bit.
// Meaningless for lanes with valid clear.
__device__ __forceinline__ unsigned digit_peers(uint32_t dg, bool valid) {
  unsigned peers = __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
  for (int bit = 0; bit < kRBits; ++bit) {
    const bool set = ((dg >> bit) & 1u) != 0;
    const unsigned b = __ballot_sync(0xFFFFFFFFu, set);
    peers &= set ? b : ~b;
  }
  return peers;
}

// Decoupled look-back of bucket b for tile t, the k-th tile (k > 0) of its
// segment, whose own count (tag 2 * (d + 1)) is already published: collects
// the counts of the segment's earlier tiles -- kLookWindow of them per round
// of loads, nearest first, until one holds the inclusive count of the tiles
// before it -- and publishes the inclusive count.  Returns the keys of
// bucket b in the segment's tiles before this one.  A wait that gives up
// raises kStatusTimeout and goes on with what it has.
__device__ __forceinline__ uint32_t look_back_from(unsigned long long *look, int64_t t, int64_t k,
                                                   int b, uint32_t count, int d,
                                                   int spin_limit = kLookSpinLimit) {
  const uint32_t tag_own = 2u * static_cast<uint32_t>(d + 1);
  const uint32_t tag_incl = tag_own + 1u;
  const int64_t stop = t - k;  // the segment's first tile: it publishes inclusive counts
  uint32_t before = 0;
  bool done = false;
  for (int64_t p = t - 1; !done && p >= stop; p -= kLookWindow) {
    unsigned long long v[kLookWindow];
#pragma unroll
    for (int i = 0; i < kLookWindow; ++i)
      v[i] = p - i >= stop ? ld_relaxed_u64(look + (p - i) * kRBuckets + b) : 0ull;
#pragma unroll
    for (int i = 0; i < kLookWindow; ++i) {
      if (done || p - i < stop) continue;
      int spins = 0;
      while (static_cast<uint32_t>(v[i] >> 32) < tag_own) {
        if (++spins > spin_limit) break;
        if (spins > kLookEagerSpins) __nanosleep(32);
        v[i] = ld_relaxed_u64(look + (p - i) * kRBuckets + b);
      }
      if (static_cast<uint32_t>(v[i] >> 32) < tag_own) {  // gave up
        raise_status(kStatusTimeout);
        done = true;
        continue;
      }
      before += static_cast<uint32_t>(v[i]);
      if (static_cast<uint32_t>(v[i] >> 32) == tag_incl) done = true;
    }
  }
  st_relaxed_u64(look + t * kRBuckets + b, look_word(tag_incl, before + count));
  return before;
}

// The whole look-back of bucket b for tile t, the k-th tile of its segment:
// publishes the tile's count, then collects the earlier tiles' (k > 0).
__device__ __forceinline__ uint32_t look_back(unsigned long long *look, int64_t t, int64_t k,
                                              int b, uint32_t count, int d,
                                              int spin_limit = kLookSpinLimit) {
  const uint32_t tag_own = 2u * static_cast<uint32_t>(d + 1);
  st_relaxed_u64(look + t * kRBuckets + b, look_word(k == 0 ? tag_own + 1u : tag_own, count));
  return k == 0 ? 0u : look_back_from(look, t, k, b, count, d, spin_limit);
}

// ---------------------------------------------------------------------------
// The radix phases of the long-segment kernel.  Called by every CTA of the
// cooperative grid (NT threads each); returns once every radix segment is
// sorted into the caller's buffers, at once when there is none.  smem: at
// least RadixShape::kBytes of dynamic shared memory.
// ---------------------------------------------------------------------------
template <typename K, bool PAIRS, int NT, typename Space>
__device__ __forceinline__ void radix_phases(const Space &sp, const LargeWs<K> &ws,
                                             unsigned char *smem, int *warp_s) {
  using RS = RadixShape<K, PAIRS, NT>;
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  constexpr int D = RS::D;
  constexpr int IPT = RS::IPT;
  constexpr int TILE = RS::TILE;
  constexpr int NW = RS::NW;

  const int32_t nj = static_cast<int32_t>(min(static_cast<int64_t>(ld_volatile(&ws.ctr[kCtrRJobs])),
                                              static_cast<int64_t>(ws.max_rjobs)));
  if (nj == 0) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t G = gridDim.x;
  K *Sk = reinterpret_cast<K *>(smem + RS::kKeys);
  uint32_t *Sv = reinterpret_cast<uint32_t *>(smem + RS::kVals);
  K *stage_k = reinterpret_cast<K *>(smem + RS::kStageK);
  uint32_t *stage_v = reinterpret_cast<uint32_t *>(smem + RS::kStageV);
  uint32_t *wcnt = reinterpret_cast<uint32_t *>(smem + RS::kWarpCnt);  // [NW][256]
  int32_t *shift = reinterpret_cast<int32_t *>(smem + RS::kShift);       // [256]
  RadixSlot *slot = reinterpret_cast<RadixSlot *>(smem + RS::kSlots);    // the tile to process
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + RS::kBar);

  // ---- setup: tile numbering (every CTA; CTA 0 stores it), cleared counts ----
  // Thread i sums the tiles of a contiguous run of jobs, one block scan
  // places the runs, then each thread writes its jobs' prefixes.
  const bool local = nj <= RS::kLocalJobs;
  int32_t *lpre = reinterpret_cast<int32_t *>(smem + RS::kStageK);  // [nj + 1] when local
  int64_t ntiles;
  bool interleave;
  {
    const int per = (nj + NT - 1) / NT;
    const int j0 = min(tid * per, nj), j1 = min(j0 + per, nj);
    uint32_t sum = 0;
#pragma unroll 4
    for (int j = j0; j < j1; ++j) {
      const int4 jb = ws.rjobs[j];
      sum += static_cast<uint32_t>(radix_tiles<TILE>(jb.y > jb.x ? jb.y - jb.x : 0));
    }
    uint32_t mn = 0xFFFFFFFFu, mx = 0u;
    for (int j = j0; j < j1; ++j) {
      const int4 jb = ws.rjobs[j];
      const uint32_t c = static_cast<uint32_t>(radix_tiles<TILE>(jb.y > jb.x ? jb.y - jb.x : 0));
      mn = min(mn, c);
      mx = max(mx, c);
    }
    {
      __shared__ uint32_t mm_s[2][NT / 32];
      mn = __reduce_min_sync(0xFFFFFFFFu, mn);
      mx = __reduce_max_sync(0xFFFFFFFFu, mx);
      if (lane == 0) {
        mm_s[0][warp] = mn;
        mm_s[1][warp] = mx;
      }
      __syncthreads();
#pragma unroll
      for (int w = 0; w < NT / 32; ++w) {
        mn = min(mn, mm_s[0][w]);
        mx = max(mx, mm_s[1][w]);
      }
    }
    // Every segment the same number of tiles: interleaved tile order.
    interleave = nj > 1 && mn == mx;
    uint32_t total;
    uint32_t run = block_exclusive_add<NT>(sum, total, warp_s);
    for (int j = j0; j < j1; ++j) {
      const int4 jb = ws.rjobs[j];
      const int32_t at = static_cast<int32_t>(min(static_cast<int64_t>(run), ws.max_rtiles));
      if (local) lpre[j] = at;
      if (blockIdx.x == 0) ws.rtile_prefix[j] = at;
      run += static_cast<uint32_t>(radix_tiles<TILE>(jb.y > jb.x ? jb.y - jb.x : 0));
    }
    ntiles = min(static_cast<int64_t>(total), ws.max_rtiles);
    if (tid == 0) {
      if (local) lpre[nj] = static_cast<int32_t>(ntiles);
      if (blockIdx.x == 0) {
        ws.rtile_prefix[nj] = static_cast<int32_t>(ntiles);
        ws.ctr[kCtrRTiles] = static_cast<uint32_t>(ntiles);
      }
    }
  }
  {
    const int64_t words = static_cast<int64_t>(nj) * D * kRBuckets;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * NT + tid; i < words; i += G * NT)
      ws.rhist[i] = 0u;
  }
  grid_barrier(ws.ctr);

  // ---- counts: every digit position of every key, one read; the tile
  // descriptors the later phases read.  The next tile's keys are loaded
  // while this tile's are counted. ------------------------------------------
  {
    // The job of tile t: the local prefix (every thread, the same probes) or
    // a warp-cooperative search of the stored one.
    auto job_of = [&](int64_t t) -> int32_t {
      if (local) {
        int32_t lo = 0, hi = nj - 1;
        while (lo < hi) {
          const int32_t mid = (lo + hi + 1) >> 1;
          if (lpre[mid] <= t) lo = mid; else hi = mid - 1;
        }
        return lo;
      }
      return warp_find_rjob(ws.rtile_prefix, nj, t);
    };
    struct Tile {
      int64_t t;
      int32_t j;
      int cnt;
      Bits bits[IPT];
    };
    auto fetch = [&](int64_t t, Tile &T) {
      T.t = t;
      int64_t k;
      if (interleave) {
        T.j = static_cast<int32_t>(t % nj);
        k = t / nj;
      } else {
        T.j = job_of(t);
        k = t - (local ? lpre[T.j] : ws.rtile_prefix[T.j]);
      }
      const int4 jb = ws.rjobs[T.j];
      const int64_t a = jb.x + k * TILE;
      T.cnt = static_cast<int>(min(static_cast<int64_t>(TILE), static_cast<int64_t>(jb.y) - a));
      const K *src = sp(jb.w).keys + a;
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int e = i * NT + tid;
        T.bits[i] = e < T.cnt ? Ord::to_bits(src[e]) : Bits(0);
      }
      if (tid == 0)
        ws.rtile_desc[t] = make_int4(static_cast<int32_t>(a), T.cnt, T.j, static_cast<int32_t>(k));
      ws.rlook[t * kRBuckets + tid] = 0ull;  // the tile's look-back words, for the passes
    };
    Tile cur, nxt;
    if (static_cast<int64_t>(blockIdx.x) < ntiles) fetch(blockIdx.x, cur);
    for (int64_t t = blockIdx.x; t < ntiles; t += G) {
      if (t + G < ntiles) fetch(t + G, nxt);  // in flight while this tile is counted
      for (int i = tid; i < D * kRBuckets; i += NT) wcnt[i] = 0u;
      __syncthreads();
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int e = i * NT + tid;
        const bool valid = e < cur.cnt;
        const unsigned act = __ballot_sync(0xFFFFFFFFu, valid);
        if (act == 0u) continue;
        const int first = __ffs(act) - 1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const uint32_t dg = radix_digit(cur.bits[i], d);
          // A warp whose keys share the digit (low-entropy keys) adds once.
          const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, dg, first);
          if (__all_sync(0xFFFFFFFFu, !valid || dg == d0)) {
            if (lane == first) atomicAdd(&wcnt[d * kRBuckets + d0], static_cast<uint32_t>(__popc(act)));
          } else if (valid) {
            atomicAdd(&wcnt[d * kRBuckets + dg], 1u);
          }
        }
      }
      __syncthreads();
      uint32_t *gh = ws.rhist + static_cast<int64_t>(cur.j) * D * kRBuckets;
      for (int i = tid; i < D * kRBuckets; i += NT) {
        const uint32_t c = wcnt[i];
        if (c) atomicAdd(gh + i, c);
      }
      __syncthreads();
      cur = nxt;
    }
  }
  grid_barrier(ws.ctr);

  // ---- bucket starts and varying digits, one segment per CTA --------------
  for (int64_t j = blockIdx.x; j < nj; j += G) {
    const int4 jb = ws.rjobs[j];
    const uint32_t len = static_cast<uint32_t>(jb.y - jb.x);
    uint32_t *gh = ws.rhist + j * D * kRBuckets;
    uint32_t c[D];
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = gh[d * kRBuckets + tid];
    uint32_t varying = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      uint32_t tot;
      gh[d * kRBuckets + tid] = block_exclusive_add<NT>(c[d], tot, warp_s);
      if (!__syncthreads_or(c[d] == len)) varying |= 1u << d;
    }
    if (ws.msd_stage && __popc(varying) >= kMsdMinDigits) {
      // MSD route when the top varying digit splits the segment into
      // sub-buckets the tile sort can take.
      const int dt = 31 - __clz(varying);
      uint32_t mine = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) mine = d == dt ? c[d] : mine;
      const uint32_t wmax = __reduce_max_sync(0xFFFFFFFFu, mine);
      if (lane == 0) warp_s[warp] = static_cast<int>(wmax);
      __syncthreads();
      uint32_t mx = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) mx = max(mx, static_cast<uint32_t>(warp_s[w]));
      __syncthreads();
      // (A sub-bucket must stay at most the radix threshold: the second
      // stage gives longer ones radix passes, which read the caller's buffers.)
      const int64_t lim = min(static_cast<int64_t>(kMsdMaxBucketTiles) * ws.tile_cap, ws.radix_min);
      if (mx <= static_cast<uint64_t>(lim)) varying = (1u << dt) | kRDigitMsd;
    }
    if (ws.msd_stage && !(varying & kRDigitMsd) && static_cast<int64_t>(len) <= ws.lsd_min)
      varying = kRDigitDefer;
    if (tid == 0) {
      ws.rdigits[j] = varying;
      if (varying) atomicOr(&ws.ctr[kCtrRDigits], varying);
    }
  }
  grid_barrier(ws.ctr);
  const uint32_t any_varying = ld_volatile(&ws.ctr[kCtrRDigits]);

  // ---- one stable counting pass per digit position that varies ------------
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t copies = 0;  // bulk-copy phases of the mbarrier so far
  // Thread 0: describes tile t of pass d in *sl from its descriptor and its
  // segment's varying digits (loaded ahead by the caller).
  auto describe = [&](int64_t t, const int4 &de, uint32_t varying, int32_t base, int d,
                      RadixSlot *sl) {
    sl->t = t;
    sl->j = de.z;
    sl->a = de.x;
    sl->cnt = de.y;
    sl->k = de.w;
    sl->w = base + de.w;
    sl->from_tmp = __popc(varying & ((1u << d) - 1u)) & 1;
    sl->active = (varying >> d) & 1u;
  };
  // Thread 0: bulk copies of the tile in *sl into the staging buffers.
  auto issue = [&](const RadixSlot *sl, int instance) {
    const SideBuffers<K> B = sp(instance);
    const K *src_k = (sl->from_tmp ? B.tmp_keys : B.keys) + sl->a;
    const StagedSpan<K> rk(src_k, sl->cnt);
    uint32_t bytes = rk.bytes();
    const uint32_t *src_v = nullptr;
    if constexpr (PAIRS) {
      src_v = (sl->from_tmp ? B.tmp_vals : B.vals) + sl->a;
      bytes += StagedSpan<uint32_t>(src_v, sl->cnt).bytes();
    }
    mbar_arrive_expect_tx(bar, bytes);
    rk.issue(stage_k, src_k, bar);
    if constexpr (PAIRS) StagedSpan<uint32_t>(src_v, sl->cnt).issue(stage_v, src_v, bar);
  };
#pragma unroll 1
  for (int d = 0; d < D; ++d) {
    if (!((any_varying >> d) & 1u)) continue;  // uniform: no CTA has work
    if (tid == 0 && static_cast<int64_t>(blockIdx.x) < ntiles) {
      // The keys were written by the previous phase (generic proxy, made
      // visible by the grid barrier); the bulk copies read them through the
      // async proxy.
      asm volatile("fence.proxy.async.global;" ::: "memory");
      const int4 de = ws.rtile_desc[blockIdx.x];
      describe(blockIdx.x, de, ws.rdigits[de.z], ws.rtile_prefix[de.z], d, &slot[0]);
      if (slot[0].active) issue(&slot[0], ws.rjobs[de.z].w);
    }
    __syncthreads();
    for (int64_t t = blockIdx.x; t < ntiles; t += G) {
      const RadixSlot cur = slot[0];
      // Thread 0 loads the next tile's descriptor now and uses it once this
      // tile has left the staging buffers.
      const int64_t tn = t + G;
      int4 nde = make_int4(0, 0, 0, 0);
      if (tid == 0 && tn < ntiles) nde = ws.rtile_desc[tn];
      if (!cur.active) {  // the segment does not vary in this digit (uniform)
        __syncthreads();  // every thread has read slot[0]
        if (tid == 0 && tn < ntiles) {
          describe(tn, nde, ws.rdigits[nde.z], ws.rtile_prefix[nde.z], d, &slot[0]);
          if (slot[0].active) issue(&slot[0], ws.rjobs[nde.z].w);
        }
        __syncthreads();
        continue;
      }
      const int cnt = cur.cnt;
      int mis_k, mis_v = 0;
      {
        const SideBuffers<K> B = sp(ws.rjobs[cur.j].w);
        mis_k = StagedSpan<K>((cur.from_tmp ? B.tmp_keys : B.keys) + cur.a, cnt).mis;
        if constexpr (PAIRS)
          mis_v = StagedSpan<uint32_t>((cur.from_tmp ? B.tmp_vals : B.vals) + cur.a, cnt).mis;
      }

      // Wait for the staged tile (bounded).  A wait that gives up raises
      // kStatusTimeout and waits once more, so that no copy of this tile can
      // still be landing when the next one is issued or the kernel ends.
      if (!mbar_wait(bar, copies & 1u)) {
        if (tid == 0) raise_status(kStatusTimeout);
        mbar_wait(bar, copies & 1u);
      }
      ++copies;
      // Thread 0: the next tile's segment, loaded under the ranking.
      uint32_t nvary = 0;
      int ninst = 0;
      int32_t nbase = 0;
      if (tid == 0 && tn < ntiles) {
        nvary = ws.rdigits[nde.z];
        ninst = ws.rjobs[nde.z].w;
        nbase = ws.rtile_prefix[nde.z];
      }

      // Keys of the tile, read from the staging buffer where needed: warp w
      // takes positions [w * 32 * IPT, ...), item i of lane l is position
      // w * 32 * IPT + 32 * i + l (consecutive lanes, consecutive words).
      const int wbase = warp * 32 * IPT;
      const K *sk = stage_k + mis_k + wbase + lane;
      uint32_t rank[IPT];
      uint32_t *wc = wcnt + warp * kRBuckets;
#pragma unroll
      for (int q = 0; q < kRBuckets / 32; ++q) wc[q * 32 + lane] = 0u;
      __syncwarp();
      // Rank of each key among the warp's earlier keys of its digit: the
      // lowest lane of each digit bumps the warp's counter and hands the old
      // count to the others.
      auto rank_item = [&](int i, bool valid) {
        const uint32_t dg = valid ? radix_digit(Ord::to_bits(sk[32 * i]), d) : 0u;
        const unsigned peers = digit_peers(dg, valid);
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0u;
        if (valid && lane == leader) {
          old = wc[dg];
          wc[dg] = old + __popc(peers);
        }
        old = __shfl_sync(0xFFFFFFFFu, old, leader & 31);
        rank[i] = old + __popc(peers & lanemask_lt());
        __syncwarp();
      };
      if (cnt == TILE) {
#pragma unroll
        for (int i = 0; i < IPT; ++i) rank_item(i, true);
      } else {
#pragma unroll
        for (int i = 0; i < IPT; ++i) rank_item(i, wbase + 32 * i + lane < cnt);
      }
      __syncthreads();
      // Thread b owns bucket b: the warps' counts become their first local
      // positions; the tile's count is published for the tiles after it.
      const int b = tid;
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const uint32_t c = wcnt[w * kRBuckets + b];
        wcnt[w * kRBuckets + b] = run;
        run += c;
      }
      const uint32_t tag_own = 2u * static_cast<uint32_t>(d + 1);
      st_relaxed_u64(ws.rlook + static_cast<int64_t>(cur.w) * kRBuckets + b,
                     look_word(cur.k == 0 ? tag_own + 1u : tag_own, run));
      uint32_t tile_total;
      const uint32_t lstart = block_exclusive_add<NT>(run, tile_total, warp_s);
#pragma unroll
      for (int w = 0; w < NW; ++w) wcnt[w * kRBuckets + b] += lstart;
      __syncthreads();
      // Reorder the tile by digit in shared memory (values straight from the
      // staging buffer).
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int e = wbase + 32 * i + lane;
        if (e < cnt) {
          const K kk = sk[32 * i];
          const uint32_t p = wc[radix_digit(Ord::to_bits(kk), d)] + rank[i];
          Sk[p] = kk;
          if constexpr (PAIRS) Sv[p] = stage_v[mis_v + e];
        }
      }
      __syncthreads();  // staging buffers consumed
      if (tid == 0 && tn < ntiles) {
        describe(tn, nde, nvary, nbase, d, &slot[0]);
        if (slot[0].active) {
          fence_proxy_async();
          issue(&slot[0], ninst);
        }
      }
      // The counts of the segment's tiles before this one.
      const uint32_t before = cur.k == 0 ? 0u : look_back_from(ws.rlook, cur.w, cur.k, b, run, d);
      const uint32_t bstart = ws.rhist[(static_cast<int64_t>(cur.j) * D + d) * kRBuckets + b];
      shift[b] = static_cast<int32_t>(bstart + before) - static_cast<int32_t>(lstart);
      __syncthreads();
      // Local position p of digit g goes to segment position shift[g] + p.
      // With well-formed offsets that is always inside the segment; the
      // test keeps overlapping segments (malformed, non-monotone offsets,
      // whose counts need not match the keys a pass reads) from writing
      // outside their own range.
      const int4 jb = ws.rjobs[cur.j];
      const SideBuffers<K> B = sp(jb.w);
      K *dst_k = (cur.from_tmp ? B.keys : B.tmp_keys) + jb.x;
      uint32_t *dst_v = PAIRS ? (cur.from_tmp ? B.vals : B.tmp_vals) + jb.x : nullptr;
      const uint32_t len = static_cast<uint32_t>(jb.y - jb.x);
#pragma unroll 4
      for (int q = 0; q < IPT; ++q) {
        const int p = q * NT + tid;
        if (p < cnt) {
          const K kk = Sk[p];
          const int32_t to = shift[radix_digit(Ord::to_bits(kk), d)] + p;
          if (static_cast<uint32_t>(to) < len) {
            dst_k[to] = kk;
            if constexpr (PAIRS) dst_v[to] = Sv[p];
          }
        }
      }
      __syncthreads();  // Sk, Sv and shift are free again; slot[0] is the next tile
    }
    grid_barrier(ws.ctr);
  }

  // ---- segments that ran an odd number of passes: tmp -> caller ------------
  for (int64_t t = blockIdx.x; t < ntiles; t += G) {
    const int4 de = ws.rtile_desc[t];
    // (Not the MSD route's segments: their second stage reads the temporary
    // buffers.)
    const uint32_t v = ws.rdigits[de.z];
    if (!(__popc(v & kRDigitMask) & 1) || (v & kRDigitMsd)) continue;
    const int cnt = de.y;
    const SideBuffers<K> B = sp(ws.rjobs[de.z].w);
    K kk[IPT];
    uint32_t vv[IPT];
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int e = i * NT + tid;
      if (e < cnt) {
        kk[i] = B.tmp_keys[de.x + e];
        if constexpr (PAIRS) vv[i] = B.tmp_vals[de.x + e];
      }
    }
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int e = i * NT + tid;
      if (e < cnt) {
        B.keys[de.x + e] = kk[i];
        if constexpr (PAIRS) B.vals[de.x + e] = vv[i];
      }
    }
  }
  __syncthreads();
}

}  // namespace segsort
