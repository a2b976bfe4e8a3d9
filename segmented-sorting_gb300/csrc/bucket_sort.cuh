// Bucket sort of a tile chunk: the first try for every chunk the tile kernel
// sorts, with the comparison sort of tile_sort.cuh as the fallback.
//
// A chunk holds whole segments (or one CAP-run of a long segment).  Every
// key of segment [s, t) (chunk positions) is sent to the bucket
//     s + floor(x * (t - s) / 2^W),
// x its order bits shifted left past the bits that are equal over the whole
// chunk (W = the bit width), so the buckets of a segment are its own
// positions, in key order: a key in a lower bucket is smaller than every key
// in a higher one.  With keys spread over their range the buckets hold about
// one key each.  One shared-memory atomic per key counts the buckets (and
// gives each key a slot in its bucket, in no particular order), an exclusive
// scan turns the counts into bucket starts, the keys -- as (order bits,
// chunk index) words, the tile sort's composite words without the segment
// field -- and the values are scattered to their buckets, and every key's
// final position is its bucket's start plus the number of the bucket's words
// below its own: the stable order.  A thread per slot keeps a warp's stores
// on consecutive positions.
//
// The ranking costs the sum of the squared bucket sizes.  When that sum is
// above kBucketSkew * m, or a bucket holds more than kBucketMaxSize keys, a
// second level spreads every bucket's keys over the bucket's own positions by
// where they lie inside it (x * (t - s) mod 2^W), which evens out densities
// that vary over the key range (float bit patterns).  A chunk still skewed
// after that (few distinct keys, many equal keys), or one whose keys can take
// fewer values than half its average segment, is refused: the function
// returns false having written nothing to the result (a chunk read from the
// temporary buffers is first copied to the caller's), and the caller sorts
// it with the comparison sort.  A chunk whose keys are all equal is already
// in its stable order (copied when the result goes elsewhere).
//
// The result is the same as the comparison sort's, bit for bit: both give the
// stable order of each segment, which is unique.  The reference sorts these
// lengths with per-length-bin register networks and block merges
// (src/bb_segsort/bb_segsort.h:71-164); this is a different method with the
// same output.
#pragma once

#include "tile_sort.cuh"

namespace segsort {

// Shortest average segment of a chunk the bucket sort is tried on: below it
// the comparison sort is faster (its merge levels stop at the segment length;
// on GB300, 2^24 u32 pairs: 0.20 against 0.25 ms at 64 keys per segment, even
// at 128).
constexpr int64_t kBucketMinAvg = 128;
constexpr uint32_t kBucketSkew = 3;      // sum of squared bucket sizes <= 3 m
constexpr uint32_t kBucketMaxSize = 24;  // largest bucket a thread ranks alone
// Buckets up to this size are ranked by an unrolled loop of this many
// compares; with about one key per bucket (Poisson sizes) a larger bucket
// is rare.
constexpr int kBucketUnroll = 6;

template <typename Bits>
__device__ __forceinline__ uint32_t bucket_scale(Bits x, uint32_t len);
template <>
__device__ __forceinline__ uint32_t bucket_scale<uint32_t>(uint32_t x, uint32_t len) {
  return __umulhi(x, len);
}
template <>
__device__ __forceinline__ uint32_t bucket_scale<uint64_t>(uint64_t x, uint32_t len) {
  return static_cast<uint32_t>(__umul64hi(x, static_cast<uint64_t>(len)));
}

template <typename Bits>
__device__ __forceinline__ int leading_zeros(Bits x);
template <>
__device__ __forceinline__ int leading_zeros<uint32_t>(uint32_t x) { return __clz(x); }
template <>
__device__ __forceinline__ int leading_zeros<uint64_t>(uint64_t x) {
  return __clzll(static_cast<long long>(x));
}

// Shared memory of the bucket sort (dynamic; the tile kernel's buffer is
// sized for the larger of this and the comparison sort's layout).
template <typename Cfg, bool PAIRS>
struct BucketLayout {
  static constexpr int CAP = Cfg::CAP;
  // Word[CAP + kPad]: the words past the chunk's last read as the largest
  // word, so the ranking of a bucket near the end never compares garbage.
  static constexpr int kPad = 8;
  static constexpr size_t kWords = 0;
  static constexpr size_t kVals = kWords + (CAP + kPad) * sizeof(typename Cfg::Word);  // uint32[CAP]
  static constexpr size_t kBkt = kVals + (PAIRS ? CAP * sizeof(uint32_t) : 0);  // uint16[CAP]
  static constexpr size_t kCnt = (kBkt + CAP * sizeof(uint16_t) + 15) / 16 * 16;
  // Bucket counters, then starts: one padding word per 32 keeps the blocked
  // scan free of bank conflicts; one past the last bucket holds m.
  static constexpr int kCntSlots = CAP + CAP / 32 + 2;
  static constexpr size_t kBytes = kCnt + kCntSlots * sizeof(uint32_t);
  static __device__ __forceinline__ int cslot(int b) { return b + (b >> 5); }
};

// Sorts chunk C by buckets, or returns false (uniformly over the CTA) having
// written nothing.  Every thread of the CTA calls it; hb is the tile
// kernel's head bitmask (CAP / 32 words), warp_s its scan scratch.  It passes
// a barrier before its first shared-memory write, so it may follow any other
// use of the shared memory; the caller synchronises before using the shared
// memory after it (the next call does).
template <typename Cfg, bool PAIRS, typename K>
__device__ __forceinline__ bool bucket_sort_body(const TileChunk &C, K *keys, uint32_t *vals,
                                                 const Offsets &off, K *tmp_keys,
                                                 uint32_t *tmp_vals, unsigned char *smem,
                                                 uint32_t *hb, int *warp_s) {
  using Ord = typename Cfg::Ord;
  using Bits = typename Cfg::Bits;
  using WT = typename Cfg::WT;
  using Word = typename Cfg::Word;
  using BL = BucketLayout<Cfg, PAIRS>;
  constexpr int NT = Cfg::NT;
  constexpr int CAP = Cfg::CAP;
  constexpr int IPT = CAP / NT;
  constexpr int NW = NT / 32;
  constexpr int HW = CAP / 32;  // head words
  constexpr int WPL = HW / 32;  // head words per lane of warp 0
  static_assert(HW % 32 == 0, "head words split evenly over a warp");
  static_assert(CAP <= 32768, "bucket and slot share a 32-bit word");
  __shared__ uint32_t red_s[4][NW];
  __shared__ int32_t hprev[HW], hnext[HW];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const ChunkIO<K, PAIRS> io(C, keys, vals, tmp_keys, tmp_vals);
  const int m = C.m;
  const bool multi = C.hi - C.lo > 1;
  Word *SW = reinterpret_cast<Word *>(smem + BL::kWords);
  uint32_t *SV = reinterpret_cast<uint32_t *>(smem + BL::kVals);
  uint16_t *SB = reinterpret_cast<uint16_t *>(smem + BL::kBkt);
  uint32_t *CN = reinterpret_cast<uint32_t *>(smem + BL::kCnt);

  // Per-segment flags (the MSD route's second stage): the order bits a
  // segment's keys share, which are shifted out too so that its keys spread
  // over its buckets, and whether the segment's keys are in the temporary
  // buffers (the MSD pass left them there).  Per head position in SH (over
  // the bucket indices' region, unused until the scatter).
  const bool hinted = off.flags != nullptr;
  uint8_t *SH = reinterpret_cast<uint8_t *>(smem + BL::kBkt);
  const uint8_t one_flag = hinted && !multi ? off.flags[C.lo] : 0;

  // Segment [s, t) of chunk position i (multi: from the head bitmask).
  auto bounds = [&](int i, int &s, int &t) {
    const int w = i >> 5, bit = i & 31;
    const uint32_t x = hb[w];
    const uint32_t below = x & (0xFFFFFFFFu >> (31 - bit));
    s = below ? (w << 5) + 31 - __clz(below) : max(hprev[w], 0);
    const uint32_t above = bit == 31 ? 0u : x & (0xFFFFFFFEu << bit);
    t = above ? (w << 5) + __ffs(above) - 1 : hnext[w];
  };
  // ---- keys and values to registers (position q * NT + tid), each from the
  // buffer its segment is in: first all from the buffer of the chunk's first
  // segment (in flight during the head phase), then, for a chunk of several
  // segments, again from the other buffer where a segment's flag says so
  // (only chunks that straddle an MSD segment's end) --------------------------------
  Bits kb[IPT];
  uint32_t kv[IPT];
  const bool spec_tmp = hinted && ((multi ? off.flags[C.lo] : one_flag) & kSegTmp) != 0;
  bool any_tmp = spec_tmp && m > 0;
  {
    const K *sk = (spec_tmp ? tmp_keys : keys) + C.a;
    const uint32_t *sv = PAIRS ? (spec_tmp ? tmp_vals : vals) + C.a : nullptr;
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
      const int i = q * NT + tid;
      kb[q] = 0;
      kv[q] = 0;
      if (i < m) {
        kb[q] = Ord::to_bits(sk[i]);
        if constexpr (PAIRS) kv[q] = sv[i];
      }
    }
  }
  __syncthreads();  // earlier readers of the shared memory are done
  for (int i = tid; i < BL::kCntSlots; i += NT) CN[i] = 0u;
  if (multi)
    for (int i = tid; i < HW; i += NT) hb[i] = 0u;
  // ---- segment heads; per head word the last head before it and the first
  // after it ------------------------------------------------------------------------
  bool other_buffer = false;  // a segment whose keys are not where the speculative load read
  if (multi) {
    __syncthreads();  // cleared head words
    for (int64_t j = C.lo + tid; j < C.hi; j += NT) {
      const int64_t b0 = off(j);
      const int64_t p = b0 - C.a;
      if (p >= 0 && p < m) {
        atomicOr(&hb[p >> 5], 1u << (p & 31));
        if (hinted && off(j + 1) > b0) {
          const uint8_t f = off.flags[j];
          SH[p] = f;
          other_buffer |= ((f & kSegTmp) != 0) != spec_tmp;
        }
      }
    }
    other_buffer = __syncthreads_or(other_buffer);
    if (warp == 0) {
      int last[WPL], first[WPL];
      int lmax = -1, lmin = m;
#pragma unroll
      for (int k = 0; k < WPL; ++k) {
        const int w = lane * WPL + k;
        const uint32_t x = hb[w];
        last[k] = x ? (w << 5) + 31 - __clz(x) : -1;
        first[k] = x ? (w << 5) + __ffs(x) - 1 : m;
        lmax = max(lmax, last[k]);
        lmin = min(lmin, first[k]);
      }
      // Exclusive running maximum over the lanes before, minimum over those after.
      int pre = lmax, suf = lmin;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, pre, o);
        const int z = __shfl_down_sync(0xFFFFFFFFu, suf, o);
        if (lane >= o) pre = max(pre, y);
        if (lane + o < 32) suf = min(suf, z);
      }
      pre = __shfl_up_sync(0xFFFFFFFFu, pre, 1);
      suf = __shfl_down_sync(0xFFFFFFFFu, suf, 1);
      if (lane == 0) pre = -1;
      if (lane == 31) suf = m;
#pragma unroll
      for (int k = 0; k < WPL; ++k) {
        hprev[lane * WPL + k] = pre;
        pre = max(pre, last[k]);
      }
#pragma unroll
      for (int k = WPL - 1; k >= 0; --k) {
        hnext[lane * WPL + k] = suf;
        suf = min(suf, first[k]);
      }
    }
    __syncthreads();
  }
  if (other_buffer) {
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
      const int i = q * NT + tid;
      if (i < m) {
        int s0, t0;
        bounds(i, s0, t0);
        const bool in_tmp = (SH[s0] & kSegTmp) != 0;
        if (in_tmp != spec_tmp) {
          kb[q] = Ord::to_bits((in_tmp ? tmp_keys : keys)[C.a + i]);
          if constexpr (PAIRS) kv[q] = (in_tmp ? tmp_vals : vals)[C.a + i];
        }
        any_tmp |= in_tmp;
      }
    }
  }
  // The chunk's AND and OR of the order bits.
  Bits band = ~Bits(0), bor = 0;
#pragma unroll
  for (int q = 0; q < IPT; ++q) {
    if (q * NT + tid < m) {
      band &= kb[q];
      bor |= kb[q];
    }
  }
  {
    const uint32_t a0 = __reduce_and_sync(0xFFFFFFFFu, static_cast<uint32_t>(band));
    const uint32_t o0 = __reduce_or_sync(0xFFFFFFFFu, static_cast<uint32_t>(bor));
    uint32_t a1 = 0, o1 = 0;
    if constexpr (sizeof(Bits) == 8) {
      a1 = __reduce_and_sync(0xFFFFFFFFu, static_cast<uint32_t>(static_cast<uint64_t>(band) >> 32));
      o1 = __reduce_or_sync(0xFFFFFFFFu, static_cast<uint32_t>(static_cast<uint64_t>(bor) >> 32));
    }
    if (lane == 0) {
      red_s[0][warp] = a0;
      red_s[1][warp] = a1;
      red_s[2][warp] = o0;
      red_s[3][warp] = o1;
    }
  }
  // Some key came from the temporary buffers: a refusal must leave the chunk
  // in the caller's, where the comparison sort reads it.
  const bool from_tmp = hinted && __syncthreads_or(any_tmp);
  if (!hinted) __syncthreads();
  auto write_back = [&](bool to_tmp) {
    K *dk = (to_tmp ? tmp_keys : keys) + C.a;
    uint32_t *dv = PAIRS ? (to_tmp ? tmp_vals : vals) + C.a : nullptr;
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
      const int i = q * NT + tid;
      if (i < m) {
        dk[i] = Ord::from_bits(kb[q]);
        if constexpr (PAIRS) dv[i] = kv[q];
      }
    }
  };
  // The warps' partials, combined across the lanes of every warp.
  static_assert(NW <= 32, "the warp partials fit one warp");
  Bits all_and, all_or;
  {
    const bool in = lane < NW;
    all_and = __reduce_and_sync(0xFFFFFFFFu, in ? red_s[0][lane] : 0xFFFFFFFFu);
    all_or = __reduce_or_sync(0xFFFFFFFFu, in ? red_s[2][lane] : 0u);
    if constexpr (sizeof(Bits) == 8) {
      all_and |= static_cast<Bits>(__reduce_and_sync(0xFFFFFFFFu, in ? red_s[1][lane] : 0xFFFFFFFFu)) << 32;
      all_or |= static_cast<Bits>(__reduce_or_sync(0xFFFFFFFFu, in ? red_s[3][lane] : 0u)) << 32;
    }
  }
  const Bits varying = all_and ^ all_or;  // bits that are not the same in every key
  if (varying == 0) {
    // Every key is equal: the stable order is the input order.
    if (from_tmp || C.tmp) write_back(C.tmp != 0);
    return true;
  }
  if (hinted && static_cast<int64_t>(C.hi - C.lo) * kBucketMinAvg > m) {
    // Short segments: the comparison sort is faster.
    if (from_tmp) write_back(false);
    return false;
  }
  const int sh = leading_zeros(varying);
  // Fewer possible key values than half the keys of an average segment
  // (low-entropy keys): equal keys would fill the buckets whatever the
  // scaling, and their atomics would serialise.  Refused before counting.
  {
    const int span = static_cast<int>(8 * sizeof(Bits)) - sh;  // bits that can differ
    const int64_t avg = m / max(C.hi - C.lo, 1);
    if (span < 31 && (int64_t{1} << span) < avg / 2) {
      if (from_tmp) write_back(false);
      return false;
    }
  }
  const int seg_sh = one_flag & kSegShared;
  // ---- bucket of every key; count (the old count is the key's slot) ----------------
  // The key's scaled position in its segment: bucket s + floor(x * len / 2^W)
  // and, in frac, the rest x * len mod 2^W (where it lies inside that bucket).
  auto place = [&](int q, int i, Bits &frac) -> int {
    int s = 0, t = m;
    if (multi) bounds(i, s, t);
    const uint32_t len = t > s ? static_cast<uint32_t>(t - s) : 1u;
    int shift = sh;
    if (hinted) shift = max(shift, multi ? static_cast<int>(SH[s] & kSegShared) : seg_sh);
    shift = min(shift, static_cast<int>(8 * sizeof(Bits)) - 1);
    const Bits x = kb[q] << shift;
    frac = x * static_cast<Bits>(len);
    const int b = s + static_cast<int>(bucket_scale<Bits>(x, len));
    return b < 0 ? 0 : (b >= m ? m - 1 : b);  // only malformed offsets reach the clamp
  };
  uint32_t pk[IPT];
#pragma unroll
  for (int q = 0; q < IPT; ++q) {
    const int i = q * NT + tid;
    pk[q] = 0;
    if (i < m) {
      Bits frac;
      const int b = place(q, i, frac);
      const uint32_t slot = atomicAdd(&CN[BL::cslot(b)], 1u);
      pk[q] = static_cast<uint32_t>(b) | (slot << 16);
    }
  }
  __syncthreads();
  // ---- exclusive scan of the counts (thread t: buckets [t*IPT, t*IPT+IPT));
  // sum of squared sizes and the largest bucket -------------------------------------
  auto scan_counts = [&](uint32_t &sq_all, uint32_t &mx_all) {
    uint32_t sum = 0, sq = 0, mx = 0;
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const uint32_t c = CN[BL::cslot(tid * IPT + j)];
      sum += c;
      sq += c * c;
      mx = max(mx, c);
    }
    uint32_t total;
    uint32_t run = block_exclusive_add<NT, false>(sum, total, warp_s);  // barrier below
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      uint32_t *at = CN + BL::cslot(tid * IPT + j);
      const uint32_t c = *at;
      *at = run;
      run += c;
    }
    if (tid == 0) CN[BL::cslot(CAP)] = total;
    const uint32_t sq_w = __reduce_add_sync(0xFFFFFFFFu, sq);
    const uint32_t mx_w = __reduce_max_sync(0xFFFFFFFFu, mx);
    if (lane == 0) {
      red_s[0][warp] = sq_w;
      red_s[1][warp] = mx_w;
    }
    __syncthreads();
    sq_all = __reduce_add_sync(0xFFFFFFFFu, lane < NW ? red_s[0][lane] : 0u);
    mx_all = __reduce_max_sync(0xFFFFFFFFu, lane < NW ? red_s[1][lane] : 0u);
  };
  auto skewed = [&](uint32_t sq_all, uint32_t mx_all) {
    return sq_all > kBucketSkew * static_cast<uint32_t>(m) || mx_all > kBucketMaxSize;
  };
  uint32_t sq_all, mx_all;
  scan_counts(sq_all, mx_all);
  if (skewed(sq_all, mx_all)) {
    // Second level: the keys of bucket c (start S, n keys) spread over the n
    // positions [S, S + n) by where they lie inside c (frac), which evens out
    // densities that vary over the key range (float bit patterns, for one:
    // every binade is a quarter of the patterns of the one above it but may
    // hold more keys).  Still in key order: a finer bucket of c is one of
    // c's positions, and frac grows with the key inside c.
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
      if (q * NT + tid < m) {
        const int c = static_cast<int>(pk[q] & 0xFFFFu);
        const uint32_t S = CN[BL::cslot(c)];
        pk[q] = S | ((CN[BL::cslot(c + 1)] - S) << 16);
      }
    }
    __syncthreads();
    for (int i = tid; i < BL::kCntSlots; i += NT) CN[i] = 0u;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < IPT; ++q) {
      const int i = q * NT + tid;
      if (i < m) {
        Bits frac;
        place(q, i, frac);
        const uint32_t S = pk[q] & 0xFFFFu, n = max(pk[q] >> 16, 1u);
        int f = static_cast<int>(S + bucket_scale<Bits>(frac, n));
        f = f >= m ? m - 1 : f;
        const uint32_t slot = atomicAdd(&CN[BL::cslot(f)], 1u);
        pk[q] = static_cast<uint32_t>(f) | (slot << 16);
      }
    }
    __syncthreads();
    scan_counts(sq_all, mx_all);
    if (skewed(sq_all, mx_all)) {
      if (from_tmp) write_back(false);
      return false;
    }
  }
  // ---- scatter to the buckets --------------------------------------------------------
#pragma unroll
  for (int q = 0; q < IPT; ++q) {
    const int i = q * NT + tid;
    if (i < m) {
      const int b = static_cast<int>(pk[q] & 0xFFFFu);
      const int p = static_cast<int>(CN[BL::cslot(b)] + (pk[q] >> 16));
      SW[p] = WT::make(kb[q], static_cast<uint32_t>(i));
      if constexpr (PAIRS) SV[p] = kv[q];
      SB[p] = static_cast<uint16_t>(b);
    }
  }
  if (tid < BL::kPad) SW[m + tid] = WT::maxv();
  __syncthreads();
  // ---- every slot's key to its place: its bucket's start plus the bucket's
  // words below it ----------------------------------------------------------------
  for (int p = tid; p < m; p += NT) {
    const int b = SB[p];
    const int S = static_cast<int>(CN[BL::cslot(b)]);
    const int E = static_cast<int>(CN[BL::cslot(b + 1)]);
    const Word w = SW[p];
    const int n = E - S;
    int r = 0;
    if (n > kBucketUnroll) {
      for (int y = S; y < E; ++y) r += WT::lt(SW[y], w);
    } else if (n > 1) {
      // Fixed trip count: a warp whose buckets differ in size does not
      // diverge.  Words past E are read (at most kBucketUnroll - 2 of them,
      // inside the padded array).  In a chunk of one segment they are never
      // below w -- later buckets hold larger keys, the padding the largest
      // word -- so they need no test; with several segments the next
      // segment's first buckets may hold smaller keys, so they are masked.
      if (!multi) {
#pragma unroll
        for (int k = 0; k < kBucketUnroll; ++k) r += WT::lt(SW[S + k], w);
      } else {
#pragma unroll
        for (int k = 0; k < kBucketUnroll; ++k) r += (k < n) & WT::lt(SW[S + k], w);
      }
    }
    io.dst_keys[S + r] = Ord::from_bits(WT::bits(w));
    if constexpr (PAIRS) io.dst_vals[S + r] = SV[p];
  }
  return true;
}

// ---------------------------------------------------------------------------
// The bucket route of the tile sort: two kernels.  tile_bucket_kernel: CTA t
// plans tile t (plan_tile) and bucket-sorts its chunks; a chunk of segments
// shorter than kBucketMinAvg on average, or one the bucket sort refuses, is
// appended to the fallback list.  tile_list_kernel: persistent CTAs sort the
// listed chunks with the comparison sort (its own launch shape: 256 threads,
// 128 registers).  The list holds at most kMaxTileChunks chunks per tile.
// ---------------------------------------------------------------------------
// One CTA of the bucket kernel: tile t of a problem (instance inst of a
// batch) whose half-tile map is half_first.
template <typename K, bool PAIRS, int NT, int KPT>
__device__ __forceinline__ void bucket_tile(K *__restrict__ keys, uint32_t *__restrict__ vals,
                                            const Offsets &off,
                                            const int32_t *__restrict__ half_first, int64_t t,
                                            K *__restrict__ tmp_keys,
                                            uint32_t *__restrict__ tmp_vals, int64_t radix_min,
                                            TileChunk *fallback, uint32_t *fallback_count,
                                            int64_t max_fallback, int32_t inst) {
  using Cfg = TileConfig<K, PAIRS, NT, KPT>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ TilePlan plan_s;
  __shared__ uint32_t hb[Cfg::CAP / 32];
  __shared__ int warp_s[NT / 16];
  if (t * Cfg::CAP >= off.n) return;
  if (threadIdx.x == 0)
    plan_tile<Cfg::CAP>(off, half_first, t, tmp_keys != nullptr, radix_min, plan_s);
  __syncthreads();
  const int nc = plan_s.nc;
  for (int c = 0; c < nc; ++c) {
    const TileChunk &C = plan_s.c[c];
    // With segment flags the body loads every chunk (some keys may be in the
    // temporary buffers) and makes the short-segment test itself.
    if ((off.flags != nullptr || static_cast<int64_t>(C.hi - C.lo) * kBucketMinAvg <= C.m) &&
        bucket_sort_body<Cfg, PAIRS>(C, keys, vals, off, tmp_keys, tmp_vals, smem, hb, warp_s))
      continue;
    if (threadIdx.x == 0) {
      const uint32_t at = atomicAdd(fallback_count, 1u);
      if (at < max_fallback) {
        TileChunk L = C;
        L.inst = inst;
        fallback[at] = L;
      }
    }
  }
}

template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_bucket_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                   const int32_t *__restrict__ half_first, K *__restrict__ tmp_keys,
                   uint32_t *__restrict__ tmp_vals, int64_t radix_min, TileChunk *fallback,
                   uint32_t *fallback_count, int64_t max_fallback) {
  pdl_wait();     // the classify kernel's map and jobs
  pdl_trigger();  // the list kernel may launch under this one (it waits for it)
  bucket_tile<K, PAIRS, NT, KPT>(keys, vals, off, half_first, blockIdx.x, tmp_keys, tmp_vals,
                                 radix_min, fallback, fallback_count, max_fallback, 0);
}

template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_list_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                 K *__restrict__ tmp_keys, uint32_t *__restrict__ tmp_vals,
                 const TileChunk *__restrict__ list, const uint32_t *count, int64_t max_list,
                 uint32_t *tickets) {
  using Cfg = TileConfig<K, PAIRS, NT, KPT>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t hb[Cfg::CAP / 32];
  __shared__ int warp_s[NT / 16];
  __shared__ int64_t next_s;
  pdl_wait();  // the list of the kernel before
  const int64_t c = min(static_cast<int64_t>(*count), max_list);
  // Chunks are taken from a ticket counter: a static split over the
  // resident CTAs ends unevenly (chunks cost alike).
  for (;;) {
    if (threadIdx.x == 0) next_s = static_cast<int64_t>(atomicAdd(tickets, 1u));
    __syncthreads();
    const int64_t i = next_s;
    __syncthreads();
    if (i >= c) break;
    const TileChunk C = list[i];
    sort_tile_chunk<Cfg, PAIRS>(C, keys, vals, off, tmp_keys, tmp_vals, smem, hb, warp_s);
  }
}

// The batched forms: CTA t of the bucket kernel takes the tile of the last
// instance whose first tile is at or before t (find_instance, as the batched
// comparison kernel); the list kernel finds each listed chunk's instance in
// the chunk.
template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_bucket_batch_kernel(const BatchInst *__restrict__ tab, int32_t count,
                         const int32_t *__restrict__ half_first, K *__restrict__ tmp_keys,
                         uint32_t *__restrict__ tmp_vals, int64_t radix_min,
                         TileChunk *fallback, uint32_t *fallback_count, int64_t max_fallback) {
  const int64_t t = blockIdx.x;
  const int32_t i = find_instance(tab, count, t, &BatchInst::tile_base);
  const BatchInst &I = tab[i];
  bucket_tile<K, PAIRS, NT, KPT>(static_cast<K *>(I.keys), I.vals, I.offsets_view(),
                                 half_first + I.half_base, t - I.tile_base,
                                 tmp_keys + I.tmp_base, PAIRS ? tmp_vals + I.tmp_base : nullptr,
                                 radix_min, fallback, fallback_count, max_fallback, i);
}

template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_list_batch_kernel(const BatchInst *__restrict__ tab, K *__restrict__ tmp_keys,
                       uint32_t *__restrict__ tmp_vals, const TileChunk *__restrict__ list,
                       const uint32_t *count, int64_t max_list, uint32_t *tickets) {
  using Cfg = TileConfig<K, PAIRS, NT, KPT>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t hb[Cfg::CAP / 32];
  __shared__ int warp_s[NT / 16];
  __shared__ int64_t next_s;
  const int64_t c = min(static_cast<int64_t>(*count), max_list);
  for (;;) {
    if (threadIdx.x == 0) next_s = static_cast<int64_t>(atomicAdd(tickets, 1u));
    __syncthreads();
    const int64_t i = next_s;
    __syncthreads();
    if (i >= c) break;
    const TileChunk C = list[i];
    const BatchInst &I = tab[C.inst];
    sort_tile_chunk<Cfg, PAIRS>(C, static_cast<K *>(I.keys), I.vals, I.offsets_view(),
                                tmp_keys + I.tmp_base, PAIRS ? tmp_vals + I.tmp_base : nullptr,
                                smem, hb, warp_s);
  }
}

}  // namespace segsort
