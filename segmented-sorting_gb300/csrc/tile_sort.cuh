// Tile sort: every segment of at most CAP = NT * KPT elements is sorted by
// one CTA, entirely in shared memory and registers (one HBM read and one HBM
// write per element).
//
// Work split.  Half-tiles are CAP/2 elements wide; half_first[h] (written by
// the classify kernel) is the first segment starting at or after h * CAP/2.
// CTA t owns the segments starting in half-tiles 2t and 2t+1.  In a half-tile
// every segment but the last is at most CAP/2 long (a longer one runs past
// the half-tile's end, so nothing else starts after it there), so the short
// segments of a half-tile span less than CAP elements and form one chunk; the
// two halves' chunks are joined when they are contiguous and fit together.
// A last segment longer than CAP/2 is a chunk of its own (up to CAP) or, when
// longer than CAP, a long segment whose first CAP-run the CTA sorts for the
// merge passes.  With the CAP-run of a long segment that started before the
// tile, a CTA sorts at most five chunks (kMaxTileChunks), found from three
// half_first entries and a few offsets, without any search.
//
// Chunk sort.  Every element becomes a composite word
//     (segment start within the chunk, order bits of the key, chunk index)
// compared as one unsigned integer.  Words are unique, so any sorting method
// gives the stable per-segment order the reference's oracle produces with
// std::stable_sort (src/bb_segsort/main.cu:152-173), and segments never mix
// because the segment start is the most significant field.  Segment starts
// come from a shared-memory bitmask of segment heads and a block-wide running
// maximum.  The sort is a merge sort: each thread sorts KPT words in registers
// with a sorting network, then log2(chunk / KPT) merge-path levels merge pairs
// of runs through shared memory.  A pair whose runs are already in order (last
// word of the first run <= first word of the second) is left as it is, so
// chunks of short aligned segments skip the upper levels.  Values are staged
// once in shared memory and gathered through the index field at the end.
//
// The reference sorts these lengths with one kernel per power-of-two length
// bin (src/bb_segsort/bb_segsort.h:71-164, bins from bb_bin.h:54-100) using
// unstable register networks; this kernel replaces that whole family and its
// host round trip for the bin counts (bb_bin.h:46).
#pragma once

#include <cstring>

#include "segsort_common.cuh"

namespace segsort {

// ---------------------------------------------------------------------------
// Composite words.
// ---------------------------------------------------------------------------
template <typename Bits> struct WordTraits;

// 32-bit order bits: [63]=0 | [62:48] segment start | [47:16] bits | [15:0] index
template <> struct WordTraits<uint32_t> {
  using T = uint64_t;
  static __device__ __forceinline__ T make(uint32_t bits, uint32_t idx) {
    return (static_cast<uint64_t>(bits) << 16) | idx;
  }
  static __device__ __forceinline__ T with_seg(T w, uint32_t seg_start) {
    return w | (static_cast<uint64_t>(seg_start) << 48);
  }
  static __device__ __forceinline__ uint32_t bits(T w) { return static_cast<uint32_t>(w >> 16); }
  static __device__ __forceinline__ uint32_t index(T w) { return static_cast<uint32_t>(w) & 0xFFFFu; }
  static __device__ __forceinline__ uint32_t seg(T w) { return static_cast<uint32_t>(w >> 48); }
  static __device__ __forceinline__ T maxv() { return ~0ull; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
};

// 64-bit order bits: hi = [63]=0 | [62:48] segment start | [47:0] bits[63:16]
//                    lo = [31:16] bits[15:0] | [15:0] index
struct Word96 {
  uint64_t hi;
  uint32_t lo;
  uint32_t pad;
};

template <> struct WordTraits<uint64_t> {
  using T = Word96;
  static __device__ __forceinline__ T make(uint64_t bits, uint32_t idx) {
    T w;
    w.hi = bits >> 16;
    w.lo = (static_cast<uint32_t>(bits & 0xFFFFu) << 16) | idx;
    w.pad = 0;
    return w;
  }
  static __device__ __forceinline__ T with_seg(T w, uint32_t seg_start) {
    w.hi |= static_cast<uint64_t>(seg_start) << 48;
    return w;
  }
  static __device__ __forceinline__ uint64_t bits(T w) {
    return ((w.hi & 0xFFFFFFFFFFFFull) << 16) | (w.lo >> 16);
  }
  static __device__ __forceinline__ uint32_t index(T w) { return w.lo & 0xFFFFu; }
  static __device__ __forceinline__ uint32_t seg(T w) { return static_cast<uint32_t>(w.hi >> 48); }
  static __device__ __forceinline__ T maxv() {
    T w;
    w.hi = ~0ull;
    w.lo = ~0u;
    w.pad = 0;
    return w;
  }
  static __device__ __forceinline__ bool le(T a, T b) {
    return (a.hi < b.hi) || (a.hi == b.hi && a.lo <= b.lo);
  }
  static __device__ __forceinline__ bool lt(T a, T b) {
    return (a.hi < b.hi) || (a.hi == b.hi && a.lo < b.lo);
  }
};

// ---------------------------------------------------------------------------
// Shared-memory layout and launch shape of one tile-sort instantiation.
// ---------------------------------------------------------------------------
template <typename K, bool PAIRS, int NT_, int KPT_>
struct TileConfig {
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  using WT = WordTraits<Bits>;
  using Word = typename WT::T;
  static constexpr int NT = NT_;
  static constexpr int KPT = KPT_;
  static constexpr int CAP = NT * KPT;
  static_assert((KPT & (KPT - 1)) == 0, "items per thread must be a power of two");
  static_assert((NT & (NT - 1)) == 0, "threads per CTA must be a power of two");
  static_assert(CAP <= 32768, "chunk index and segment start are 15-bit fields");
  // One padding word per 128 bytes keeps blocked (thread-contiguous) word
  // accesses free of bank conflicts.
  static constexpr int WUNIT = 128 / static_cast<int>(sizeof(Word));
  static constexpr int WSLOTS = CAP + CAP / WUNIT;
  // Output staging (keys then values), one padding slot per 32 elements.
  static constexpr int OSLOTS = CAP + CAP / 32;
  static constexpr int HALF = CAP / 2;
  static constexpr size_t kWordBytes = static_cast<size_t>(WSLOTS) * sizeof(Word);
  static constexpr size_t kOutBytes =
      static_cast<size_t>(OSLOTS) * (sizeof(K) + (PAIRS ? sizeof(uint32_t) : 0));
  static constexpr size_t kMainBytes =
      ((kWordBytes > kOutBytes ? kWordBytes : kOutBytes) + 15) / 16 * 16;
  static constexpr size_t kValBytes = PAIRS ? CAP * sizeof(uint32_t) : 0;
  static constexpr size_t kSmemBytes = kMainBytes + kValBytes;

  static __device__ __forceinline__ int wslot(int i) { return i + i / WUNIT; }
  static __device__ __forceinline__ int oslot(int i) { return i + (i >> 5); }
};

// Sorting network over KPT words held in registers (ascending): Batcher's
// odd-even merge sort, 63 compare-exchanges for 16 words and 19 for 8 (the
// bitonic network takes 80 and 24).  BatcherNet<N>::pair(c) enumerates the
// network's exchanges in order at compile time, and thread_sort instantiates
// one exchange per index, so every word index is a constant and the words
// stay in registers.  Checked exhaustively over 0-1 inputs (the 0-1
// principle) for 4, 8 and 16 words.
template <int N>
struct BatcherNet {
  struct Pair {
    int a, b;
  };
  // Exchange number `c` (a < b); {-1, -1} past the end.
  static constexpr Pair pair(int c) {
    int at = 0;
    for (int p = 1; p < N; p <<= 1)
      for (int k = p; k >= 1; k >>= 1)
        for (int j = k % p; j + k < N; j += 2 * k)
          for (int i = 0; i < k && i < N - j - k; ++i)
            if ((i + j) / (2 * p) == (i + j + k) / (2 * p)) {
              if (at == c) return Pair{i + j, i + j + k};
              ++at;
            }
    return Pair{-1, -1};
  }
  static constexpr int count() {
    int c = 0;
    while (pair(c).a >= 0) ++c;
    return c;
  }
};

template <typename WT, int KPT, int C = 0>
__device__ __forceinline__ void thread_sort(typename WT::T (&w)[KPT]) {
  if constexpr (C < BatcherNet<KPT>::count()) {
    constexpr int a = BatcherNet<KPT>::pair(C).a;
    constexpr int b = BatcherNet<KPT>::pair(C).b;
    const typename WT::T x = w[a], y = w[b];
    const bool swap = WT::lt(y, x);
    w[a] = swap ? y : x;
    w[b] = swap ? x : y;
    thread_sort<WT, KPT, C + 1>(w);
  }
}
static_assert(BatcherNet<16>::count() == 63 && BatcherNet<8>::count() == 19,
              "Batcher's network sizes");

// `rounds` rounds of odd-even transposition over KPT words (even pairs first).
// Any run of at most `rounds` words is sorted afterwards, whichever parity
// its first position has, when no exchange crosses its ends.
template <typename WT, int KPT>
__device__ __forceinline__ void transposition_sort(typename WT::T (&w)[KPT], int rounds) {
  auto cas = [](typename WT::T &a, typename WT::T &b) {
    const typename WT::T x = a, y = b;
    const bool swap = WT::lt(y, x);
    a = swap ? y : x;
    b = swap ? x : y;
  };
  for (int r = 0; r < rounds; ++r) {
    if ((r & 1) == 0) {
#pragma unroll
      for (int i = 0; i + 1 < KPT; i += 2) cas(w[i], w[i + 1]);
    } else {
#pragma unroll
      for (int i = 1; i + 1 < KPT; i += 2) cas(w[i], w[i + 1]);
    }
  }
}

// Longest segment (in words) for which the transposition rounds cost fewer
// exchanges than the sorting network: about KPT/2 - 1/2 exchanges a round
// against 63 (16 words) or 19 (8 words) for Batcher's network.
template <int KPT>
constexpr int kTranspositionMaxRounds = KPT >= 16 ? 8 : (KPT >= 8 ? 5 : 2);

// ---------------------------------------------------------------------------
// Range copies between global memory and per-element callbacks: 16-byte
// vector accesses for the aligned middle, UNROLL vectors per thread in flight,
// scalar accesses for the unaligned head and tail.  The pair forms move keys
// and values in one loop when both arrays share their 16-byte alignment.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ int align_head(const T *p, int m) {
  const int h = static_cast<int>(((16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15) / sizeof(T));
  return h < m ? h : m;
}

template <int NT, int UNROLL, typename T, typename F>
__device__ __forceinline__ void load_range(const T *__restrict__ src, int m, F &&f) {
  constexpr int V = 16 / static_cast<int>(sizeof(T));
  const int tid = threadIdx.x;
  const int head = align_head(src, m);
  const int nvec = (m - head) / V;
  const int tail0 = head + nvec * V;
  if (tid < head) f(tid, __ldcs(src + tid));
  const uint4 *pv = reinterpret_cast<const uint4 *>(src + head);
  for (int k0 = tid; k0 < nvec; k0 += UNROLL * NT) {
    uint4 v[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const int k = k0 + u * NT;
      if (k < nvec) v[u] = __ldcs(pv + k);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const int k = k0 + u * NT;
      if (k < nvec) {
        T e[V];
        memcpy(e, &v[u], 16);
#pragma unroll
        for (int c = 0; c < V; ++c) f(head + k * V + c, e[c]);
      }
    }
  }
  if (tail0 + tid < m) f(tail0 + tid, __ldcs(src + tail0 + tid));
}

// 32-bit keys and 32-bit values with the same alignment: one loop.
template <int NT, int UNROLL, typename K, typename FK, typename FV>
__device__ __forceinline__ void load_pairs(const K *__restrict__ ks, const uint32_t *__restrict__ vs,
                                           int m, FK &&fk, FV &&fv) {
  static_assert(sizeof(K) == 4, "paired loop needs 32-bit keys");
  const int head = align_head(ks, m);
  if (head != align_head(vs, m)) {
    load_range<NT, UNROLL>(ks, m, fk);
    load_range<NT, UNROLL>(vs, m, fv);
    return;
  }
  const int tid = threadIdx.x;
  const int nvec = (m - head) / 4;
  const int tail0 = head + nvec * 4;
  if (tid < head) {
    fk(tid, __ldcs(ks + tid));
    fv(tid, __ldcs(vs + tid));
  }
  const uint4 *pk = reinterpret_cast<const uint4 *>(ks + head);
  const uint4 *pvv = reinterpret_cast<const uint4 *>(vs + head);
  for (int k0 = tid; k0 < nvec; k0 += UNROLL * NT) {
    uint4 a[UNROLL], b[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const int k = k0 + u * NT;
      if (k < nvec) {
        a[u] = __ldcs(pk + k);
        b[u] = __ldcs(pvv + k);
      }
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const int k = k0 + u * NT;
      if (k < nvec) {
        K e[4];
        memcpy(e, &a[u], 16);
        const int i = head + k * 4;
        fk(i, e[0]); fk(i + 1, e[1]); fk(i + 2, e[2]); fk(i + 3, e[3]);
        fv(i, b[u].x); fv(i + 1, b[u].y); fv(i + 2, b[u].z); fv(i + 3, b[u].w);
      }
    }
  }
  if (tail0 + tid < m) {
    fk(tail0 + tid, __ldcs(ks + tail0 + tid));
    fv(tail0 + tid, __ldcs(vs + tail0 + tid));
  }
}

template <int NT, typename T, typename G>
__device__ __forceinline__ void store_range(T *__restrict__ dst, int m, G &&g) {
  constexpr int V = 16 / static_cast<int>(sizeof(T));
  const int tid = threadIdx.x;
  const int head = align_head(dst, m);
  const int nvec = (m - head) / V;
  const int tail0 = head + nvec * V;
  if (tid < head) __stcs(dst + tid, g(tid));
  uint4 *pv = reinterpret_cast<uint4 *>(dst + head);
  for (int k = tid; k < nvec; k += NT) {
    T e[V];
#pragma unroll
    for (int c = 0; c < V; ++c) e[c] = g(head + k * V + c);
    uint4 v;
    memcpy(&v, e, 16);
    __stcs(pv + k, v);
  }
  if (tail0 + tid < m) __stcs(dst + tail0 + tid, g(tail0 + tid));
}

// Asks L2 for the elements [0, count) of p: one prefetch per 128-byte line,
// spread over the CTA's threads.  A hint for data a later CTA or item reads.
template <int NT, typename T>
__device__ __forceinline__ void prefetch_l2(const T *p, int64_t count) {
  const char *b = reinterpret_cast<const char *>(p);
  const int64_t bytes = count * static_cast<int64_t>(sizeof(T));
  for (int64_t o = static_cast<int64_t>(threadIdx.x) * 128; o < bytes; o += NT * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(b + o));
}

// Exclusive running maximum over the threads of the CTA (-1 for thread 0).
template <int NT>
__device__ __forceinline__ int block_exclusive_max(int v, int *warp_s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x = max(x, y);
  }
  int before = __shfl_up_sync(0xFFFFFFFFu, x, 1);
  if (lane == 0) before = -1;
  if (lane == 31) warp_s[warp] = x;
  __syncthreads();
#pragma unroll
  for (int w = 0; w < NT / 32; ++w)
    if (w < warp) before = max(before, warp_s[w]);
  __syncthreads();
  return before;
}

// In one pass: the exclusive running maximum of a over the threads of the CTA
// (-1 for thread 0) and the maximum of b (-1 when every b is -1).  warp_s
// holds 2 * NT / 32 ints.
template <int NT>
__device__ __forceinline__ void block_exmax_max(int a, int b, int &a_before, int &b_max,
                                                int *warp_s) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = a;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x = max(x, y);
  }
  int before = __shfl_up_sync(0xFFFFFFFFu, x, 1);
  if (lane == 0) before = -1;
  const int bw = static_cast<int>(__reduce_max_sync(0xFFFFFFFFu, static_cast<unsigned>(b + 1))) - 1;
  if (lane == 31) warp_s[warp] = x;
  if (lane == 0) warp_s[NW + warp] = bw;
  __syncthreads();
  int r = -1;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    if (w < warp) before = max(before, warp_s[w]);
    r = max(r, warp_s[NW + w]);
  }
  __syncthreads();
  a_before = before;
  b_max = r;
}

// Block-wide sum (exclusive prefix and total) of one value per thread.
// kSyncAfter: a closing barrier, so that warp_s may be written again at
// once (callers that pass another barrier first leave it out).
template <int NT, bool kSyncAfter = true>
__device__ __forceinline__ uint32_t block_exclusive_add(uint32_t v, uint32_t &total, int *warp_s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_s[warp] = static_cast<int>(x);
  __syncthreads();
  // Every warp scans the warp totals across its lanes.
  constexpr int NW = NT / 32;
  static_assert(NW <= 32, "the warp totals fit one warp");
  uint32_t w = lane < NW ? static_cast<uint32_t>(warp_s[lane]) : 0u;
#pragma unroll
  for (int o = 1; o < NW; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
    if (lane >= o) w += y;
  }
  const uint32_t before = __shfl_sync(0xFFFFFFFFu, w, warp > 0 ? warp - 1 : 0);
  total = __shfl_sync(0xFFFFFFFFu, w, NW - 1);
  if constexpr (kSyncAfter) __syncthreads();
  return (warp > 0 ? before : 0u) + x - v;
}

// Writes a sorted chunk: thread t holds the words of positions
// [t*KPT, t*KPT+KPT); they are staged as keys and gathered values in shared
// memory (over the word buffer, which must no longer be read) and stored with
// 16-byte stores.
template <typename Cfg, bool PAIRS, typename K>
__device__ __forceinline__ void write_chunk(const typename Cfg::Word (&w)[Cfg::KPT], int m,
                                            unsigned char *smem, K *dst_keys,
                                            uint32_t *dst_vals) {
  using Ord = typename Cfg::Ord;
  using WT = typename Cfg::WT;
  constexpr int NT = Cfg::NT;
  constexpr int KPT = Cfg::KPT;
  K *KO = reinterpret_cast<K *>(smem);
  uint32_t *VO = reinterpret_cast<uint32_t *>(smem + Cfg::OSLOTS * sizeof(K));
  const uint32_t *Vs = reinterpret_cast<const uint32_t *>(smem + Cfg::kMainBytes);
  const int base = threadIdx.x * KPT;
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const int i = base + j;
    if (i < m) {
      KO[Cfg::oslot(i)] = Ord::from_bits(WT::bits(w[j]));
      if constexpr (PAIRS) VO[Cfg::oslot(i)] = Vs[WT::index(w[j])];
    }
  }
  __syncthreads();
  store_range<NT>(dst_keys, m, [&](int i) { return KO[Cfg::oslot(i)]; });
  if constexpr (PAIRS) store_range<NT>(dst_vals, m, [&](int i) { return VO[Cfg::oslot(i)]; });
  __syncthreads();
}


// ---------------------------------------------------------------------------
// The element sinks a chunk loader feeds: key i of the chunk becomes word i
// (order bits, chunk index) in W, value i goes to Vs, and segment heads set
// bits of the head bitmask hb.
// ---------------------------------------------------------------------------
template <typename Cfg, typename K>
struct ChunkSinks {
  unsigned char *smem;
  uint32_t *hb;
  int m;
  __device__ __forceinline__ void key(int i, K k) const {
    reinterpret_cast<typename Cfg::Word *>(smem)[Cfg::wslot(i)] =
        Cfg::WT::make(Cfg::Ord::to_bits(k), static_cast<uint32_t>(i));
  }
  __device__ __forceinline__ void val(int i, uint32_t v) const {
    reinterpret_cast<uint32_t *>(smem + Cfg::kMainBytes)[i] = v;
  }
  __device__ __forceinline__ void head(int64_t p) const {
    if (p >= 0 && p < m) atomicOr(&hb[p >> 5], 1u << (p & 31));
  }
};

// Clears the head bitmask of a chunk of several segments; the caller
// synchronises before the loader runs.
template <int NT>
__device__ __forceinline__ void clear_heads(uint32_t *hb, int m, bool multi) {
  if (multi)
    for (int i = threadIdx.x; i < (m + 31) / 32; i += NT) hb[i] = 0;
}

template <typename Cfg, bool PAIRS, typename K, bool kShort = false, typename Dst>
__device__ __forceinline__ void sort_loaded(Dst &&dst, int m, bool multi, unsigned char *smem,
                                            uint32_t *hb, int *warp_s);

// Destination arrays of a sorted chunk.
template <typename K>
struct ChunkDst {
  K *dst_keys;
  uint32_t *dst_vals;
};

// ---------------------------------------------------------------------------
// Sorts one chunk of m <= CAP elements: reads src_keys/src_vals[0, m), writes
// the result to dst_keys/dst_vals[0, m) (the same arrays for an in-place
// sort; every read finishes before the first write).  `multi` says the chunk
// holds more than one segment; then heads(set) is called by every thread and
// must call set(p) for the local start p of each segment (any thread, any
// order, repeats allowed).
// ---------------------------------------------------------------------------
template <typename Cfg, bool PAIRS, typename K, bool kShort = false, typename Heads>
__device__ __forceinline__ void sort_chunk(const K *src_keys, const uint32_t *src_vals,
                                           K *dst_keys, uint32_t *dst_vals, int m, bool multi,
                                           Heads &&heads, unsigned char *smem, uint32_t *hb,
                                           int *warp_s) {
  constexpr int NT = Cfg::NT;
  clear_heads<NT>(hb, m, multi);
  if (multi) __syncthreads();
  // ---- load: keys -> words, values -> Vs, segment heads -> bitmask ----------
  const ChunkSinks<Cfg, K> S{smem, hb, m};
  auto fk = [&](int i, K k) { S.key(i, k); };
  auto fv = [&](int i, uint32_t v) { S.val(i, v); };
  if constexpr (PAIRS && sizeof(K) == 4) {
    load_pairs<NT, 4>(src_keys, src_vals, m, fk, fv);
  } else {
    load_range<NT, 4>(src_keys, m, fk);
    if constexpr (PAIRS) load_range<NT, 4>(src_vals, m, fv);
  }
  if (multi) heads([&](int64_t p) { S.head(p); });
  __syncthreads();
  sort_loaded<Cfg, PAIRS, K, kShort>([&] { return ChunkDst<K>{dst_keys, dst_vals}; }, m, multi,
                                     smem, hb, warp_s);
}

// The sort proper of a loaded chunk: W holds word i at slot wslot(i), Vs the
// values, hb the segment heads (when multi); every thread has passed a
// barrier since the loads.  dst() gives the destination (members dst_keys,
// dst_vals); it is called when the sorted chunk is written.  kShort compiles
// in the transposition rounds for chunks of short segments (the streamed
// kernel, which runs problems of short segments; kept out of the plain
// kernel, whose register allocation for the merge levels it disturbs).
template <typename Cfg, bool PAIRS, typename K, bool kShort, typename Dst>
__device__ __forceinline__ void sort_loaded(Dst &&dst, int m, bool multi, unsigned char *smem,
                                            uint32_t *hb, int *warp_s) {
  using WT = typename Cfg::WT;
  using Word = typename Cfg::Word;
  constexpr int NT = Cfg::NT;
  constexpr int KPT = Cfg::KPT;
  Word *W = reinterpret_cast<Word *>(smem);
  const int tid = threadIdx.x;
  const int base = tid * KPT;

  // ---- blocked words + segment field ------------------------------------------
  // The merge at level l joins runs of KPT * 2^l words and has work only where
  // one of its run boundaries -- an odd multiple of KPT * 2^l, i.e. the first
  // position of a thread t with ctz(t) = l -- falls inside a segment.  A chunk
  // of several segments runs only the levels up to the highest such one (none
  // at all when every thread's first position starts a segment).
  Word w[KPT];
  int levels = 31;
  uint32_t mask = 0;  // segment heads among this thread's positions (bit j: base + j)
  if (multi) {
    constexpr uint32_t kLow = KPT >= 32 ? 0xFFFFFFFFu : ((1u << KPT) - 1);
    mask = base < m ? (hb[base >> 5] >> (base & 31)) & kLow : 0u;
    const int mylast = mask ? base + 31 - __clz(mask) : -1;
    const int need = (tid > 0 && base < m && !(mask & 1u)) ? __ffs(tid) - 1 : -1;
    int carry, top;
    block_exmax_max<NT>(mylast, need, carry, top, warp_s);
    levels = top + 1;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const int i = base + j;
      if (i < m) {
        const uint32_t mj = mask & ((2u << j) - 1u);
        const int h = mj ? base + 31 - __clz(mj) : carry;
        w[j] = WT::with_seg(W[Cfg::wslot(i)], static_cast<uint32_t>(h));
      } else {
        w[j] = WT::maxv();
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const int i = base + j;
      w[j] = (i < m) ? W[Cfg::wslot(i)] : WT::maxv();
    }
  }

  // ---- in-register sort ----------------------------------------------------------
  // Without merge levels no segment crosses a thread's block, and R rounds of
  // odd-even transposition sort every segment of at most R words (words of
  // different segments are already in order, so no exchange crosses a
  // segment's boundary): cheaper than the sorting network for short ones.
  int rounds = KPT;
  if (kShort && levels == 0) {
    const int lim = base < m ? min(KPT, m - base) : 0;
    uint32_t rest = (mask | (1u << lim)) & ~1u;  // segment ends after position 0
    int longest = 0, prev = 0;
    while (rest) {
      const int b = __ffs(rest) - 1;
      longest = max(longest, b - prev);
      prev = b;
      rest &= rest - 1;
    }
    rounds = static_cast<int>(__reduce_max_sync(0xFFFFFFFFu, static_cast<unsigned>(longest)));
  }
  if constexpr (kShort) {
    if (rounds <= kTranspositionMaxRounds<KPT>) {
      transposition_sort<WT, KPT>(w, rounds);
    } else {
      thread_sort<WT, KPT>(w);
    }
  } else {
    thread_sort<WT, KPT>(w);
  }

  // ---- merge levels ---------------------------------------------------------------
  // A level whose pairs of runs span at most one warp (2 * run <= 32 * KPT)
  // reads and writes only its own warp's part of W, so a warp barrier
  // orders it; a level whose pairs span several warps needs block barriers,
  // and so does the level after it (its readers crossed warps).  Before the
  // first level every thread has read only its own words.
  bool dirty = true;  // W does not hold this thread's current words
  bool prev_local = true;
  int level = 0;
  for (int run = KPT; run < m && level < levels; run <<= 1, ++level) {
    const int pair_threads = (2 * run) / KPT;
    const bool local = pair_threads <= 32;
    if (prev_local) __syncwarp(); else __syncthreads();  // previous readers of W are done
    if (dirty) {
#pragma unroll
      for (int j = 0; j < KPT; ++j) W[Cfg::wslot(base + j)] = w[j];
    }
    if (local) __syncwarp(); else __syncthreads();
    prev_local = local;
    const int r = tid & (pair_threads - 1);
    const int a_beg = (tid - r) * KPT;
    const int a_end = a_beg + run;
    const int b_end = a_end + run;
    // Run A holds the sorted words of chunk positions [a_beg, a_end) and run B
    // those of [a_end, b_end).  Segments are contiguous and the segment start
    // is the top field, so every word of A is below every word of B except
    // for the one segment that straddles position a_end.  Runs already in
    // order: the merge is the concatenation, which is what this thread holds
    // (and what W holds at its slots).
    const Word x_last = W[Cfg::wslot(a_end - 1)];
    const Word y_first = W[Cfg::wslot(a_end)];
    if (WT::le(x_last, y_first)) {
      dirty = false;
      continue;
    }
    // Only the straddling segment's words [lo_p, hi_p) move.  They are a
    // suffix of A and a prefix of B, so a thread whose own words (the run
    // positions it holds) miss segment sg keeps them without searching.
    int lo_p = a_beg, hi_p = b_end;
    if (multi) {
      const uint32_t sg = WT::seg(y_first);
      const bool in_a = base < a_end;
      if (WT::seg(in_a ? w[KPT - 1] : w[0]) != sg) {
        dirty = false;
        continue;
      }
      int l = a_beg, h = a_end - 1;  // first word of A in segment sg
      while (l < h) {
        const int mid = (l + h) >> 1;
        if (WT::seg(W[Cfg::wslot(mid)]) < sg) l = mid + 1; else h = mid;
      }
      lo_p = l;
      l = a_end + 1;
      h = b_end;  // first word of B past segment sg
      while (l < h) {
        const int mid = (l + h) >> 1;
        if (WT::seg(W[Cfg::wslot(mid)]) <= sg) l = mid + 1; else h = mid;
      }
      hi_p = l;
    }
    if (base + KPT <= lo_p || base >= hi_p) {
      dirty = false;
      continue;
    }
    dirty = true;
    const int la = a_end - lo_p, lb = hi_p - a_end;
    const int p0 = base > lo_p ? base : lo_p;
    const int diag = p0 - lo_p;
    int l = diag > lb ? diag - lb : 0;
    int h = diag < la ? diag : la;
    while (l < h) {
      const int mid = (l + h) >> 1;
      const Word x = W[Cfg::wslot(lo_p + mid)];
      const Word y = W[Cfg::wslot(a_end + diag - 1 - mid)];
      if (WT::le(x, y)) l = mid + 1; else h = mid;
    }
    int ai = lo_p + l;
    int bi = a_end + diag - l;
    Word av = ai < a_end ? W[Cfg::wslot(ai)] : WT::maxv();
    Word bv = bi < hi_p ? W[Cfg::wslot(bi)] : WT::maxv();
    auto step = [&](Word &out) {
      const bool take_a = WT::le(av, bv);
      out = take_a ? av : bv;
      ai += take_a;
      bi += !take_a;
      const int nx = take_a ? ai : bi;
      const int lim = take_a ? a_end : hi_p;
      const Word nv = nx < lim ? W[Cfg::wslot(nx)] : WT::maxv();
      av = take_a ? nv : av;
      bv = take_a ? bv : nv;
    };
    if (base >= lo_p && base + KPT <= hi_p) {
      // Every position of this thread is in the merge (always, for a chunk
      // of one segment): no per-position check.
#pragma unroll
      for (int j = 0; j < KPT; ++j) step(w[j]);
    } else {
#pragma unroll
      for (int j = 0; j < KPT; ++j) {
        const int p = base + j;
        if (p >= lo_p && p < hi_p) step(w[j]);
      }
    }
  }
  __syncthreads();
  const auto out = dst();
  write_chunk<Cfg, PAIRS>(w, m, smem, out.dst_keys, out.dst_vals);
}

// Merge passes a long segment of len elements needs after its CAP-runs are
// sorted: ceil(log2(ceil(len / CAP))).
__host__ __device__ __forceinline__ int merge_passes(int64_t len, int64_t cap) {
  int p = 0;
  for (int64_t runs = (len + cap - 1) / cap; runs > 1; runs = (runs + 1) >> 1) ++p;
  return p;
}

// ---------------------------------------------------------------------------
// The chunks of one tile.  A chunk is m elements from element a on; lo < hi:
// it holds the segments [lo, hi) (several when hi - lo > 1); lo == hi: it is
// a CAP-run of long segment lo; tmp: its result goes to the temporary
// buffers (the buffer the segment's first merge pass reads).
// ---------------------------------------------------------------------------
constexpr int kMaxTileChunks = 5;
struct TileChunk {
  int64_t a;
  int32_t lo, hi, m, tmp;
  int32_t inst;  // instance of a batch (the bucket route's fallback list; 0 otherwise)
};
struct TilePlan {
  TileChunk c[kMaxTileChunks];
  int32_t nc;
};

// The chunk list of tile t of a problem whose half-tile map is half_first
// (null: the problem is one tile, n <= CAP, and the plan is one chunk with
// every segment).  runs: the caller forms the CAP-runs of long segments.
//
// With runs, the plan also holds the sorted runs of long segments (longer
// than CAP, at most radix_min: longer ones take the radix passes and are not
// touched here) for the merge passes: every CAP-chunk [b + k*CAP, ...) of such a
// segment is sorted by the CTA of the tile its first element lies in, into
// the buffer the segment's first merge pass reads (the caller's buffers when
// the segment needs an even number of passes, tmp otherwise, so that its last
// pass writes the caller's buffers).  A tile holds at most one such chunk of
// the segment running into it and the first chunk of at most one long
// segment starting in each of its halves.  One thread computes a plan.
template <int CAP>
__device__ __forceinline__ void plan_tile(const Offsets &off, const int32_t *__restrict__ half_first,
                                          int64_t t, bool runs, int64_t radix_min, TilePlan &P) {
  constexpr int64_t HALF = CAP / 2;
  const int64_t nseg = off.nseg;
  int nc = 0;
  auto add = [&](int64_t lo, int64_t hi) {
    if (hi <= lo) return;
    const int64_t a = off(lo);
    const int64_t m = off(hi) - a;
    if (m <= 0 || m > CAP) return;
    P.c[nc] = TileChunk{a, static_cast<int32_t>(lo), static_cast<int32_t>(hi),
                        static_cast<int32_t>(m), 0};
    ++nc;
  };
  // The CAP-chunk of long segment s that starts at c.
  auto add_run = [&](int64_t s, int64_t c) {
    if (!runs) return;
    const int64_t b = off(s), e = off(s + 1);
    if (e - b <= CAP || e - b > radix_min || c < b || c >= e) return;
    P.c[nc] = TileChunk{c, static_cast<int32_t>(s), static_cast<int32_t>(s),
                        static_cast<int32_t>(min(static_cast<int64_t>(CAP), e - c)),
                        merge_passes(e - b, CAP) & 1};
    ++nc;
  };
  if (half_first == nullptr) {
    add(0, nseg);
  } else if (t * CAP < off.n) {
    auto clampi = [&](int64_t v, int64_t lo) { return v < lo ? lo : (v > nseg ? nseg : v); };
    const int64_t h0 = clampi(__ldg(half_first + 2 * t), 0);
    const int64_t h1 = clampi(__ldg(half_first + 2 * t + 1), h0);
    const int64_t h2 = clampi(__ldg(half_first + 2 * t + 2), h1);
    // A long segment that starts before the tile and runs into it.
    if (runs && h0 > 0) {
      const int64_t b = off(h0 - 1), e = off(h0), t0 = t * CAP;
      if (e - b > CAP && b < t0 && e > t0) {
        const int64_t c = b + (t0 - b + CAP - 1) / CAP * CAP;
        if (c < e && c < t0 + CAP) add_run(h0 - 1, c);
      }
    }
    // A last segment of a half-tile longer than HALF is a chunk of its own,
    // or, when longer than CAP, a long segment whose first run starts here.
    const bool big_a = h1 > h0 && off(h1) - off(h1 - 1) > HALF;
    const bool big_b = h2 > h1 && off(h2) - off(h2 - 1) > HALF;
    const int64_t end_a = big_a ? h1 - 1 : h1;
    const int64_t end_b = big_b ? h2 - 1 : h2;
    if (!big_a && off(end_b) - off(h0) <= CAP) {
      add(h0, end_b);  // both halves' short segments in one chunk
    } else {
      add(h0, end_a);
      if (big_a) {
        add(h1 - 1, h1);
        add_run(h1 - 1, off(h1 - 1));
      }
      add(h1, end_b);
    }
    if (big_b) {
      add(h2 - 1, h2);
      add_run(h2 - 1, off(h2 - 1));
    }
  }
  P.nc = nc;
}

// Where chunk C of a tile reads and writes.
template <typename K, bool PAIRS>
struct ChunkIO {
  const K *src_keys;
  const uint32_t *src_vals;
  K *dst_keys;
  uint32_t *dst_vals;
  __device__ __forceinline__ ChunkIO(const TileChunk &C, K *keys, uint32_t *vals, K *tmp_keys,
                                     uint32_t *tmp_vals) {
    src_keys = keys + C.a;
    src_vals = PAIRS ? vals + C.a : nullptr;
    dst_keys = (C.tmp ? tmp_keys : keys) + C.a;
    dst_vals = PAIRS ? (C.tmp ? tmp_vals : vals) + C.a : nullptr;
  }
};

// Sorts chunk C of a tile with loads straight from global memory.
template <typename Cfg, bool PAIRS, bool kShort = false, typename K>
__device__ __forceinline__ void sort_tile_chunk(const TileChunk &C, K *keys, uint32_t *vals,
                                                const Offsets &off, K *tmp_keys,
                                                uint32_t *tmp_vals, unsigned char *smem,
                                                uint32_t *hb, int *warp_s) {
  const ChunkIO<K, PAIRS> io(C, keys, vals, tmp_keys, tmp_vals);
  const int64_t a = C.a, lo = C.lo, hi = C.hi;
  sort_chunk<Cfg, PAIRS, K, kShort>(io.src_keys, io.src_vals, io.dst_keys, io.dst_vals, C.m,
                                    hi - lo > 1,
                         [&](auto &&set) {
                           for (int64_t j = lo + threadIdx.x; j < hi; j += Cfg::NT)
                             set(off(j) - a);
                         },
                         smem, hb, warp_s);
}


// ---------------------------------------------------------------------------
// One CTA of the tile sort: tile t of a problem whose half-tile map is
// half_first (null: the problem is one tile).  With tmp_keys given the CTA
// also forms the CAP-runs of the long segments of at most radix_min
// elements (plan_tile).
// ---------------------------------------------------------------------------
template <typename K, bool PAIRS, int NT, int KPT>
__device__ __forceinline__ void tile_cta(K *__restrict__ keys, uint32_t *__restrict__ vals,
                                         const Offsets &off, const int32_t *__restrict__ half_first,
                                         int64_t t, K *__restrict__ tmp_keys = nullptr,
                                         uint32_t *__restrict__ tmp_vals = nullptr,
                                         int64_t radix_min = 0) {
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
  for (int c = 0; c < nc; ++c)
    sort_tile_chunk<Cfg, PAIRS>(plan_s.c[c], keys, vals, off, tmp_keys, tmp_vals, smem, hb,
                                warp_s);
}

// ---------------------------------------------------------------------------
// The kernel: CTA t sorts tile t.
// ---------------------------------------------------------------------------
template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_sort_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                 const int32_t *__restrict__ half_first, K *__restrict__ tmp_keys,
                 uint32_t *__restrict__ tmp_vals, int64_t radix_min) {
  pdl_wait();  // the classify kernel's map and jobs
  tile_cta<K, PAIRS, NT, KPT>(keys, vals, off, half_first, blockIdx.x, tmp_keys, tmp_vals,
                              radix_min);
}

}  // namespace segsort
