// Tile sort: every segment of at most CAP = NT * KPT elements is sorted by
// one CTA, entirely in shared memory and registers (one HBM read and one HBM
// write per element).
//
// Work split.  CTA t owns the segments whose first element lies in the
// nominal range [t*CAP, (t+1)*CAP).  It walks them in order and packs
// consecutive segments into chunks of at most CAP elements (a binary search
// over the offsets finds each chunk's last segment), so a chunk is a
// contiguous element range made of whole segments.  Segments longer than CAP
// are skipped here; the large-segment path sorts them.
//
// Chunk sort.  Every element becomes a composite word
//     (segment start within the chunk, order bits of the key, chunk index)
// compared as one unsigned integer.  Words are unique, so any sorting method
// gives the stable per-segment order the reference's oracle produces with
// std::stable_sort (src/bb_segsort/main.cu:152-173), and segments never mix
// because the segment start is the most significant field.  The sort is a
// merge sort: each thread sorts KPT words in registers with a bitonic network,
// then log2(chunk / KPT) merge-path levels merge pairs of runs through
// shared memory.  A pair whose runs are already in order (last word of the
// first run <= first word of the second) is left as it is, so chunks of short
// aligned segments skip the upper levels.  Values are staged once in shared
// memory and gathered through the index field at the end.
//
// The reference sorts these lengths with one kernel per power-of-two length
// bin (src/bb_segsort/bb_segsort.h:71-164, bins from bb_bin.h:54-100) using
// unstable register networks; this kernel replaces that whole family and its
// host round trip for the bin counts (bb_bin.h:46).
#pragma once

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
  static constexpr size_t kWordBytes = static_cast<size_t>(WSLOTS) * sizeof(Word);
  static constexpr size_t kOutBytes =
      static_cast<size_t>(OSLOTS) * (sizeof(K) + (PAIRS ? sizeof(uint32_t) : 0));
  static constexpr size_t kMainBytes =
      ((kWordBytes > kOutBytes ? kWordBytes : kOutBytes) + 15) / 16 * 16;
  static constexpr size_t kSmemBytes = kMainBytes + (PAIRS ? CAP * sizeof(uint32_t) : 0);

  static __device__ __forceinline__ int wslot(int i) { return i + i / WUNIT; }
  static __device__ __forceinline__ int oslot(int i) { return i + (i >> 5); }
};

// Bitonic sorting network over KPT words held in registers (ascending).
template <typename WT, int KPT>
__device__ __forceinline__ void thread_sort(typename WT::T (&w)[KPT]) {
#pragma unroll
  for (int k = 2; k <= KPT; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int i = 0; i < KPT; ++i) {
        const int l = i ^ j;
        if (l > i) {
          typename WT::T x = w[i], y = w[l];
          const bool up = (i & k) == 0;
          const bool swap = up ? WT::lt(y, x) : WT::lt(x, y);
          w[i] = swap ? y : x;
          w[l] = swap ? x : y;
        }
      }
    }
  }
}

template <typename K, bool PAIRS, int NT, int KPT>
__global__ void __launch_bounds__(NT)
tile_sort_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off) {
  using Cfg = TileConfig<K, PAIRS, NT, KPT>;
  using Ord = typename Cfg::Ord;
  using WT = typename Cfg::WT;
  using Word = typename Cfg::Word;
  constexpr int CAP = Cfg::CAP;

  extern __shared__ __align__(16) unsigned char smem[];
  Word *W = reinterpret_cast<Word *>(smem);
  K *KO = reinterpret_cast<K *>(smem);
  uint32_t *VO = reinterpret_cast<uint32_t *>(smem + Cfg::OSLOTS * sizeof(K));
  uint32_t *Vs = reinterpret_cast<uint32_t *>(smem + Cfg::kMainBytes);
  __shared__ int64_t ctl[4];

  const int tid = threadIdx.x;
  const int64_t n = off.n;
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * CAP;
  if (t0 >= n) return;

  // Segments whose first element is in [t0, t0 + CAP): [s_cur, s_end).
  int64_t s_cur = 0, s_end = 0;
  if (tid == 0) {
    s_cur = first_offset_ge(off, t0);
    s_end = first_offset_ge(off, t0 + CAP);
  }

  while (true) {
    if (tid == 0) {
      int64_t a = 0, b = 0, lo = 0, hi = 0;
      while (s_cur < s_end) {
        a = off(s_cur);
        const int64_t j = last_offset_le(off, s_cur, s_end, a + CAP);
        if (j == s_cur) {  // longer than CAP: left to the large-segment path
          ++s_cur;
          continue;
        }
        lo = s_cur;
        hi = j;
        b = off(j);
        s_cur = j;
        break;
      }
      ctl[0] = a;
      ctl[1] = b;
      ctl[2] = lo;
      ctl[3] = hi;
    }
    __syncthreads();
    const int64_t a = ctl[0];
    const int64_t seg_lo = ctl[2], seg_hi = ctl[3];
    const int m = static_cast<int>(ctl[1] - a);
    __syncthreads();
    if (seg_hi == seg_lo) break;  // no more chunks
    if (m <= 0) continue;          // only empty segments
    const bool multi = (seg_hi - seg_lo) > 1;

    // ---- load: keys -> words (coalesced), values -> Vs -------------------
    for (int i = tid; i < m; i += NT) {
      W[Cfg::wslot(i)] = WT::make(Ord::to_bits(keys[a + i]), static_cast<uint32_t>(i));
      if constexpr (PAIRS) Vs[i] = vals[a + i];
    }
    __syncthreads();

    // ---- blocked words + segment field --------------------------------------
    Word w[KPT];
    const int base = tid * KPT;
    int64_t next_begin = INT64_MAX, seg_begin = a;
    if (multi && base < m) {
      int64_t s = last_offset_le(off, seg_lo, seg_hi - 1, a + base);
      seg_begin = off(s);
      next_begin = off(s + 1);
      // Walk forward past empty segments lazily inside the loop below.
      int64_t s_walk = s;
#pragma unroll
      for (int j = 0; j < KPT; ++j) {
        const int i = base + j;
        if (i < m) {
          while (a + i >= next_begin && s_walk + 1 < seg_hi) {
            ++s_walk;
            seg_begin = next_begin;
            next_begin = off(s_walk + 1);
          }
          w[j] = WT::with_seg(W[Cfg::wslot(i)], static_cast<uint32_t>(seg_begin - a));
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

    thread_sort<WT, KPT>(w);

    // ---- merge levels -------------------------------------------------------
    for (int run = KPT; run < m; run <<= 1) {
      __syncthreads();  // previous readers of W are done
#pragma unroll
      for (int j = 0; j < KPT; ++j) W[Cfg::wslot(base + j)] = w[j];
      __syncthreads();
      const int pair_threads = (2 * run) / KPT;
      const int r = tid & (pair_threads - 1);
      const int a_beg = (tid - r) * KPT;
      const int a_end = a_beg + run;
      const int b_end = a_end + run;
      // Runs already in order: the merge is the concatenation, which is what
      // this thread holds.
      if (WT::le(W[Cfg::wslot(a_end - 1)], W[Cfg::wslot(a_end)])) continue;
      const int diag = r * KPT;
      int lo = diag > run ? diag - run : 0;
      int hi = diag < run ? diag : run;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const Word x = W[Cfg::wslot(a_beg + mid)];
        const Word y = W[Cfg::wslot(a_end + diag - 1 - mid)];
        if (WT::le(x, y)) lo = mid + 1; else hi = mid;
      }
      int ai = a_beg + lo;
      int bi = a_end + diag - lo;
      Word av = ai < a_end ? W[Cfg::wslot(ai)] : WT::maxv();
      Word bv = bi < b_end ? W[Cfg::wslot(bi)] : WT::maxv();
#pragma unroll
      for (int j = 0; j < KPT; ++j) {
        const bool take_a = WT::le(av, bv);
        w[j] = take_a ? av : bv;
        ai += take_a;
        bi += !take_a;
        const int nx = take_a ? ai : bi;
        const int lim = take_a ? a_end : b_end;
        const Word nv = nx < lim ? W[Cfg::wslot(nx)] : WT::maxv();
        av = take_a ? nv : av;
        bv = take_a ? bv : nv;
      }
    }
    __syncthreads();

    // ---- output: stage in shared memory, then coalesced stores -------------
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const int i = base + j;
      if (i < m) {
        KO[Cfg::oslot(i)] = Ord::from_bits(WT::bits(w[j]));
        if constexpr (PAIRS) VO[Cfg::oslot(i)] = Vs[WT::index(w[j])];
      }
    }
    __syncthreads();
    for (int i = tid; i < m; i += NT) {
      keys[a + i] = KO[Cfg::oslot(i)];
      if constexpr (PAIRS) vals[a + i] = VO[Cfg::oslot(i)];
    }
    __syncthreads();
  }
}

}  // namespace segsort
