// Tiny segments: problems whose segments average at most kTinyMaxAvg keys.
//
// Sorting a chunk of segments of a few keys costs little next to moving it,
// so this route is built around the copies: persistent CTAs (512 threads,
// two per SM) take tiles b, b + G, ... and keep two tiles' copies in flight
// -- the keys, values and segment starts of a tile's first chunk arrive by
// bulk asynchronous copy into one of two staging buffers, issued two tiles
// ahead.  A chunk whose segments are all at most kTinyMax keys is sorted in
// the staging buffer, each segment by one thread through a sorting network
// over (order bits, slot) composites in registers, and goes back to global
// memory as 16-byte stores (not at all when no key moved: segments of one
// key, or already in order).  No sort words, no head bitmask, no scan.  A
// chunk with a longer segment (and any chunk after a tile's first) is
// appended to the bucket route's fallback list for the comparison sort
// (tile_list_kernel), CAP-runs of long segments included.
//
// The reference sorts these lengths with its smallest bb_segsort bins
// (register networks of 2..8 keys per thread group, src/bb_segsort/
// bb_comput_s.h); the result here is the stable order of each segment.
#pragma once

#include "bucket_sort.cuh"
#include "tile_stream.cuh"

namespace segsort {

constexpr int kTinyMax = 8;  // longest segment of a chunk the network sort takes

// The keys of one segment of at most kTinyMax keys as (order bits, slot)
// composites: compared as one value they give the stable order (equal keys
// by slot), and the slots past the segment hold a composite above every real
// one, so they sort last whatever the network's width.
template <typename Bits>
struct TinyWord;
template <>
struct TinyWord<uint32_t> {
  uint64_t w;  // bits << 4 | slot; the padding ~0
  __device__ __forceinline__ static TinyWord make(uint32_t bits, int q) {
    return {(static_cast<uint64_t>(bits) << 4) | static_cast<uint64_t>(q)};
  }
  __device__ __forceinline__ static TinyWord pad() { return {~0ull}; }
  __device__ __forceinline__ uint32_t bits() const { return static_cast<uint32_t>(w >> 4); }
  __device__ __forceinline__ int slot() const { return static_cast<int>(w & 15u); }
  __device__ __forceinline__ static void cx(TinyWord &a, TinyWord &b) {
    const uint64_t lo = min(a.w, b.w), hi = max(a.w, b.w);
    a.w = lo;
    b.w = hi;
  }
};
template <>
struct TinyWord<uint64_t> {
  uint64_t k;
  uint32_t q;  // slot; 15 for the padding
  __device__ __forceinline__ static TinyWord make(uint64_t bits, int q) {
    return {bits, static_cast<uint32_t>(q)};
  }
  __device__ __forceinline__ static TinyWord pad() { return {~0ull, 15u}; }
  __device__ __forceinline__ uint64_t bits() const { return k; }
  __device__ __forceinline__ int slot() const { return static_cast<int>(q); }
  __device__ __forceinline__ static void cx(TinyWord &a, TinyWord &b) {
    const bool sw = b.k < a.k || (b.k == a.k && b.q < a.q);
    const TinyWord x = sw ? b : a, y = sw ? a : b;
    a = x;
    b = y;
  }
};

// Sorts segment [0, len) of the staged keys sk (and values sv), len <= N,
// in place: composites in N registers through a sorting network of width N
// -- one comparator for 2 keys, five for 4 (Batcher), nineteen for 8
// (Batcher's odd-even merge sort; each checked on all 0-1 inputs) -- then
// every value from its key's original slot.  Returns whether any key moved.
template <int N, typename K, bool PAIRS>
__device__ __forceinline__ bool tiny_sort_segment(K *sk, uint32_t *sv, int len) {
  static_assert(N == 2 || N == 4 || N == 8, "network widths 2, 4, 8");
  using Ord = KeyOrder<K>;
  using W = TinyWord<typename Ord::Bits>;
  W w[N];
#pragma unroll
  for (int q = 0; q < N; ++q) w[q] = q < len ? W::make(Ord::to_bits(sk[q]), q) : W::pad();
  if constexpr (N == 2) {
    W::cx(w[0], w[1]);
  } else if constexpr (N == 4) {
    W::cx(w[0], w[1]); W::cx(w[2], w[3]);
    W::cx(w[0], w[2]); W::cx(w[1], w[3]);
    W::cx(w[1], w[2]);
  } else {
    W::cx(w[0], w[1]); W::cx(w[2], w[3]); W::cx(w[4], w[5]); W::cx(w[6], w[7]);
    W::cx(w[0], w[2]); W::cx(w[1], w[3]); W::cx(w[4], w[6]); W::cx(w[5], w[7]);
    W::cx(w[1], w[2]); W::cx(w[5], w[6]);
    W::cx(w[0], w[4]); W::cx(w[1], w[5]); W::cx(w[2], w[6]); W::cx(w[3], w[7]);
    W::cx(w[2], w[4]); W::cx(w[3], w[5]);
    W::cx(w[1], w[2]); W::cx(w[3], w[4]); W::cx(w[5], w[6]);
  }
  // Two keys: about half the pairs are in order already, and skip the writes.
  if (N == 2 && w[0].slot() == 0) return false;
  uint32_t v[N];
  if constexpr (PAIRS) {
#pragma unroll
    for (int q = 0; q < N; ++q)
      if (q < len) v[q] = sv[w[q].slot()];
  }
  bool moved = N == 2;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    if (q < len) {
      sk[q] = Ord::from_bits(w[q].bits());
      if constexpr (PAIRS) sv[q] = v[q];
      moved |= w[q].slot() != q;
    }
  }
  return moved;
}

// Stores staged elements [0, m) (stage[mis + i] is dst[i]; stage and dst - mis
// are 16-byte aligned, the granules a StagedSpan copied) back to dst: the
// granules that lie wholly inside [0, m) as 16-byte stores, the ragged ends
// element by element.
template <int NT, typename T>
__device__ __forceinline__ void store_staged(const T *stage, T *dst, int mis, int m) {
  constexpr int E = 16 / static_cast<int>(sizeof(T));
  const int tid = threadIdx.x;
  const int g0 = (mis + E - 1) / E, g1 = (mis + m) / E;  // whole granules [g0, g1)
  if (g1 > g0) {
    const uint4 *src = reinterpret_cast<const uint4 *>(stage);
    uint4 *out = reinterpret_cast<uint4 *>(dst - mis);
    for (int g = g0 + tid; g < g1; g += NT) out[g] = src[g];
    const int h = g0 * E - mis;  // head elements [0, h)
    const int t = g1 * E - mis;  // tail elements [t, m)
    if (tid < h) dst[tid] = stage[mis + tid];
    if (tid < m - t) dst[t + tid] = stage[mis + t + tid];
  } else {
    for (int i = tid; i < m; i += NT) dst[i] = stage[mis + i];
  }
}

// Shared memory: two staging buffers (keys, values, segment starts of a
// chunk: the granules that cover them).  For 32-bit pairs (CAP 4096) that
// is 96 KB, and two CTAs fit an SM.
template <typename K, bool PAIRS, int CAP>
struct TinyLayout {
  static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
  static constexpr int kOffsCap = CAP;  // segment starts staged per chunk
  static constexpr size_t kStageKeys = up16((CAP + 32 / sizeof(K)) * sizeof(K));
  static constexpr size_t kStageVals = PAIRS ? up16((CAP + 8) * sizeof(uint32_t)) : 0;
  static constexpr size_t kStageOffs = up16((kOffsCap + 8) * sizeof(int32_t));
  static constexpr size_t kStage = kStageKeys + kStageVals + kStageOffs;
  static constexpr size_t kBytes = 2 * kStage;
};

template <typename K, bool PAIRS, int NT, int CAP, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_tiny_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                 const int32_t *__restrict__ half_first, int64_t ntiles, bool runs,
                 int64_t radix_min, TileChunk *fallback, uint32_t *fallback_count,
                 int64_t max_fallback) {
  using TL = TinyLayout<K, PAIRS, CAP>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ TilePlan plans[kPlanRing];
  __shared__ __align__(8) uint64_t bars[2];
  const int tid = threadIdx.x;
  const int64_t t0 = blockIdx.x, G = gridDim.x;
  pdl_wait();     // the classify kernel's map and jobs
  pdl_trigger();  // the list kernel may launch under this one (it waits for it)
  if (t0 >= ntiles) return;
  const int64_t iters = (ntiles - t0 + G - 1) / G;  // tiles of this CTA: t0 + i * G
  auto stage_k = [&](int s) { return reinterpret_cast<K *>(smem + s * TL::kStage); };
  auto stage_v = [&](int s) {
    return reinterpret_cast<uint32_t *>(smem + s * TL::kStage + TL::kStageKeys);
  };
  auto stage_o = [&](int s) {
    return reinterpret_cast<int32_t *>(smem + s * TL::kStage + TL::kStageKeys + TL::kStageVals);
  };

  // Plans of iterations [i0, i0 + kPlanBatch), one per lane of warp 0.
  auto make_plans = [&](int64_t i0) {
    if (tid < 32) {
      const int64_t i = i0 + tid;
      if (tid < kPlanBatch && i < iters)
        plan_tile<CAP>(off, half_first, t0 + i * G, runs, radix_min, plans[i % kPlanRing]);
      __syncwarp();
    }
  };
  // Thread 0: the bulk copies of iteration i's first chunk into stage i & 1
  // (the barrier phase completes even when nothing is copied).
  auto issue = [&](int64_t i) {
    const int s = static_cast<int>(i & 1);
    const TilePlan &P = plans[i % kPlanRing];
    uint64_t *bar = &bars[s];
    if (P.nc == 0) {
      mbar_arrive_expect_tx(bar, 0);
      return;
    }
    const TileChunk &C = P.c[0];
    const StagedSpan<K> rk(keys + C.a, C.m);
    const StagedSpan<uint32_t> rv(PAIRS ? vals + C.a : nullptr, PAIRS ? C.m : 0);
    const int cnt = C.hi - C.lo;
    const bool offs = cnt > 1 && cnt <= TL::kOffsCap;
    const StagedSpan<int32_t> ro(off.p + C.lo, offs ? cnt : 0);
    uint32_t bytes = rk.bytes();
    if (PAIRS) bytes += rv.bytes();
    if (offs) bytes += ro.bytes();
    mbar_arrive_expect_tx(bar, bytes);
    rk.issue(stage_k(s), keys + C.a, bar);
    if (PAIRS) rv.issue(stage_v(s), vals + C.a, bar);
    if (offs) ro.issue(stage_o(s), off.p + C.lo, bar);
  };
  auto list = [&](const TileChunk &C) {
    const uint32_t at = atomicAdd(fallback_count, 1u);
    if (at < max_fallback) fallback[at] = C;
  };

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  make_plans(0);
  if (tid == 0) {
    issue(0);
    if (iters > 1) issue(1);
  }
  __syncthreads();

  for (int64_t i = 0; i < iters; ++i) {
    const int s = static_cast<int>(i & 1);
    const bool ok = mbar_wait(&bars[s], static_cast<uint32_t>((i >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      // A copy of this stage did not complete in time: wait once more
      // (bounded) for the copies this CTA has in flight -- this stage's and
      // the next one's -- so that none can land after the CTA has returned.
      if (tid == 0) {
        raise_status(kStatusTimeout);
        mbar_wait(&bars[s], static_cast<uint32_t>((i >> 1) & 1));
        if (i + 1 < iters) mbar_wait(&bars[s ^ 1], static_cast<uint32_t>(((i + 1) >> 1) & 1));
      }
      __syncthreads();
      return;
    }
    const TilePlan &P = plans[i % kPlanRing];
    const int nc = P.nc;
    if (nc > 0) {
      const TileChunk C = P.c[0];
      const int m = C.m, cnt = C.hi - C.lo;
      const int64_t a = C.a;
      // Tiny: one segment, or staged starts.  Every thread sorts whole
      // segments in the staging buffer; a segment longer than kTinyMax keys
      // sends the chunk to the list (its keys in global memory are still
      // untouched), otherwise the chunk goes back to global memory, unless
      // no key moved.  A CAP-run of a long segment (cnt == 0) is listed.
      const bool staged_offs = cnt > 1 && cnt <= TL::kOffsCap;
      if (cnt == 1 || staged_offs) {
        const int mis_k = StagedSpan<K>(keys + a, m).mis;
        const int mis_v = PAIRS ? StagedSpan<uint32_t>(vals + a, m).mis : 0;
        K *sk = stage_k(s) + mis_k;
        uint32_t *sv = PAIRS ? stage_v(s) + mis_v : nullptr;
        const int32_t *so =
            stage_o(s) + (staged_offs ? StagedSpan<int32_t>(off.p + C.lo, cnt).mis : 0);
        auto local = [&](int32_t v) {
          const int64_t x = clamp_offset(v, off.n) - a;
          return static_cast<int>(x < 0 ? 0 : (x > m ? m : x));
        };
        bool too_long = false, moved = false;
        for (int j = tid; j < cnt; j += NT) {
          const int b0 = cnt > 1 ? local(so[j]) : 0;
          const int e0 = j + 1 < cnt ? local(so[j + 1]) : m;
          const int len = e0 - b0;
          if (len > kTinyMax) {
            too_long = true;
          } else if (len > 4) {
            moved |= tiny_sort_segment<8, K, PAIRS>(sk + b0, PAIRS ? sv + b0 : nullptr, len);
          } else if (len > 2) {
            moved |= tiny_sort_segment<4, K, PAIRS>(sk + b0, PAIRS ? sv + b0 : nullptr, len);
          } else if (len == 2) {
            moved |= tiny_sort_segment<2, K, PAIRS>(sk + b0, PAIRS ? sv + b0 : nullptr, 2);
          }
        }
        if (__syncthreads_or(too_long)) {
          if (tid == 0) list(C);
        } else if (__syncthreads_or(moved)) {
          store_staged<NT>(stage_k(s), keys + a, mis_k, m);
          if constexpr (PAIRS) store_staged<NT>(stage_v(s), vals + a, mis_v, m);
        }
      } else if (tid == 0) {
        list(C);
      }
      if (tid == 0)
        for (int c = 1; c < nc; ++c) list(P.c[c]);
    }
    __syncthreads();  // stage s is free again
    if (i + 2 < iters) {
      // Plans are made a batch at a time, each batch just before its first
      // copies; the ring holds it beside the two plans still in use.
      if ((i + 2) % kPlanBatch == 0) make_plans(i + 2);
      if (tid == 0) {
        fence_proxy_async();
        issue(i + 2);
      }
    }
  }
}

}  // namespace segsort
