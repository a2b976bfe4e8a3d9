// Tiny segments: problems whose segments average at most kTinyMaxAvg keys.
//
// Sorting a chunk of segments of a few keys costs little next to moving it,
// so this route is built around the copies: persistent CTAs (512 threads,
// two per SM) take tiles b, b + G, ... and keep two tiles' copies in flight
// -- the keys, values and segment starts of a tile's first chunk arrive by
// bulk asynchronous copy into one of two staging buffers, issued two tiles
// ahead -- and sort a chunk whose segments are all at most kTinyMax keys by
// ranking in place: every key of segment [s, t) counts the keys of [s, t)
// below it, and the keys equal to it and before it, which is its place in
// the stable order, and is written there.  No sort words, no head bitmask,
// no scan.  A chunk with a longer segment (and any chunk after a tile's
// first) is appended to the bucket route's fallback list for the comparison
// sort (tile_list_kernel), CAP-runs of long segments included.
//
// The reference sorts these lengths with its smallest bb_segsort bins
// (register networks of 2..8 keys per thread group, src/bb_segsort/
// bb_comput_s.h); the result here is the stable order of each segment.
#pragma once

#include "bucket_sort.cuh"
#include "tile_stream.cuh"

namespace segsort {

constexpr int kTinyMax = 8;  // longest segment of a chunk the rank sort takes

// Shared memory: two staging buffers (keys, values, segment starts of a
// chunk: the granules that cover them), then the segment of every position
// of the chunk being ranked, as its start | length << 12 in 16 bits.  For
// 32-bit pairs (CAP 4096) that is 104 KB, and two CTAs fit an SM.
template <typename K, bool PAIRS, int CAP>
struct TinyLayout {
  static_assert(CAP <= 4096, "segment starts are packed in 12 bits");
  static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
  static constexpr int kOffsCap = CAP;  // segment starts staged per chunk
  static constexpr size_t kStageKeys = up16((CAP + 32 / sizeof(K)) * sizeof(K));
  static constexpr size_t kStageVals = PAIRS ? up16((CAP + 8) * sizeof(uint32_t)) : 0;
  static constexpr size_t kStageOffs = up16((kOffsCap + 8) * sizeof(int32_t));
  static constexpr size_t kStage = kStageKeys + kStageVals + kStageOffs;
  static constexpr size_t kBounds = 2 * kStage;  // uint16[CAP]
  static constexpr size_t kBytes = kBounds + CAP * sizeof(uint16_t);
};

template <typename K, bool PAIRS, int NT, int CAP, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_tiny_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                 const int32_t *__restrict__ half_first, int64_t ntiles, bool runs,
                 int64_t radix_min, TileChunk *fallback, uint32_t *fallback_count,
                 int64_t max_fallback) {
  using TL = TinyLayout<K, PAIRS, CAP>;
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ TilePlan plans[kPlanRing];
  __shared__ __align__(8) uint64_t bars[2];
  const int tid = threadIdx.x;
  const int64_t t0 = blockIdx.x, G = gridDim.x;
  if (t0 >= ntiles) return;
  const int64_t iters = (ntiles - t0 + G - 1) / G;  // tiles of this CTA: t0 + i * G
  uint16_t *bd = reinterpret_cast<uint16_t *>(smem + TL::kBounds);
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
      // Tiny: one segment of at most kTinyMax keys, or staged starts whose
      // segments are all that short (uniform over the CTA).  A CAP-run of a
      // long segment (cnt == 0) never is.
      bool tiny = false;
      int mis_o = 0;
      if (cnt == 1) {
        tiny = m <= kTinyMax;
      } else if (cnt > 1 && cnt <= TL::kOffsCap) {
        mis_o = StagedSpan<int32_t>(off.p + C.lo, cnt).mis;
        const int32_t *so = stage_o(s) + mis_o;
        bool too_long = false;
        for (int j = tid; j < cnt; j += NT) {
          const int64_t b0 = clamp_offset(so[j], off.n);
          const int64_t e0 = j + 1 < cnt ? clamp_offset(so[j + 1], off.n) : a + m;
          too_long |= e0 - b0 > kTinyMax;
        }
        tiny = !__syncthreads_or(too_long);
      }
      if (tiny) {
        // Bounds of every position, then every key to its place.
        auto local = [&](int64_t v) {
          const int64_t x = v - a;
          return static_cast<int>(x < 0 ? 0 : (x > m ? m : x));
        };
        if (cnt == 1) {
          for (int x = tid; x < m; x += NT) bd[x] = static_cast<uint16_t>(m << 12);
        } else {
          const int32_t *so = stage_o(s) + mis_o;
          for (int j = tid; j < cnt; j += NT) {
            const int b0 = local(clamp_offset(so[j], off.n));
            const int e0 = j + 1 < cnt ? local(clamp_offset(so[j + 1], off.n)) : m;
            const int len = min(e0 - b0, kTinyMax);
            const uint16_t packed = static_cast<uint16_t>(b0 | (len << 12));
            for (int x = b0; x < b0 + len; ++x) bd[x] = packed;
          }
        }
        __syncthreads();
        const K *sk = stage_k(s) + StagedSpan<K>(keys + a, m).mis;
        const uint32_t *sv =
            PAIRS ? stage_v(s) + StagedSpan<uint32_t>(vals + a, m).mis : nullptr;
        for (int e = tid; e < m; e += NT) {
          const uint32_t u = bd[e];
          const int b0 = min(static_cast<int>(u & 0xFFFu), m);
          const int e0 = min(b0 + static_cast<int>(u >> 12), m);
          const K key = sk[e];
          const Bits kb = Ord::to_bits(key);
          int r = 0;
          for (int x = b0; x < e0; ++x) {
            const Bits b = Ord::to_bits(sk[x]);
            r += (b < kb) | ((b == kb) & (x < e));
          }
          const int p = b0 + r;
          // A warp whose keys all stay where they are writes nothing (every
          // segment of length 1, or already in order).
          if (__any_sync(__activemask(), p != e) && p < m) {  // p < m: always, with
            keys[a + p] = key;                                // well-formed offsets
            if constexpr (PAIRS) vals[a + p] = sv[e];
          }
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
