// Streamed tile sort: the tile sort of a problem of more than one tile, run
// by persistent CTAs that fetch the next tile's data into shared memory while
// they sort the current one.
//
// The per-tile work is the tile sort's (tile_sort.cuh): the same chunk plan,
// the same composite words and merge levels, the same writes.  What changes
// is how a tile's first chunk reaches shared memory.  A CTA of the plain
// kernel loads, sorts and stores one tile in turn, with two CTAs per SM (128
// registers a thread); while it waits for its loads the SM has little else
// to run, which leaves short-segment problems at a fraction of HBM
// bandwidth.  Here CTA b sorts tiles b, b + G, b + 2G, ... (G = grid size),
// and as soon as tile t's first chunk has left the staging buffers, one
// thread issues bulk asynchronous copies (cp.async.bulk, completing on an
// mbarrier) of tile t + G's first chunk -- keys, values and, for a chunk of
// several segments, its segment starts -- so that the copy runs under the
// sort of tile t.  Each array is copied as the 16-byte granules that cover
// its range, so the conversion into sort words reads shared memory only.  A
// tile's further chunks (long-segment runs beside short segments) are loaded
// directly, as in the plain kernel.
//
// Chunk plans (plan_tile) are computed 16 tiles at a time by lanes of warp 0
// into a ring of 32, one batch ahead of the copies that need them.
// Every wait on the mbarrier is bounded; a wait that gives up raises
// kStatusTimeout, waits once more (bounded) for the copies of that stage --
// the only ones the CTA has in flight -- and the CTA returns.
#pragma once

#include "tile_sort.cuh"

namespace segsort {

constexpr int kStageSpinLimit = 1 << 22;  // ~0.3 s with the back-off below

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy wrappers (PTX ISA: mbarrier, cp.async.bulk).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Makes the initialised barrier visible to the async proxy and other threads.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this CTA's earlier shared-memory accesses (made visible to the
// calling thread by a barrier) before its later bulk copies.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the completion of the barrier phase with the given parity;
// false when it did not complete within the spin limit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          int spin_limit = kStageSpinLimit) {
  for (int it = 0; it < spin_limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it >= 8) __nanosleep(64);
  }
  return false;
}

// Global -> shared bulk copy of `bytes` (a multiple of 16; both addresses
// 16-byte aligned), completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  uint64_t g;
  asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(g), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// Staging geometry of m >= 1 elements at src: the nvec 16-byte granules that
// cover them are copied in bulk, from the granule boundary mis elements
// below src, so that element i lands at stage[mis + i].  The granules lie
// within the array's own 16-byte-aligned extent (each holds an element of
// the range); elements of a granule outside the range are never used.
// ---------------------------------------------------------------------------
template <typename T>
struct StagedSpan {
  static constexpr int V = 16 / static_cast<int>(sizeof(T));
  int mis, nvec;
  __device__ __forceinline__ StagedSpan(const T *src, int m) {
    mis = static_cast<int>((reinterpret_cast<uintptr_t>(src) & 15) / sizeof(T));
    nvec = m > 0 ? (mis + m + V - 1) / V : 0;
  }
  __device__ __forceinline__ uint32_t bytes() const { return static_cast<uint32_t>(nvec) * 16u; }
  __device__ __forceinline__ void issue(T *stage, const T *src, uint64_t *bar) const {
    if (nvec > 0) bulk_g2s(stage, src - mis, bytes(), bar);
  }
};

// Feeds f(i, element) for i in [0, m) from the staged granules.
template <int NT, typename T, typename F>
__device__ __forceinline__ void read_staged(const T *stage, const T *src, int m, F &&f) {
  constexpr int V = StagedSpan<T>::V;
  const StagedSpan<T> r(src, m);
  const uint4 *sv = reinterpret_cast<const uint4 *>(stage);
  for (int k = threadIdx.x; k < r.nvec; k += NT) {
    const uint4 v = sv[k];
    T e[V];
    memcpy(e, &v, 16);
#pragma unroll
    for (int c = 0; c < V; ++c) {
      const int i = k * V + c - r.mis;
      if (i >= 0 && i < m) f(i, e[c]);
    }
  }
}

// ---------------------------------------------------------------------------
// Shared-memory layout: the tile sort's region, then the staging buffers.
// ---------------------------------------------------------------------------
template <typename Cfg, typename K, bool PAIRS>
struct StreamLayout {
  static constexpr size_t up16(size_t x) { return (x + 15) / 16 * 16; }
  static constexpr int kOffsCap = Cfg::CAP / 2;  // segment starts staged per chunk
  static constexpr size_t kKeys = up16(Cfg::kSmemBytes);
  static constexpr size_t kVals = kKeys + up16((Cfg::CAP + 32 / sizeof(K)) * sizeof(K));
  static constexpr size_t kOffs = kVals + (PAIRS ? up16((Cfg::CAP + 8) * sizeof(uint32_t)) : 0);
  static constexpr size_t kBytes = kOffs + up16((kOffsCap + 8) * sizeof(int32_t));
};

// Plans computed at a time (by lanes of warp 0) and held (the batch in use
// and the next).  Two CTAs of the 32-bit pair sort then take 196 KB of shared
// memory, which leaves the SM 60 KB of L1 for the sort's register spills.
constexpr int kPlanBatch = 16;
constexpr int kPlanRing = 32;

// Clamps a raw offset into [0, n] as Offsets does.
__device__ __forceinline__ int64_t clamp_offset(int32_t v, int64_t n) {
  const int64_t x = v < 0 ? 0 : static_cast<int64_t>(v);
  return x > n ? n : x;
}

// ---------------------------------------------------------------------------
// The kernel: a problem of ntiles > 1 tiles with its half-tile map; the
// grid is at most ntiles CTAs.
// ---------------------------------------------------------------------------
template <typename K, bool PAIRS, int NT, int KPT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
tile_stream_kernel(K *__restrict__ keys, uint32_t *__restrict__ vals, Offsets off,
                   const int32_t *__restrict__ half_first, K *__restrict__ tmp_keys,
                   uint32_t *__restrict__ tmp_vals, int64_t ntiles, int64_t radix_min) {
  using Cfg = TileConfig<K, PAIRS, NT, KPT>;
  using SL = StreamLayout<Cfg, K, PAIRS>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ TilePlan plans[kPlanRing];
  __shared__ uint32_t hb[Cfg::CAP / 32];
  __shared__ int warp_s[NT / 16];
  __shared__ __align__(8) uint64_t bar;
  K *SK = reinterpret_cast<K *>(smem + SL::kKeys);
  uint32_t *SV = reinterpret_cast<uint32_t *>(smem + SL::kVals);
  int32_t *SO = reinterpret_cast<int32_t *>(smem + SL::kOffs);

  const int tid = threadIdx.x;
  const int64_t t0 = blockIdx.x, G = gridDim.x;
  pdl_wait();  // the classify kernel's map and jobs
  if (t0 >= ntiles) return;
  const int64_t iters = (ntiles - t0 + G - 1) / G;  // tiles of this CTA: t0 + i * G
  const bool runs = tmp_keys != nullptr;

  // Plans of iterations [i0, i0 + kPlanBatch), one per lane of warp 0.
  auto make_plans = [&](int64_t i0) {
    if (tid < 32) {
      const int64_t i = i0 + tid;
      if (tid < kPlanBatch && i < iters)
        plan_tile<Cfg::CAP>(off, half_first, t0 + i * G, runs, radix_min, plans[i % kPlanRing]);
      __syncwarp();
    }
  };
  // Thread 0: bulk copies of iteration i's first chunk.  The barrier phase
  // completes even when nothing is copied.
  auto issue = [&](int64_t i) {
    const TilePlan &P = plans[i % kPlanRing];
    if (P.nc == 0) {
      mbar_arrive_expect_tx(&bar, 0);
      return;
    }
    const TileChunk &C = P.c[0];
    const StagedSpan<K> rk(keys + C.a, C.m);
    const StagedSpan<uint32_t> rv(PAIRS ? vals + C.a : nullptr, PAIRS ? C.m : 0);
    const int cnt = C.hi - C.lo;
    const bool offs = cnt > 1 && cnt <= SL::kOffsCap;
    const StagedSpan<int32_t> ro(off.p + C.lo, offs ? cnt : 0);
    uint32_t bytes = rk.bytes();
    if (PAIRS) bytes += rv.bytes();
    if (offs) bytes += ro.bytes();
    mbar_arrive_expect_tx(&bar, bytes);
    rk.issue(SK, keys + C.a, &bar);
    if (PAIRS) rv.issue(SV, vals + C.a, &bar);
    if (offs) ro.issue(SO, off.p + C.lo, &bar);
  };

  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  make_plans(0);
  __syncthreads();
  if (tid == 0) issue(0);

  for (int64_t i = 0; i < iters; ++i) {
    const TilePlan &P = plans[i % kPlanRing];
    const int nc = P.nc;
    TileChunk C0{};
    if (nc > 0) C0 = P.c[0];
    const int m = C0.m;
    const bool multi = nc > 0 && C0.hi - C0.lo > 1;
    if (nc > 0) clear_heads<NT>(hb, m, multi);
    const bool ok = mbar_wait(&bar, static_cast<uint32_t>(i & 1));
    if (__syncthreads_or(!ok)) {
      // The copies of this stage are the only ones the CTA has issued and not
      // seen complete (the next stage is issued only after this wait).  A
      // timeout means their bytes have not all arrived; wait for them once
      // more, bounded, so that the CTA does not end while a copy may still
      // write its shared memory, then give up on the rest of the tiles.
      if (tid == 0) {
        raise_status(kStatusTimeout);
        mbar_wait(&bar, static_cast<uint32_t>(i & 1));
      }
      __syncthreads();
      return;
    }
    // ---- staged chunk -> words, values, segment heads -----------------------
    if (nc > 0) {
      const ChunkSinks<Cfg, K> S{smem, hb, m};
      read_staged<NT>(SK, keys + C0.a, m, [&](int j, K k) { S.key(j, k); });
      if constexpr (PAIRS)
        read_staged<NT>(SV, vals + C0.a, m, [&](int j, uint32_t v) { S.val(j, v); });
      if (multi) {
        const int cnt = C0.hi - C0.lo;
        if (cnt <= SL::kOffsCap) {
          read_staged<NT>(SO, off.p + C0.lo, cnt,
                          [&](int, int32_t v) { S.head(clamp_offset(v, off.n) - C0.a); });
        } else {
          for (int64_t j = C0.lo + tid; j < C0.hi; j += NT) S.head(off(j) - C0.a);
        }
      }
    }
    __syncthreads();  // staging buffers consumed; W, Vs and hb hold the chunk
    // ---- next tile's copies, under this tile's sort ---------------------------
    if (i + 1 < iters) {
      if ((i + 1) % kPlanBatch == 0) {
        make_plans(i + 1);
        __syncthreads();  // the batch is read by every warp from the next iteration on
      }
      if (tid == 0) {
        fence_proxy_async();
        issue(i + 1);
      }
    }
    if (nc > 0) {
      const ChunkIO<K, PAIRS> io(C0, keys, vals, tmp_keys, tmp_vals);
      sort_loaded<Cfg, PAIRS, K, true>([=] { return io; }, m, multi, smem, hb, warp_s);
      for (int c = 1; c < nc; ++c)
        sort_tile_chunk<Cfg, PAIRS, true>(P.c[c], keys, vals, off, tmp_keys, tmp_vals, smem, hb,
                                          warp_s);
    }
  }
}

}  // namespace segsort
