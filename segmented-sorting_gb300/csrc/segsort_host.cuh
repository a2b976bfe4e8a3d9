// Host-side pieces shared by the library's translation units: kernel shapes,
// the workspace layout, per-device state with the stream-ordered pool, and
// launch helpers.  Mutable state is `inline` so that every unit of the
// library sees one copy.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <shared_mutex>
#include <unordered_map>
#include <utility>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_common.cuh"
#include "tile_sort.cuh"
#include "bucket_sort.cuh"
#include "tile_stream.cuh"
#include "tiny_sort.cuh"
#include "classify.cuh"
#include "merge_sort.cuh"
#include "radix_sort.cuh"
#include "msd_route.cuh"

namespace segsort {

constexpr int kMaxDevices = 64;

// ---------------------------------------------------------------------------
// Tile-sort shape per key width: 4096-element chunks for 32-bit keys (256
// threads x 16 words), 2048 for 64-bit keys (256 threads x 8 words).
// Build-time tuning knobs (defaults are the measured best on GB300).
#ifndef SEGSORT_TILE_NT32
#define SEGSORT_TILE_NT32 256
#endif
#ifndef SEGSORT_TILE_KPT32
#define SEGSORT_TILE_KPT32 16
#endif
#ifndef SEGSORT_TILE_MINB
#define SEGSORT_TILE_MINB 2
#endif
template <typename K, bool PAIRS>
struct TileFor {
  using Cfg = TileConfig<K, PAIRS, sizeof(K) == 4 ? SEGSORT_TILE_NT32 : 256,
                         sizeof(K) == 4 ? SEGSORT_TILE_KPT32 : 8>;
  static constexpr int kMinBlocks = SEGSORT_TILE_MINB;  // resident CTAs per SM the registers must allow
};

// Launch shape of the bucket-route tile kernel (tile_bucket_kernel): the
// same tile capacity, 512 threads.  At 64 registers two CTAs fill an SM with
// 32 warps; measured on GB300 (2^24 u32 pairs, 2^12-key segments) 0.16 ms
// against 0.19 ms for 256 threads at 128 registers.
template <typename K, bool PAIRS>
struct BucketFor {
  static constexpr int kNT = 512;
  using Cfg = TileConfig<K, PAIRS, kNT, TileFor<K, PAIRS>::Cfg::CAP / kNT>;
  static constexpr int kMinBlocks = 2;
};

template <typename K>
constexpr int64_t tile_cap() {
  return TileFor<K, false>::Cfg::CAP;
}

// ---------------------------------------------------------------------------
// Radix threshold: segments longer than this take the LSD radix passes,
// shorter long segments the merge passes.  Never below the radix tile (so a
// radix job spans at least two tiles and the job count stays within the
// layout's bound) nor the tile capacity.  Run-time parameter
// (segsort_set_param).  Defaults measured on GB300 over 2^24 uint32 pairs in
// equal segments: the LSD radix route takes about 0.62 ms whatever the
// length, the MSD route (msd_route.cuh) 0.52-0.60 ms from 2^17 up, the merge
// route over bucket-sorted runs 0.27 ms at 2^13, 0.49 ms at 2^16, 0.58 ms
// at 2^17 and 0.66 ms at 2^18.  64-bit keys need twice the radix passes.
constexpr int64_t kRadixTile = static_cast<int64_t>(kRBuckets) * kRItems;
constexpr int64_t kRadixMinFloor = kRadixTile;
inline std::atomic<int64_t> g_radix_min32{int64_t{1} << 16};
inline std::atomic<int64_t> g_radix_min64{int64_t{1} << 18};

template <typename K>
inline int64_t clamp_radix_min(int64_t v) {
  return std::max<int64_t>(std::max<int64_t>(v, kRadixMinFloor), tile_cap<K>());
}

template <typename K>
inline int64_t radix_min_for() {
  return clamp_radix_min<K>(
      (sizeof(K) == 8 ? g_radix_min64 : g_radix_min32).load(std::memory_order_relaxed));
}

// Segments longer than this try the MSD route (in calls that take it) even
// below the radix threshold; one that does not qualify and is not longer
// than the radix threshold goes back to the merge passes.  Measured on GB300
// (2^24 pairs, 64-bit keys whose top varying digit splits them finely): the
// MSD route 0.77 / 0.73 / 0.82 ms at 2^15 / 2^16 / 2^17 against the merge
// route's 0.88 / 1.05 / 1.21 ms; for 32-bit keys it meets the merge route at
// 2^16, the radix threshold.
template <typename K>
inline int64_t msd_min_for(int64_t radix_min) {
  const int64_t m = sizeof(K) == 8 ? (int64_t{1} << 15) : (int64_t{1} << 16);
  return clamp_radix_min<K>(std::min(radix_min, m));
}

// Problems whose average segment is at most this long take the half-tile
// classify and the streamed tile kernel (measured on GB300 over 2^24 pairs:
// both faster up to 32, slower from 64).  Run-time parameter
// (segsort_set_param); a huge value sends every multi-tile problem through
// them.
inline std::atomic<int64_t> g_stream_max_avg{32};

// Problems (not streamed) whose average segment is at least this long take
// the bucket route of the tile sort (tile_bucket_kernel, then
// tile_list_kernel for the chunks it refuses); 0: never.  Below 128 keys per
// segment the comparison sort is faster (measured on GB300, 2^24 u32 pairs:
// 0.20 against 0.25 ms at 64, even at 128).  Run-time parameter.
inline std::atomic<int64_t> g_bucket_min_avg{128};

// Problems whose average segment is longer than the radix threshold take
// the MSD route for their radix segments (msd_route.cuh) when this is set
// and the library owns the workspace.  Run-time parameter.
inline std::atomic<int64_t> g_msd_on{1};

// Problems whose average segment is at most this long take the tiny route
// (tile_tiny_kernel, then tile_list_kernel for the chunks it lists); 0:
// never.  Run-time parameter.
inline std::atomic<int64_t> g_tiny_max_avg{8};

// Launch shape of the tiny route: 512 threads, two CTAs per SM (two staging
// buffers of a tile each).
constexpr int kTinyThreads = 512;

// ---------------------------------------------------------------------------
// Route of one plain call: the radix threshold, the streamed-tile threshold,
// the resident CTAs per SM of the long-segment kernel (0: as many as fit),
// the bucket-route threshold and the MSD route switch.  From the process-wide
// parameters, unless the tuner recorded a route for the call's class
// (segsort_tune_pairs_u32 / segsort_tune_load).
struct CallRoute {
  int64_t radix_min;
  int64_t stream_max_avg;
  int32_t merge_per_sm;
  int64_t bucket_min_avg = 128;  // bucket route from this average segment on (0: never)
  int32_t msd = 1;               // MSD route for calls whose segments average above radix_min
};

// Class of a plain call: key width, log2 of n, log2 of the average segment.
inline uint32_t route_class(int key_bytes, int64_t n, int32_t nseg) {
  auto lg = [](int64_t x) {
    int l = 0;
    while (x > 1) {
      x >>= 1;
      ++l;
    }
    return static_cast<uint32_t>(l);
  };
  const int64_t avg = nseg > 0 ? std::max<int64_t>(1, n / nseg) : 1;
  return (static_cast<uint32_t>(key_bytes) << 16) | (lg(n) << 8) | lg(avg);
}

struct TunedRoutes {
  std::shared_mutex mu;
  std::unordered_map<uint32_t, CallRoute> by_class;
  std::atomic<bool> any{false};
};
inline TunedRoutes g_tuned;

inline bool tuned_route(uint32_t cls, CallRoute *r) {
  if (!g_tuned.any.load(std::memory_order_acquire)) return false;
  std::shared_lock<std::shared_mutex> lk(g_tuned.mu);
  const auto it = g_tuned.by_class.find(cls);
  if (it == g_tuned.by_class.end()) return false;
  *r = it->second;
  return true;
}

template <typename K>
inline CallRoute route_for(int64_t n, int32_t nseg) {
  CallRoute r{radix_min_for<K>(), g_stream_max_avg.load(std::memory_order_relaxed), 0,
              g_bucket_min_avg.load(std::memory_order_relaxed),
              static_cast<int32_t>(g_msd_on.load(std::memory_order_relaxed))};
  CallRoute t;
  if (tuned_route(route_class(static_cast<int>(sizeof(K)), n, nseg), &t)) {
    r = t;
    r.radix_min = clamp_radix_min<K>(r.radix_min);
  }
  return r;
}

// ---------------------------------------------------------------------------
// Workspace layout (every region 256-byte aligned).
struct WsLayout {
  size_t ctr = 0, jobs = 0, prefix = 0, half_first = 0, item_job = 0, split = 0, item_desc = 0,
         tmp_keys = 0, tmp_vals = 0, rjobs = 0, rprefix = 0, rtile_desc = 0, rdigits = 0,
         rhist = 0, rlook = 0, fallback = 0;
  size_t total = 0;
  int64_t max_fallback = 0;
  int32_t max_jobs = 0;
  int32_t max_rjobs = 0;
  int64_t max_items = 0;
  int64_t halves = 0;
  int64_t max_rtiles = 0;
  int64_t radix_min = 0;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// item: outputs per merge item.  half_entries: entries of the half-tile map
// (default: one problem of n elements, 2 * tiles + 1); a batch passes the sum
// over its instances and always needs the workspace.  radix_min: the radix
// threshold the workspace serves (kRadixMinFloor bounds every threshold);
// digits: radix digit positions of the key type.
constexpr WsLayout make_layout(int64_t n, int key_bytes, int val_bytes, int64_t cap,
                               int64_t item, int64_t half_entries = -1,
                               int64_t radix_min = kRadixMinFloor) {
  WsLayout L;
  if (n <= cap && half_entries < 0) return L;  // one tile: no workspace
  const int64_t rmin = radix_min > kRadixMinFloor ? radix_min : kRadixMinFloor;
  L.radix_min = rmin > cap ? rmin : cap;
  // Jobs are longer than cap: at most n / (cap + 1) of them; radix jobs are
  // longer than radix_min.
  L.max_jobs = static_cast<int32_t>(n / (cap + 1) + 1);
  L.max_rjobs = static_cast<int32_t>(n / (L.radix_min + 1) + 1);
  // Merge items: ceil(len / item) per job.
  L.max_items = n / item + L.max_jobs + 1;
  // Radix tiles: ceil(len / tile) per radix job.
  L.max_rtiles = n / kRadixTile + L.max_rjobs + 1;
  L.halves = half_entries < 0 ? 2 * ((n + cap - 1) / cap) : half_entries - 1;
  size_t off = 0;
  auto take = [&off](size_t bytes) {
    const size_t at = off;
    off = align256(off + bytes);
    return at;
  };
  const size_t mj = static_cast<size_t>(L.max_jobs);
  const size_t mi = static_cast<size_t>(L.max_items);
  const size_t mr = static_cast<size_t>(L.max_rjobs);
  const size_t digits = static_cast<size_t>(key_bytes);  // 8-bit digits
  L.ctr = take(kCtrWords * sizeof(uint32_t));
  L.jobs = take(mj * sizeof(int4));
  L.prefix = take((mj + 1) * 4);
  L.half_first = take(static_cast<size_t>(L.halves + 1) * 4);
  L.item_job = take(mi * 4);
  L.split = take(mi * 4);
  L.item_desc = take(mi * 2 * sizeof(int4));
  L.rjobs = take(mr * sizeof(int4));
  L.rprefix = take((mr + 1) * 4);
  L.rtile_desc = take(static_cast<size_t>(L.max_rtiles) * sizeof(int4));
  L.rdigits = take(mr * 4);
  L.rhist = take(mr * digits * kRBuckets * 4);
  L.rlook = take(static_cast<size_t>(L.max_rtiles) * kRBuckets * 8);
  // Every chunk of every tile may fall back from the bucket sort.
  L.max_fallback = kMaxTileChunks * ((L.halves + 1) / 2 + 1);
  L.fallback = take(static_cast<size_t>(L.max_fallback) * sizeof(TileChunk));
  L.tmp_keys = take(static_cast<size_t>(n) * key_bytes);
  L.tmp_vals = take(static_cast<size_t>(n) * val_bytes);
  L.total = off;
  return L;
}

// The layout a call of n elements uses, for its radix threshold.
template <typename K, bool PAIRS>
inline WsLayout layout_for(int64_t n, int64_t radix_min) {
  return make_layout(n, sizeof(K), PAIRS ? 4 : 0, tile_cap<K>(), MergeShape<K>::T, -1, radix_min);
}

// A layout that serves every radix threshold (caller-sized workspaces).
template <typename K, bool PAIRS>
inline WsLayout layout_any_threshold(int64_t n) {
  return make_layout(n, sizeof(K), PAIRS ? 4 : 0, tile_cap<K>(), MergeShape<K>::T, -1,
                     kRadixMinFloor);
}

// Device views of a workspace laid out by make_layout at `base`.
template <typename K, bool PAIRS>
inline LargeWs<K> ws_views(unsigned char *base, const WsLayout &L) {
  LargeWs<K> W;
  W.ctr = reinterpret_cast<uint32_t *>(base + L.ctr);
  W.jobs = reinterpret_cast<int4 *>(base + L.jobs);
  W.item_prefix = reinterpret_cast<int32_t *>(base + L.prefix);
  W.half_first = reinterpret_cast<int32_t *>(base + L.half_first);
  W.item_job = reinterpret_cast<int32_t *>(base + L.item_job);
  W.split = reinterpret_cast<uint32_t *>(base + L.split);
  W.item_desc = reinterpret_cast<int4 *>(base + L.item_desc);
  W.tmp_keys = reinterpret_cast<K *>(base + L.tmp_keys);
  W.tmp_vals = PAIRS ? reinterpret_cast<uint32_t *>(base + L.tmp_vals) : nullptr;
  W.rjobs = reinterpret_cast<int4 *>(base + L.rjobs);
  W.rtile_prefix = reinterpret_cast<int32_t *>(base + L.rprefix);
  W.rtile_desc = reinterpret_cast<int4 *>(base + L.rtile_desc);
  W.rdigits = reinterpret_cast<uint32_t *>(base + L.rdigits);
  W.rhist = reinterpret_cast<uint32_t *>(base + L.rhist);
  W.rlook = reinterpret_cast<unsigned long long *>(base + L.rlook);
  W.fallback = reinterpret_cast<TileChunk *>(base + L.fallback);
  W.max_fallback = L.max_fallback;
  W.max_jobs = L.max_jobs;
  W.max_rjobs = L.max_rjobs;
  W.max_items = L.max_items;
  W.halves = L.halves;
  W.max_rtiles = L.max_rtiles;
  W.radix_min = L.radix_min;
  W.msd_stage = 0;
  W.lsd_min = L.radix_min;
  W.tile_cap = static_cast<int32_t>(tile_cap<K>());
  return W;
}

// ---------------------------------------------------------------------------
// Per-device state: SM count and a library-owned memory pool that keeps its
// memory between calls (release threshold = max), so stream-ordered
// allocations after the first are cheap and never synchronise.
struct DeviceState {
  std::once_flag once;
  int sms = 0;
  int coop = 0;  // cooperative launches supported
  cudaError_t init_err = cudaSuccess;
  std::once_flag pool_once;  // the pool is created on the first internal allocation
  cudaMemPool_t pool = nullptr;
  cudaError_t pool_err = cudaSuccess;
  std::atomic<bool> pool_made{false};  // set once the pool exists
};
inline DeviceState g_dev[kMaxDevices];

inline DeviceState *device_state(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  DeviceState &S = g_dev[dev];
  std::call_once(S.once, [&] {
    cudaError_t e = cudaDeviceGetAttribute(&S.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&S.coop, cudaDevAttrCooperativeLaunch, dev);
    S.init_err = e;
  });
  return S.init_err == cudaSuccess ? &S : nullptr;
}

inline cudaMemPool_t device_pool(DeviceState &S, int dev) {
  std::call_once(S.pool_once, [&] {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaError_t e = cudaMemPoolCreate(&S.pool, &props);
    if (e == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      e = cudaMemPoolSetAttribute(S.pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    S.pool_err = e;
    if (e == cudaSuccess) S.pool_made.store(true, std::memory_order_release);
  });
  return S.pool_err == cudaSuccess ? S.pool : nullptr;
}

// Launches a kernel that begins with pdl_wait() right behind the kernel
// before it on the stream (programmatic stream serialization): its CTAs may
// be scheduled while that kernel finishes.  A failed launch is also recorded
// for cudaGetLastError(), which the sort checks after each stage, as for its
// <<<>>> launches.
template <typename... KArgs, typename... Args>
cudaError_t launch_after(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                         cudaStream_t stream, Args &&...args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Opt a kernel into more than 48 KB of dynamic shared memory once per device.
template <typename Kern>
cudaError_t ensure_smem(Kern kernel, size_t bytes, std::atomic<uint64_t> &done, int dev) {
  const uint64_t bit = 1ull << dev;
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(bytes));
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
  return e;
}

// Resident CTAs per SM of a kernel, cached per device.
template <typename Kern>
int occupancy(Kern kernel, int threads, size_t smem, std::atomic<int> (&cache)[kMaxDevices],
              int dev) {
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, threads, smem) != cudaSuccess ||
      v < 1)
    v = 1;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

// Status word of the batched form's translation unit (segsort_batch.cu).
cudaError_t batch_device_status(bool clear, uint32_t *value);

}  // namespace segsort
