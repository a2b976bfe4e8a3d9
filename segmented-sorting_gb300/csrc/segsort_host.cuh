// Host-side pieces shared by the library's translation units: kernel shapes,
// the workspace layout, per-device state with the stream-ordered pool, and
// launch helpers.  Mutable state is `inline` so that every unit of the
// library sees one copy.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_common.cuh"
#include "tile_sort.cuh"
#include "tile_stream.cuh"
#include "classify.cuh"
#include "merge_sort.cuh"

namespace segsort {

constexpr int kMaxDevices = 64;

// ---------------------------------------------------------------------------
// Tile-sort shape per key width: 4096-element chunks for 32-bit keys (256
// threads x 16 words), 2048 for 64-bit keys (256 threads x 8 words).
// Build-time tuning knobs (defaults are the measured best on GB300).
#ifndef SEGSORT_TILE_KPT32
#define SEGSORT_TILE_KPT32 16
#endif
#ifndef SEGSORT_TILE_MINB
#define SEGSORT_TILE_MINB 2
#endif
template <typename K, bool PAIRS>
struct TileFor {
  using Cfg = TileConfig<K, PAIRS, 256, sizeof(K) == 4 ? SEGSORT_TILE_KPT32 : 8>;
  static constexpr int kMinBlocks = SEGSORT_TILE_MINB;  // resident CTAs per SM the registers must allow
};

template <typename K>
constexpr int64_t tile_cap() {
  return TileFor<K, false>::Cfg::CAP;
}

// ---------------------------------------------------------------------------
// Workspace layout (every region 256-byte aligned).
struct WsLayout {
  size_t ctr = 0, jobs = 0, prefix = 0, half_first = 0, item_job = 0, split = 0, item_desc = 0,
         tmp_keys = 0, tmp_vals = 0;
  size_t total = 0;
  int32_t max_jobs = 0;
  int64_t max_items = 0;
  int64_t halves = 0;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// item: outputs per merge item.  half_entries: entries of the half-tile map
// (default: one problem of n elements, 2 * tiles + 1); a batch passes the sum
// over its instances and always needs the workspace.
constexpr WsLayout make_layout(int64_t n, int key_bytes, int val_bytes, int64_t cap,
                               int64_t item, int64_t half_entries = -1) {
  WsLayout L;
  if (n <= cap && half_entries < 0) return L;  // one tile: no workspace
  // Jobs are longer than cap: at most n / (cap + 1) of them.
  L.max_jobs = static_cast<int32_t>(n / (cap + 1) + 1);
  // Merge items: ceil(len / item) per job.
  L.max_items = n / item + L.max_jobs + 1;
  L.halves = half_entries < 0 ? 2 * ((n + cap - 1) / cap) : half_entries - 1;
  size_t off = 0;
  auto take = [&off](size_t bytes) {
    const size_t at = off;
    off = align256(off + bytes);
    return at;
  };
  const size_t mj = static_cast<size_t>(L.max_jobs);
  const size_t mi = static_cast<size_t>(L.max_items);
  L.ctr = take(kCtrWords * sizeof(uint32_t));
  L.jobs = take(mj * sizeof(int4));
  L.prefix = take((mj + 1) * 4);
  L.half_first = take(static_cast<size_t>(L.halves + 1) * 4);
  L.item_job = take(mi * 4);
  L.split = take(mi * 4);
  L.item_desc = take(mi * 2 * sizeof(int4));
  L.tmp_keys = take(static_cast<size_t>(n) * key_bytes);
  L.tmp_vals = take(static_cast<size_t>(n) * val_bytes);
  L.total = off;
  return L;
}

template <typename K, bool PAIRS>
inline WsLayout layout_for(int64_t n) {
  return make_layout(n, sizeof(K), PAIRS ? 4 : 0, tile_cap<K>(), MergeShape<K>::T);
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
  W.max_jobs = L.max_jobs;
  W.max_items = L.max_items;
  W.halves = L.halves;
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
  });
  return S.pool_err == cudaSuccess ? S.pool : nullptr;
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
