// C ABI of the segmented sort: argument checks, workspace layout, the
// stream-ordered workspace pool and the launch sequence of one call.  The
// batched form lives in segsort_batch.cu.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_host.cuh"

namespace segsort {
namespace {

// ---------------------------------------------------------------------------
// Opt-in phase timing (segsort_profile_enable / segsort_profile_read).
struct PhaseRecord {
  cudaEvent_t t0 = nullptr, t1 = nullptr, l0 = nullptr, l1 = nullptr;
  cudaEvent_t m0 = nullptr, m1 = nullptr;  // stage 1 of the MSD route (counted as large)
  int tile_launches = 1;
  int large_launches = 0;
};
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<PhaseRecord> g_prof_pending;
double g_prof_tile_ms = 0.0, g_prof_large_ms = 0.0;
int64_t g_prof_tile_launches = 0, g_prof_large_launches = 0;

cudaEvent_t prof_event(cudaStream_t stream) {
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  if (cudaEventRecord(e, stream) != cudaSuccess) {
    cudaEventDestroy(e);
    return nullptr;
  }
  return e;
}

// ---------------------------------------------------------------------------
// One plain call.  forced: the route to take (the tuner's trials); null: the
// call's own (route_for).
template <typename K, bool PAIRS>
int sort_impl(K *keys, uint32_t *vals, int64_t n, const int32_t *offsets, int32_t nseg,
              bool heads, void *ws, size_t ws_bytes, cudaStream_t stream,
              const CallRoute *forced = nullptr) {
  if (n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  if (n == 0 || nseg == 0) return SEGSORT_OK;
  if (keys == nullptr || offsets == nullptr || (PAIRS && vals == nullptr))
    return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  DeviceState *S = device_state(dev);
  if (S == nullptr) return SEGSORT_ERR_CUDA;

  const Offsets off{offsets, nseg, heads ? 1 : 0, n};
  CallRoute R = forced != nullptr ? *forced : route_for<K>(n, nseg);
  R.radix_min = clamp_radix_min<K>(R.radix_min);

  // ---- shapes ---------------------------------------------------------------
  using Cfg = typename TileFor<K, PAIRS>::Cfg;
  auto tile_kernel = tile_sort_kernel<K, PAIRS, Cfg::NT, Cfg::KPT, TileFor<K, PAIRS>::kMinBlocks>;
  static std::atomic<uint64_t> tile_attr_done{0};
  if (ensure_smem(tile_kernel, Cfg::kSmemBytes, tile_attr_done, dev) != cudaSuccess)
    return SEGSORT_ERR_CUDA;
  const int64_t tiles = (n + Cfg::CAP - 1) / Cfg::CAP;
  const bool prof = g_prof_on.load(std::memory_order_relaxed);
  PhaseRecord rec;

  // ---- one tile: every segment fits, no workspace, one kernel ---------------
  if (tiles == 1) {
    if (prof) rec.t0 = prof_event(stream);
    tile_kernel<<<1, Cfg::NT, Cfg::kSmemBytes, stream>>>(keys, vals, off, nullptr, nullptr, nullptr,
                                                          0);
    if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
    if (prof) {
      rec.t1 = prof_event(stream);
      std::lock_guard<std::mutex> lk(g_prof_mu);
      g_prof_pending.push_back(rec);
    }
    return SEGSORT_OK;
  }

  // ---- workspace ----------------------------------------------------------------
  // A caller's workspace is sized for every radix threshold
  // (segsort_workspace_bytes); the library's own is sized for the current one.
  // MSD route (msd_route.cuh): problems whose average segment is longer than
  // the MSD threshold, in a workspace the library owns (the expansion's
  // arrays grow with nseg).  Its first stage takes the segments longer than
  // that threshold, which may be below the radix threshold.
  const int64_t msd_min = msd_min_for<K>(R.radix_min);
  const bool msd = R.msd != 0 && ws == nullptr && n > msd_min * static_cast<int64_t>(nseg);
  const WsLayout L = ws != nullptr ? layout_any_threshold<K, PAIRS>(n)
                                   : layout_for<K, PAIRS>(n, msd ? msd_min : R.radix_min);
  const int64_t c_len = msd ? msd_stage2_segments(nseg, L.max_rjobs) : 0;
  size_t msd_at[6] = {0, 0, 0, 0, 0, 0};  // sub, flags, jbeg, jidx, jextra, end
  if (msd) {
    const size_t rj = static_cast<size_t>(L.max_rjobs) + 1;
    const size_t sizes[5] = {static_cast<size_t>(c_len + 1) * 4, static_cast<size_t>(c_len),
                             rj * 4, rj * 4, rj * 4};
    size_t at = L.total;
    for (int i = 0; i < 5; ++i) {
      msd_at[i] = at;
      at = align256(at + sizes[i]);
    }
    msd_at[5] = at;
  }
  const size_t alloc_bytes = msd ? msd_at[5] : L.total;
  bool owned = false;
  unsigned char *base = static_cast<unsigned char *>(ws);
  if (base == nullptr) {
    cudaMemPool_t pool = device_pool(*S, dev);
    if (pool == nullptr ||
        cudaMallocFromPoolAsync(reinterpret_cast<void **>(&base), alloc_bytes, pool, stream) !=
            cudaSuccess) {
      cudaGetLastError();
      return SEGSORT_ERR_NO_MEMORY;
    }
    owned = true;
  } else if (ws_bytes < L.total || (reinterpret_cast<uintptr_t>(base) & 255) != 0) {
    return SEGSORT_ERR_WORKSPACE;
  }

  LargeWs<K> W = ws_views<K, PAIRS>(base, L);
  W.radix_min = std::max<int64_t>(L.radix_min, R.radix_min);
  W.lsd_min = W.radix_min;

  // The long-segment kernel: radix passes, then merge passes, one cooperative
  // launch (returns at once without long segments).  All resident CTAs, but
  // no more than one per merge item of the whole problem: small calls then
  // leave the rest of the GPU to other work.
  using MS = LongSmem<K, PAIRS>;
  auto merge_kernel = long_segment_kernel<K, PAIRS, SingleSpace<K>>;
  static std::atomic<uint64_t> merge_attr_done{0};
  static std::atomic<int> merge_occ[kMaxDevices];
  auto launch_long = [&](LargeWs<K> &Wl) -> int {
    if (!S->coop || ensure_smem(merge_kernel, MS::kBytes, merge_attr_done, dev) != cudaSuccess)
      return SEGSORT_ERR_CUDA;
    const int mo = occupancy(merge_kernel, kMThreads, MS::kBytes, merge_occ, dev);
    const int per_sm = R.merge_per_sm > 0 ? std::min(R.merge_per_sm, mo) : mo;
    const int64_t items = n / MergeShape<K>::T + 1;
    const unsigned merge_grid =
        static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(per_sm) * S->sms, items));
    SingleSpace<K> sp{keys, vals, W.tmp_keys, W.tmp_vals};
    int64_t cap = tile_cap<K>();
    void *args[] = {&sp, &Wl, &cap};
    if (cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(merge_kernel), dim3(merge_grid),
                                    dim3(kMThreads), args, MS::kBytes, stream) != cudaSuccess)
      return SEGSORT_ERR_CUDA;
    return SEGSORT_OK;
  };
  auto segment_classify = [&](const Offsets &o) {
    const unsigned blocks = static_cast<unsigned>((static_cast<int64_t>(o.nseg) + 1 + 255) / 256);
    large_classify_kernel<K><<<blocks, 256, 0, stream>>>(o, tile_cap<K>(), tile_cap<K>() / 2, W);
  };

  int rc = SEGSORT_OK;
  do {
    Offsets O = off;  // the offsets the tile sort and the merge passes see
    if (msd) {
      // ---- MSD route, stage 1 and the expansion (msd_route.cuh) ------------
      MsdWs M{reinterpret_cast<int32_t *>(base + msd_at[0]),
              reinterpret_cast<uint8_t *>(base + msd_at[1]), c_len,
              reinterpret_cast<int32_t *>(base + msd_at[2]),
              reinterpret_cast<int32_t *>(base + msd_at[3]),
              reinterpret_cast<int32_t *>(base + msd_at[4])};
      if (cudaMemsetAsync(W.ctr, 0, kCtrWords * sizeof(uint32_t), stream) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      const int64_t lsd_radix_min = W.radix_min;
      W.radix_min = std::max<int64_t>(msd_min, L.radix_min);  // stage 1's jobs
      segment_classify(off);
      if (prof) rec.m0 = prof_event(stream);
      W.msd_stage = 1;
      rc = launch_long(W);
      W.msd_stage = 0;
      if (rc != SEGSORT_OK) break;
      launch_after(msd_rank_kernel<K>, static_cast<unsigned>((W.max_rjobs + 255) / 256), 256, 0,
                   stream, W, M);
      launch_after(msd_expand_kernel<K>,
                   static_cast<unsigned>((std::max<int64_t>(nseg, c_len) + 256) / 256), 256, 0,
                   stream, off, W, M);
      launch_after(msd_sub_kernel<K>, static_cast<unsigned>(W.max_rjobs), kRBuckets, 0, stream, W,
                   M);
      if (prof) rec.m1 = prof_event(stream);
      if (cudaGetLastError() != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      O = Offsets{M.sub, static_cast<int32_t>(c_len), 0, n, M.flags};
      W.radix_min = lsd_radix_min;
    }
    // ---- classify: half-tile -> first segment map, jobs for long segments ----
    if (cudaMemsetAsync(W.ctr, 0, kCtrWords * sizeof(uint32_t), stream) != cudaSuccess) {
      rc = SEGSORT_ERR_CUDA;
      break;
    }
    // Short segments on average: one search per half-tile (work ~ n / CAP);
    // otherwise one thread per segment boundary (work ~ nseg, fewer rounds
    // of dependent loads).  The two write the same map and jobs.  The MSD
    // route's sub-buckets are long on average (the expansion pads the
    // offsets with empty segments, so n / O.nseg understates them).
    const bool short_avg =
        !msd && R.stream_max_avg > 0 && n <= R.stream_max_avg * static_cast<int64_t>(nseg);
    const int64_t bucket_min = R.bucket_min_avg;
    if (short_avg) {
      const unsigned blocks =
          static_cast<unsigned>((W.halves + kClassifyWarps) / kClassifyWarps);  // halves + 1 entries
      large_classify_halves_kernel<K><<<blocks, (kClassifyWarps + 1) * 32, 0, stream>>>(
          off, tile_cap<K>(), tile_cap<K>() / 2, W);
    } else {
      segment_classify(O);
    }

    // ---- tile sort: every segment of at most CAP elements, and the sorted
    // CAP-runs of the longer ones.  Short segments on average: the streamed
    // kernel (persistent CTAs that copy the next tile in while they sort this
    // one; the load latency dominates there).  Otherwise one CTA per tile: the
    // sort dominates, and the hardware scheduler balances the tiles better
    // than a static split over resident CTAs.
    if (prof) rec.t0 = prof_event(stream);
    const int64_t tiny_max = g_tiny_max_avg.load(std::memory_order_relaxed);
    const bool tiny = short_avg && tiny_max > 0 && n <= tiny_max * static_cast<int64_t>(nseg);
    if (tiny) {
      // Tiny route: the network sort of chunks of segments of at most kTinyMax
      // keys, two tiles' copies in flight per CTA; the other chunks listed
      // for the comparison sort.
      using TL = TinyLayout<K, PAIRS, Cfg::CAP>;
      auto tiny_kernel = tile_tiny_kernel<K, PAIRS, kTinyThreads, Cfg::CAP, 2>;
      auto list_kernel =
          tile_list_kernel<K, PAIRS, Cfg::NT, Cfg::KPT, TileFor<K, PAIRS>::kMinBlocks>;
      static std::atomic<uint64_t> tiny_attr_done{0}, tlist_attr_done{0};
      static std::atomic<int> tiny_occ[kMaxDevices], tlist_occ[kMaxDevices];
      if (ensure_smem(tiny_kernel, TL::kBytes, tiny_attr_done, dev) != cudaSuccess ||
          ensure_smem(list_kernel, Cfg::kSmemBytes, tlist_attr_done, dev) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      const int to = occupancy(tiny_kernel, kTinyThreads, TL::kBytes, tiny_occ, dev);
      const unsigned tgrid =
          static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(to) * S->sms, tiles));
      launch_after(tiny_kernel, tgrid, kTinyThreads, TL::kBytes, stream, keys, vals, O,
                   static_cast<const int32_t *>(W.half_first), tiles, true, W.radix_min,
                   W.fallback, W.ctr + kCtrFallback, W.max_fallback);
      const int lo = occupancy(list_kernel, Cfg::NT, Cfg::kSmemBytes, tlist_occ, dev);
      const unsigned lgrid =
          static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(lo) * S->sms, tiles));
      launch_after(list_kernel, lgrid, Cfg::NT, Cfg::kSmemBytes, stream, keys, vals, O,
                   W.tmp_keys, W.tmp_vals, static_cast<const TileChunk *>(W.fallback),
                   static_cast<const uint32_t *>(W.ctr + kCtrFallback), W.max_fallback,
                   W.ctr + kCtrListTicket);
      rec.tile_launches = 2;
    } else if (short_avg) {
      using SL = StreamLayout<Cfg, K, PAIRS>;
      auto stream_kernel =
          tile_stream_kernel<K, PAIRS, Cfg::NT, Cfg::KPT, TileFor<K, PAIRS>::kMinBlocks>;
      static std::atomic<uint64_t> stream_attr_done{0};
      static std::atomic<int> stream_occ[kMaxDevices];
      if (ensure_smem(stream_kernel, SL::kBytes, stream_attr_done, dev) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      const int so = occupancy(stream_kernel, Cfg::NT, SL::kBytes, stream_occ, dev);
      const unsigned grid =
          static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(so) * S->sms, tiles));
      launch_after(stream_kernel, grid, Cfg::NT, SL::kBytes, stream, keys, vals, O,
                   static_cast<const int32_t *>(W.half_first), W.tmp_keys, W.tmp_vals, tiles,
                   W.radix_min);
    } else if (bucket_min > 0 && (msd || n >= bucket_min * static_cast<int64_t>(nseg))) {
      // Bucket route: the bucket kernel sorts the chunks it can and lists the
      // others; persistent comparison-sort CTAs take the list.
      using BF = BucketFor<K, PAIRS>;
      using BCfg = typename BF::Cfg;
      constexpr size_t kBSmem = BucketLayout<BCfg, PAIRS>::kBytes;
      auto bucket_kernel = tile_bucket_kernel<K, PAIRS, BCfg::NT, BCfg::KPT, BF::kMinBlocks>;
      auto list_kernel =
          tile_list_kernel<K, PAIRS, Cfg::NT, Cfg::KPT, TileFor<K, PAIRS>::kMinBlocks>;
      static std::atomic<uint64_t> bucket_attr_done{0}, list_attr_done{0};
      static std::atomic<int> list_occ[kMaxDevices];
      if (ensure_smem(bucket_kernel, kBSmem, bucket_attr_done, dev) != cudaSuccess ||
          ensure_smem(list_kernel, Cfg::kSmemBytes, list_attr_done, dev) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      launch_after(bucket_kernel, static_cast<unsigned>(tiles), BCfg::NT, kBSmem, stream, keys,
                   vals, O, static_cast<const int32_t *>(W.half_first), W.tmp_keys, W.tmp_vals,
                   W.radix_min, W.fallback, W.ctr + kCtrFallback, W.max_fallback);
      const int lo = occupancy(list_kernel, Cfg::NT, Cfg::kSmemBytes, list_occ, dev);
      const unsigned lgrid =
          static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(lo) * S->sms, tiles));
      launch_after(list_kernel, lgrid, Cfg::NT, Cfg::kSmemBytes, stream, keys, vals, O,
                   W.tmp_keys, W.tmp_vals, static_cast<const TileChunk *>(W.fallback),
                   static_cast<const uint32_t *>(W.ctr + kCtrFallback), W.max_fallback,
                   W.ctr + kCtrListTicket);
      rec.tile_launches = 2;
    } else {
      launch_after(tile_kernel, static_cast<unsigned>(tiles), Cfg::NT, Cfg::kSmemBytes, stream,
                   keys, vals, O, static_cast<const int32_t *>(W.half_first), W.tmp_keys,
                   W.tmp_vals, W.radix_min);
    }
    if (prof) rec.t1 = prof_event(stream);
    if (cudaGetLastError() != cudaSuccess) {
      rc = SEGSORT_ERR_CUDA;
      break;
    }

    // ---- long segments: radix passes, then merge passes ----------------------
    if (prof) rec.l0 = prof_event(stream);
    rc = launch_long(W);
    if (rc != SEGSORT_OK) break;
    if (prof) rec.l1 = prof_event(stream);
  } while (false);
  if (prof) {
    // classify and the cooperative long-segment kernel; with the MSD route
    // also the first classify and long-segment kernel and the three
    // expansion kernels.
    rec.large_launches = msd ? 7 : 2;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_pending.push_back(rec);
  }

  if (owned && cudaFreeAsync(base, stream) != cudaSuccess && rc == SEGSORT_OK) rc = SEGSORT_ERR_CUDA;
  return rc;
}

template <typename K, bool PAIRS>
size_t workspace_bytes_for(int64_t n) {
  return layout_any_threshold<K, PAIRS>(n).total;
}

// ---------------------------------------------------------------------------
// Scratch of the allocation-free entry point: the workspace of the largest
// problem it accepts (SEGSORT_NOALLOC_MAX_N uint32 key/value pairs), as part of
// the module's device image.  Host code cannot use the array's name as a
// device address; its address is looked up once per device.
constexpr int64_t kNoAllocMaxN = SEGSORT_NOALLOC_MAX_N;
constexpr size_t kNoAllocBytes =
    make_layout(kNoAllocMaxN, 4, 4, tile_cap<uint32_t>(), MergeShape<uint32_t>::T).total;
static_assert(kNoAllocBytes > 0, "the no-allocation scratch must cover the long-segment path");
// The documented figure: about 10 MiB on every GPU that loads the library.
static_assert(kNoAllocBytes > (size_t{19} << 19) && kNoAllocBytes <= (size_t{21} << 19),
              "the header, design and integration notes state about 10 MiB");

struct NoAllocScratch {
  std::once_flag once;
  void *ptr = nullptr;
  cudaError_t err = cudaSuccess;
};
NoAllocScratch g_noalloc[kMaxDevices];

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
// Device address of the scratch array on `dev`, which must be the current
// device: looked up on the first call per device, then cached.
void *noalloc_scratch(int dev) {
  NoAllocScratch &S = g_noalloc[dev];
  std::call_once(S.once, [&] { S.err = cudaGetSymbolAddress(&S.ptr, g_noalloc_scratch); });
  return S.err == cudaSuccess ? S.ptr : nullptr;
}

// ---------------------------------------------------------------------------
// Self-test kernels of the bounded waits: each wait below can never complete,
// and gives up after kSelftestSpins back-offs (a few milliseconds).
constexpr int kSelftestSpins = 1 << 12;
__device__ uint32_t g_selftest_ctr[kCtrWords];
__device__ unsigned long long g_selftest_look[2 * kRBuckets];

// A grid barrier CTA 1 never reaches (cooperative launch of two CTAs).
__global__ void selftest_barrier_kernel() {
  if (blockIdx.x != 0) return;
  grid_barrier(g_selftest_ctr, kSelftestSpins);
}

// An mbarrier phase expecting 16 bytes that no copy supplies.
__global__ void selftest_mbar_kernel() {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, 16);
    if (!mbar_wait(&bar, 0, kSelftestSpins)) raise_status(kStatusTimeout);
  }
}

// ---------------------------------------------------------------------------
// Tuner of plain calls: the median of three timed calls (after an untimed
// one) of the sort with route R, each on a fresh copy of the saved inputs.
template <typename K, bool PAIRS>
int time_route(K *keys, uint32_t *vals, const K *k0, const uint32_t *v0, int64_t n,
               const int32_t *offsets, int32_t nseg, cudaStream_t stream, const CallRoute &R,
               cudaEvent_t a, cudaEvent_t b, float *ms) {
  float t[3] = {0.f, 0.f, 0.f};
  for (int r = -1; r < 3; ++r) {
    if (cudaMemcpyAsync(keys, k0, n * sizeof(K), cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
        (PAIRS && cudaMemcpyAsync(vals, v0, n * 4, cudaMemcpyDeviceToDevice, stream) != cudaSuccess) ||
        cudaEventRecord(a, stream) != cudaSuccess)
      return SEGSORT_ERR_CUDA;
    const int rc = sort_impl<K, PAIRS>(keys, vals, n, offsets, nseg, false, nullptr, 0, stream, &R);
    if (rc != SEGSORT_OK) return rc;
    if (cudaEventRecord(b, stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess)
      return SEGSORT_ERR_CUDA;
    if (r >= 0 && cudaEventElapsedTime(&t[r], a, b) != cudaSuccess) return SEGSORT_ERR_CUDA;
  }
  std::sort(t, t + 3);
  *ms = t[1];
  return SEGSORT_OK;
}

// Coordinate search over the route of one problem: the radix threshold, then
// the streamed-tile threshold, the long-segment kernel's CTAs per SM, the
// bucket-route threshold and the MSD route; a candidate replaces the best so
// far when it is at least 2% faster.  On
// return the caller's buffers hold the problem sorted with the chosen route.
template <typename K, bool PAIRS>
int tune_impl(K *keys, uint32_t *vals, int64_t n, const int32_t *offsets, int32_t nseg,
              cudaStream_t stream, CallRoute *best) {
  if (n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  *best = route_for<K>(n, nseg);
  if (n == 0 || nseg == 0) return SEGSORT_OK;
  if (keys == nullptr || offsets == nullptr || (PAIRS && vals == nullptr))
    return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  DeviceState *S = device_state(dev);
  cudaMemPool_t pool = S ? device_pool(*S, dev) : nullptr;
  const size_t kbytes = static_cast<size_t>(n) * sizeof(K), vbytes = PAIRS ? n * 4 : 0;
  unsigned char *saved = nullptr;
  if (pool == nullptr ||
      cudaMallocFromPoolAsync(reinterpret_cast<void **>(&saved), align256(kbytes) + vbytes + 256,
                              pool, stream) != cudaSuccess) {
    cudaGetLastError();
    return SEGSORT_ERR_NO_MEMORY;
  }
  K *k0 = reinterpret_cast<K *>(saved);
  uint32_t *v0 = reinterpret_cast<uint32_t *>(saved + align256(kbytes));
  cudaEvent_t a = nullptr, b = nullptr;
  int rc = SEGSORT_OK;
  if (cudaMemcpyAsync(k0, keys, kbytes, cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
      (PAIRS && cudaMemcpyAsync(v0, vals, vbytes, cudaMemcpyDeviceToDevice, stream) != cudaSuccess) ||
      cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    rc = SEGSORT_ERR_CUDA;
  float best_ms = 0.f;
  if (rc == SEGSORT_OK)
    rc = time_route<K, PAIRS>(keys, vals, k0, v0, n, offsets, nseg, stream, *best, a, b, &best_ms);
  auto consider = [&](CallRoute R) {
    float ms = 0.f;
    if (rc != SEGSORT_OK) return;
    rc = time_route<K, PAIRS>(keys, vals, k0, v0, n, offsets, nseg, stream, R, a, b, &ms);
    if (rc == SEGSORT_OK && ms < 0.98f * best_ms) {
      *best = R;
      best_ms = ms;
    }
  };
  const CallRoute start = *best;
  for (int64_t v : {kRadixMinFloor, int64_t{1} << 15, int64_t{1} << 17, int64_t{1} << 30}) {
    CallRoute R = *best;
    R.radix_min = clamp_radix_min<K>(v);
    if (R.radix_min != start.radix_min) consider(R);
  }
  for (int64_t v : {int64_t{0}, int64_t{1} << 30}) {  // streamed tile kernel: never, always
    CallRoute R = *best;
    R.stream_max_avg = v;
    if ((n <= v * static_cast<int64_t>(nseg)) != (n <= start.stream_max_avg * static_cast<int64_t>(nseg)))
      consider(R);
  }
  for (int32_t v : {1, 2}) {
    CallRoute R = *best;
    R.merge_per_sm = v;
    consider(R);
  }
  const auto bucket_on = [&](int64_t v) { return v > 0 && n >= v * static_cast<int64_t>(nseg); };
  for (int64_t v : {int64_t{0}, int64_t{64}, int64_t{256}}) {  // bucket route: off, wider, narrower
    CallRoute R = *best;
    R.bucket_min_avg = v;
    if (bucket_on(v) != bucket_on(start.bucket_min_avg)) consider(R);
  }
  if (n > best->radix_min * static_cast<int64_t>(nseg)) {  // MSD route: the other choice
    CallRoute R = *best;
    R.msd = best->msd ? 0 : 1;
    consider(R);
  }
  // The caller's buffers end sorted with the chosen route.
  if (rc == SEGSORT_OK &&
      (cudaMemcpyAsync(keys, k0, kbytes, cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
       (PAIRS && cudaMemcpyAsync(vals, v0, vbytes, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)))
    rc = SEGSORT_ERR_CUDA;
  if (rc == SEGSORT_OK)
    rc = sort_impl<K, PAIRS>(keys, vals, n, offsets, nseg, false, nullptr, 0, stream, best);
  if (cudaFreeAsync(saved, stream) != cudaSuccess && rc == SEGSORT_OK) rc = SEGSORT_ERR_CUDA;
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  return rc;
}

// Records a route for a class in the process's table.
void record_route(uint32_t cls, const CallRoute &R) {
  std::unique_lock<std::shared_mutex> lk(g_tuned.mu);
  g_tuned.by_class[cls] = R;
  g_tuned.any.store(true, std::memory_order_release);
}

// The look-back of tile 1 of a segment whose tile 0 never publishes.
__global__ void selftest_look_kernel() {
  look_back(g_selftest_look, 1, 1, static_cast<int>(threadIdx.x), 1u, 0, kSelftestSpins);
}
}  // namespace
}  // namespace segsort

using segsort::sort_impl;

extern "C" {

#define SEGSORT_ST(s) reinterpret_cast<cudaStream_t>(s)

int segsort_keys_u32(uint32_t *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return sort_impl<uint32_t, false>(k, nullptr, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_keys_i32(int32_t *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return sort_impl<int32_t, false>(k, nullptr, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_keys_f32(float *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return sort_impl<float, false>(k, nullptr, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_keys_u64(uint64_t *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return sort_impl<uint64_t, false>(k, nullptr, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}

int segsort_pairs_u32(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                      segsort_stream_t s) {
  return sort_impl<uint32_t, true>(k, v, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_pairs_i32(int32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                      segsort_stream_t s) {
  return sort_impl<int32_t, true>(k, v, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_pairs_f32(float *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                      segsort_stream_t s) {
  return sort_impl<float, true>(k, v, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}
int segsort_pairs_u64(uint64_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                      segsort_stream_t s) {
  return sort_impl<uint64_t, true>(k, v, n, o, ns, false, nullptr, 0, SEGSORT_ST(s));
}

int segsort_pairs_u32_heads(uint32_t *k, uint32_t *v, int64_t n, const int32_t *h, int32_t ns,
                            segsort_stream_t s) {
  return sort_impl<uint32_t, true>(k, v, n, h, ns, true, nullptr, 0, SEGSORT_ST(s));
}
int segsort_keys_u32_heads(uint32_t *k, int64_t n, const int32_t *h, int32_t ns,
                           segsort_stream_t s) {
  return sort_impl<uint32_t, false>(k, nullptr, n, h, ns, true, nullptr, 0, SEGSORT_ST(s));
}

size_t segsort_workspace_bytes(int64_t n, int32_t nseg, int key_bytes, int val_bytes) {
  (void)nseg;
  if (n <= 0) return 0;
  const bool pairs = val_bytes != 0;
  if (key_bytes == 8)
    return pairs ? segsort::workspace_bytes_for<uint64_t, true>(n)
                 : segsort::workspace_bytes_for<uint64_t, false>(n);
  return pairs ? segsort::workspace_bytes_for<uint32_t, true>(n)
               : segsort::workspace_bytes_for<uint32_t, false>(n);
}

int segsort_pairs_u32_ws(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                         void *ws, size_t ws_bytes, segsort_stream_t s) {
  if (ws == nullptr && segsort_workspace_bytes(n, ns, 4, 4) != 0) return SEGSORT_ERR_WORKSPACE;
  return sort_impl<uint32_t, true>(k, v, n, o, ns, false, ws, ws_bytes, SEGSORT_ST(s));
}
int segsort_keys_u32_ws(uint32_t *k, int64_t n, const int32_t *o, int32_t ns, void *ws,
                        size_t ws_bytes, segsort_stream_t s) {
  if (ws == nullptr && segsort_workspace_bytes(n, ns, 4, 0) != 0) return SEGSORT_ERR_WORKSPACE;
  return sort_impl<uint32_t, false>(k, nullptr, n, o, ns, false, ws, ws_bytes, SEGSORT_ST(s));
}

int segsort_pairs_u32_noalloc(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                              segsort_stream_t s) {
  if (n < 0 || ns < 0) return SEGSORT_ERR_INVALID_ARG;
  if (n > segsort::kNoAllocMaxN) return SEGSORT_ERR_TOO_LARGE;
  if (n == 0 || ns == 0) return SEGSORT_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= segsort::kMaxDevices)
    return SEGSORT_ERR_CUDA;
  void *scratch = segsort::noalloc_scratch(dev);
  if (scratch == nullptr) return SEGSORT_ERR_CUDA;
  return sort_impl<uint32_t, true>(k, v, n, o, ns, false, scratch, segsort::kNoAllocBytes,
                                   SEGSORT_ST(s));
}

int segsort_device_status(int clear) {
  if (cudaDeviceSynchronize() != cudaSuccess) return SEGSORT_ERR_CUDA;
  uint32_t v = 0, vb = 0;
  if (cudaMemcpyFromSymbol(&v, segsort::g_device_status, sizeof(v)) != cudaSuccess)
    return SEGSORT_ERR_CUDA;
  if (clear) {
    const uint32_t zero = 0;
    if (cudaMemcpyToSymbol(segsort::g_device_status, &zero, sizeof(zero)) != cudaSuccess)
      return SEGSORT_ERR_CUDA;
  }
  if (segsort::batch_device_status(clear != 0, &vb) != cudaSuccess) return SEGSORT_ERR_CUDA;
  return ((v | vb) & segsort::kStatusTimeout) ? SEGSORT_ERR_TIMEOUT : SEGSORT_OK;
}

int segsort_pool_bytes(int *created, uint64_t *used) {
  using namespace segsort;
  if (created == nullptr || used == nullptr) return SEGSORT_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  DeviceState *S = device_state(dev);
  if (S == nullptr) return SEGSORT_ERR_CUDA;
  *created = 0;
  *used = 0;
  if (!S->pool_made.load(std::memory_order_acquire)) return SEGSORT_OK;
  *created = 1;
  uint64_t v = 0;
  if (cudaMemPoolGetAttribute(S->pool, cudaMemPoolAttrUsedMemCurrent, &v) != cudaSuccess)
    return SEGSORT_ERR_CUDA;
  *used = v;
  return SEGSORT_OK;
}

int segsort_set_param(int param, int64_t value) {
  using namespace segsort;
  switch (param) {
    case SEGSORT_PARAM_RADIX_MIN_32:
      if (value < kRadixMinFloor) return SEGSORT_ERR_INVALID_ARG;
      g_radix_min32.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_RADIX_MIN_64:
      if (value < kRadixMinFloor) return SEGSORT_ERR_INVALID_ARG;
      g_radix_min64.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_STREAM_MAX_AVG:
      if (value < 0) return SEGSORT_ERR_INVALID_ARG;
      g_stream_max_avg.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_BUCKET_MIN_AVG:
      if (value < 0) return SEGSORT_ERR_INVALID_ARG;
      g_bucket_min_avg.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_MSD:
      if (value != 0 && value != 1) return SEGSORT_ERR_INVALID_ARG;
      g_msd_on.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_TINY_MAX_AVG:
      if (value < 0) return SEGSORT_ERR_INVALID_ARG;
      g_tiny_max_avg.store(value, std::memory_order_relaxed);
      return SEGSORT_OK;
    default:
      return SEGSORT_ERR_INVALID_ARG;
  }
}

int segsort_get_param(int param, int64_t *value) {
  using namespace segsort;
  if (value == nullptr) return SEGSORT_ERR_INVALID_ARG;
  switch (param) {
    case SEGSORT_PARAM_RADIX_MIN_32: *value = radix_min_for<uint32_t>(); return SEGSORT_OK;
    case SEGSORT_PARAM_RADIX_MIN_64: *value = radix_min_for<uint64_t>(); return SEGSORT_OK;
    case SEGSORT_PARAM_STREAM_MAX_AVG:
      *value = g_stream_max_avg.load(std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_BUCKET_MIN_AVG:
      *value = g_bucket_min_avg.load(std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_MSD:
      *value = g_msd_on.load(std::memory_order_relaxed);
      return SEGSORT_OK;
    case SEGSORT_PARAM_TINY_MAX_AVG:
      *value = g_tiny_max_avg.load(std::memory_order_relaxed);
      return SEGSORT_OK;
    default:
      return SEGSORT_ERR_INVALID_ARG;
  }
}

int segsort_tune_pairs_u32(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           segsort_stream_t s, const char *cache_path, int64_t *radix_min,
                           int64_t *stream_max_avg, int32_t *merge_ctas_per_sm) {
  using namespace segsort;
  CallRoute R{};
  const int rc = tune_impl<uint32_t, true>(k, v, n, o, ns, SEGSORT_ST(s), &R);
  if (rc != SEGSORT_OK) return rc;
  if (n > 0 && ns > 0) {
    const uint32_t cls = route_class(4, n, ns);
    record_route(cls, R);
    if (cache_path != nullptr) {
      if (FILE *f = std::fopen(cache_path, "a")) {
        std::fprintf(f, "plain k%u n%u len%u %lld %lld %d %lld %d\n", cls >> 16, (cls >> 8) & 255u,
                     cls & 255u, static_cast<long long>(R.radix_min),
                     static_cast<long long>(R.stream_max_avg), R.merge_per_sm,
                     static_cast<long long>(R.bucket_min_avg), R.msd);
        std::fclose(f);
      }
    }
  }
  if (radix_min) *radix_min = R.radix_min;
  if (stream_max_avg) *stream_max_avg = R.stream_max_avg;
  if (merge_ctas_per_sm) *merge_ctas_per_sm = R.merge_per_sm;
  return SEGSORT_OK;
}

int segsort_tune_load(const char *cache_path) {
  using namespace segsort;
  if (cache_path == nullptr) return SEGSORT_ERR_INVALID_ARG;
  FILE *f = std::fopen(cache_path, "r");
  if (f == nullptr) return SEGSORT_ERR_INVALID_ARG;
  char line[256];
  int loaded = 0;
  while (std::fgets(line, sizeof(line), f)) {
    unsigned kb = 0, lgn = 0, lgl = 0;
    long long radix = 0, stream = 0, bucket = 128;
    int merge = 0, msd = 1;
    // Lines of six fields (written before the bucket and MSD fields existed)
    // take those two at their defaults.
    const int got = std::sscanf(line, "plain k%u n%u len%u %lld %lld %d %lld %d", &kb, &lgn, &lgl,
                                &radix, &stream, &merge, &bucket, &msd);
    if (got != 6 && got != 8) continue;  // another tuner's line
    if ((kb != 4 && kb != 8) || lgn > 40 || lgl > 40 || radix < 0 || stream < 0 || merge < 0 ||
        merge > 64 || bucket < 0 || (msd != 0 && msd != 1))
      continue;
    record_route((kb << 16) | (lgn << 8) | lgl, CallRoute{radix, stream, merge, bucket, msd});
    ++loaded;
  }
  std::fclose(f);
  return loaded;
}

void segsort_tune_clear(void) {
  using namespace segsort;
  std::unique_lock<std::shared_mutex> lk(g_tuned.mu);
  g_tuned.by_class.clear();
  g_tuned.any.store(false, std::memory_order_release);
}

int segsort_tune_lookup(int key_bytes, int64_t n, int32_t nseg, int64_t *radix_min,
                        int64_t *stream_max_avg, int32_t *merge_ctas_per_sm) {
  using namespace segsort;
  CallRoute R;
  if (!tuned_route(route_class(key_bytes, n, nseg), &R)) return 0;
  if (radix_min) *radix_min = R.radix_min;
  if (stream_max_avg) *stream_max_avg = R.stream_max_avg;
  if (merge_ctas_per_sm) *merge_ctas_per_sm = R.merge_per_sm;
  return 1;
}

int segsort_selftest_wait_timeout(int which) {
  using namespace segsort;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return SEGSORT_ERR_CUDA;
  cudaError_t e = cudaSuccess;
  switch (which) {
    case 0: {
      const uint32_t zero[kCtrWords] = {};
      e = cudaMemcpyToSymbolAsync(g_selftest_ctr, zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(selftest_barrier_kernel),
                                        dim3(2), dim3(32), nullptr, 0, st);
      break;
    }
    case 1:
      selftest_mbar_kernel<<<1, 32, 0, st>>>();
      e = cudaGetLastError();
      break;
    case 2: {
      static const unsigned long long zero[2 * kRBuckets] = {};
      e = cudaMemcpyToSymbolAsync(g_selftest_look, zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) {
        selftest_look_kernel<<<1, kRBuckets, 0, st>>>();
        e = cudaGetLastError();
      }
      break;
    }
    default:
      cudaStreamDestroy(st);
      return SEGSORT_ERR_INVALID_ARG;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return e == cudaSuccess ? SEGSORT_OK : SEGSORT_ERR_CUDA;
}

const char *segsort_error_string(int code) {
  switch (code) {
    case SEGSORT_OK: return "ok";
    case SEGSORT_ERR_INVALID_ARG: return "invalid argument";
    case SEGSORT_ERR_CUDA: return "CUDA runtime error";
    case SEGSORT_ERR_TIMEOUT: return "bounded device wait timed out";
    case SEGSORT_ERR_NO_MEMORY: return "workspace allocation failed";
    case SEGSORT_ERR_TOO_LARGE: return "problem exceeds the supported size";
    case SEGSORT_ERR_WORKSPACE: return "caller workspace too small or misaligned";
    default: return "unknown error";
  }
}

int segsort_version(void) { return 100; }

int segsort_profile_enable(int on) {
  segsort::g_prof_on.store(on != 0, std::memory_order_relaxed);
  return SEGSORT_OK;
}

int segsort_profile_read(double *tile_ms, double *large_ms, int64_t *tile_launches,
                         int64_t *large_launches, int reset) {
  using namespace segsort;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  int rc = SEGSORT_OK;
  auto span = [&](cudaEvent_t a, cudaEvent_t b) -> double {
    float ms = 0.f;
    if (a && b) {
      if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
        rc = SEGSORT_ERR_CUDA;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    return ms;
  };
  for (PhaseRecord &r : g_prof_pending) {
    g_prof_tile_ms += span(r.t0, r.t1);
    g_prof_tile_launches += r.tile_launches;
    if (r.l0 || r.l1) {
      g_prof_large_ms += span(r.l0, r.l1);
      g_prof_large_launches += r.large_launches;
    }
    if (r.m0 || r.m1) g_prof_large_ms += span(r.m0, r.m1);
  }
  g_prof_pending.clear();
  if (tile_ms) *tile_ms = g_prof_tile_ms;
  if (large_ms) *large_ms = g_prof_large_ms;
  if (tile_launches) *tile_launches = g_prof_tile_launches;
  if (large_launches) *large_launches = g_prof_large_launches;
  if (reset) {
    g_prof_tile_ms = g_prof_large_ms = 0.0;
    g_prof_tile_launches = g_prof_large_launches = 0;
  }
  return rc;
}

}  // extern "C"
