// Batched form of the segmented sort: segsort_pairs_batch and batch plans.
//
// The instances of a batch are grouped by key type.  A group is sorted by the
// same three kernels as one plain call -- classify, the tile sort, the
// cooperative long-segment kernel (radix passes, then merge passes) --
// launched once for the whole group: every kernel finds an instance through a device table (BatchInst),
// tile-sort CTAs and classify warps by binary search over the instances'
// bases, and long-segment jobs through the instance index they carry.  Small instances
// therefore share CTAs' worth of work with large ones instead of paying a
// sequence of launches and grid barriers each.
//
// A plan fixes the items, allocates one buffer for every group's table and
// workspace, and captures the launches into CUDA graphs, one per launch
// shape of the merge passes; a launch replays the chosen graph.  The tuner
// measures the shapes on the plan's own data and caches the fastest per
// class of batch (key types, sizes and mean segment length) in a file.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_host.cuh"

namespace segsort {
namespace {

constexpr int kKeyTypes = 4;
constexpr int64_t kGroupMaxN = (int64_t{1} << 31) - 1;

// Instances of one key type, placed in the batch-wide arrays.
struct Group {
  int key_type = 0;
  std::vector<BatchInst> insts;  // non-empty instances only
  int64_t total_n = 0, tiles = 0, half_entries = 0;
  WsLayout L;
  size_t tab_off = 0;  // table position in the batch buffer
  size_t ws_off = 0;   // workspace position in the batch buffer
  // MSD route (msd_route.cuh): its stage-2 table and the expansion's arrays.
  bool msd = false;
  int64_t lsd_min = 0;        // the radix threshold of stage 2
  int64_t msd_entries = 0;    // expansion entries: sum over instances of c_len + 1
  std::vector<int64_t> c_len; // per instance: its padded stage-2 segment count
  size_t tab2_off = 0, sub_off = 0, flags_off = 0, rank_off = 0;
};

// The stage-2 table of an MSD group: every instance with its expanded
// offsets and flags (pointers into the batch buffer at buf).
std::vector<BatchInst> stage2_table(const Group &G, unsigned char *buf) {
  std::vector<BatchInst> t = G.insts;
  int32_t *sub = reinterpret_cast<int32_t *>(buf + G.sub_off);
  uint8_t *flags = reinterpret_cast<uint8_t *>(buf + G.flags_off);
  for (size_t i = 0; i < t.size(); ++i) {
    t[i].offsets = sub + t[i].msd_base;
    t[i].flags = flags + t[i].msd_base;
    t[i].nseg = static_cast<int32_t>(G.c_len[i]);
    t[i].heads = 0;
  }
  return t;
}

struct BatchLayout {
  std::vector<Group> groups;
  size_t total = 0;
};

int key_bytes_of(int type) { return type == SEGSORT_KEY_U64 ? 8 : 4; }

int64_t cap_of(int type) {
  return type == SEGSORT_KEY_U64 ? tile_cap<uint64_t>() : tile_cap<uint32_t>();
}

int64_t item_of(int type) {
  return type == SEGSORT_KEY_U64 ? MergeShape<uint64_t>::T : MergeShape<uint32_t>::T;
}

int64_t radix_min_of(int type) {
  return type == SEGSORT_KEY_U64 ? radix_min_for<uint64_t>() : radix_min_for<uint32_t>();
}

int64_t msd_min_of(int type) {
  return type == SEGSORT_KEY_U64 ? msd_min_for<uint64_t>(radix_min_for<uint64_t>())
                                 : msd_min_for<uint32_t>(radix_min_for<uint32_t>());
}

// Validates the items and lays out every group.  Empty items (n == 0 or
// nseg == 0) have nothing to sort and are left out.
int build_layout(const segsort_batch_item *items, int32_t count, BatchLayout &B) {
  if (count < 0 || (count > 0 && items == nullptr)) return SEGSORT_ERR_INVALID_ARG;
  Group g[kKeyTypes];
  for (int t = 0; t < kKeyTypes; ++t) g[t].key_type = t;
  for (int32_t i = 0; i < count; ++i) {
    const segsort_batch_item &it = items[i];
    if (it.key_type < 0 || it.key_type >= kKeyTypes) return SEGSORT_ERR_INVALID_ARG;
    if (it.n < 0 || it.nseg < 0 || (it.heads != 0 && it.heads != 1)) return SEGSORT_ERR_INVALID_ARG;
    if (it.n == 0 || it.nseg == 0) continue;
    if (it.d_keys == nullptr || it.d_vals == nullptr || it.d_offsets == nullptr)
      return SEGSORT_ERR_INVALID_ARG;
    if (it.n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
    Group &G = g[it.key_type];
    const int64_t cap = cap_of(it.key_type);
    const int64_t tiles = (it.n + cap - 1) / cap;
    BatchInst I{};
    I.keys = it.d_keys;
    I.vals = it.d_vals;
    I.offsets = it.d_offsets;
    I.n = it.n;
    I.nseg = it.nseg;
    I.heads = it.heads;
    I.tmp_base = G.total_n;
    I.half_base = G.half_entries;
    I.tile_base = G.tiles;
    G.insts.push_back(I);
    G.total_n += it.n;
    G.half_entries += 2 * tiles + 1;
    G.tiles += tiles;
    if (G.total_n > kGroupMaxN) return SEGSORT_ERR_TOO_LARGE;
  }
  size_t off = 0;
  const bool msd_on = g_msd_on.load(std::memory_order_relaxed) != 0;
  for (int t = 0; t < kKeyTypes; ++t) {
    Group &G = g[t];
    if (G.insts.empty()) continue;
    // The MSD route for a group of 64-bit keys when an instance may hold a
    // segment above its threshold.  (Measured on the 64-instance benchmark
    // batch: the u64 group 3.13 -> 2.59 ms; the u32 and f32 groups, whose
    // long segments take four LSD passes, 1.38 -> 1.55 and 2.00 -> 2.18 ms,
    // the second stage's classify and expansion over all their instances
    // costing more than the passes saved.)
    const int64_t msd_min = msd_min_of(t);
    G.lsd_min = radix_min_of(t);
    if (key_bytes_of(t) == 8)
      for (const BatchInst &I : G.insts) G.msd = G.msd || (msd_on && I.n > msd_min);
    G.L = make_layout(G.total_n, key_bytes_of(t), 4, cap_of(t), item_of(t), G.half_entries,
                      G.msd ? std::min(msd_min, G.lsd_min) : G.lsd_min);
    G.tab_off = off;
    off = align256(off + G.insts.size() * sizeof(BatchInst));
    G.ws_off = off;
    off = align256(off + G.L.total);
    if (G.msd) {
      for (BatchInst &I : G.insts) {
        const int64_t c = msd_stage2_segments(I.nseg, I.n / (msd_min + 1) + 1);
        if (c >= (int64_t{1} << 31)) return SEGSORT_ERR_TOO_LARGE;
        I.msd_base = G.msd_entries;
        G.c_len.push_back(c);
        G.msd_entries += c + 1;
      }
      G.tab2_off = off;
      off = align256(off + G.insts.size() * sizeof(BatchInst));
      G.sub_off = off;
      off = align256(off + static_cast<size_t>(G.msd_entries) * 4);
      G.flags_off = off;
      off = align256(off + static_cast<size_t>(G.msd_entries));
      G.rank_off = off;
      off = align256(off + 4 * (static_cast<size_t>(G.L.max_rjobs) + 1) * 4);
    }
    B.groups.push_back(std::move(G));
  }
  B.total = off;
  return SEGSORT_OK;
}

// ---------------------------------------------------------------------------
// Table upload without host synchronisation: the entries travel as kernel
// parameters (one launch per block of kUploadBlock entries), so the host
// array may be freed as soon as the launch returns.
constexpr int kUploadBlock = 44;  // 44 * 88 bytes: inside the 4 KB parameter space
struct UploadBlock {
  BatchInst v[kUploadBlock];
  int32_t count;
};
static_assert(sizeof(UploadBlock) <= 4096, "kernel parameters must fit 4 KB");

__global__ void upload_insts_kernel(UploadBlock blk, BatchInst *dst) {
  if (static_cast<int32_t>(threadIdx.x) < blk.count) dst[threadIdx.x] = blk.v[threadIdx.x];
}

cudaError_t upload_table(const std::vector<BatchInst> &v, BatchInst *dst, cudaStream_t stream) {
  for (size_t i = 0; i < v.size(); i += kUploadBlock) {
    UploadBlock blk;
    std::memset(&blk, 0, sizeof(blk));
    blk.count = static_cast<int32_t>(std::min<size_t>(kUploadBlock, v.size() - i));
    std::copy(v.begin() + i, v.begin() + i + blk.count, blk.v);
    upload_insts_kernel<<<1, kUploadBlock, 0, stream>>>(blk, dst + i);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Kernels of one key type, their one-time attributes and launch shapes.
template <typename K>
struct BatchKernels {
  using TCfg = typename TileFor<K, true>::Cfg;
  using BF = BucketFor<K, true>;
  using BCfg = typename BF::Cfg;
  using MS = LongSmem<K, true>;
  static constexpr size_t kBSmem = BucketLayout<BCfg, true>::kBytes;
  // The tile sort: the bucket route (bucket kernel, then the comparison sort
  // of the chunks it lists), as plain calls of segments of 128 keys or more.
  static constexpr auto bucket = tile_bucket_batch_kernel<K, true, BCfg::NT, BCfg::KPT,
                                                          BF::kMinBlocks>;
  static constexpr auto list = tile_list_batch_kernel<K, true, TCfg::NT, TCfg::KPT,
                                                      TileFor<K, true>::kMinBlocks>;
  static constexpr auto merge = long_segment_kernel<K, true, BatchSpace<K>>;
  static constexpr auto classify = large_classify_halves_batch_kernel<K>;
  static inline std::atomic<uint64_t> bucket_attr{0}, list_attr{0}, merge_attr{0};
  static inline std::atomic<int> merge_occ[kMaxDevices], list_occ[kMaxDevices];

  // Attributes and occupancy, before any capture.
  static cudaError_t prepare(int dev) {
    cudaError_t e = ensure_smem(bucket, kBSmem, bucket_attr, dev);
    if (e == cudaSuccess) e = ensure_smem(list, TCfg::kSmemBytes, list_attr, dev);
    if (e == cudaSuccess) e = ensure_smem(merge, MS::kBytes, merge_attr, dev);
    if (e == cudaSuccess) occupancy(merge, kMThreads, MS::kBytes, merge_occ, dev);
    if (e == cudaSuccess) occupancy(list, TCfg::NT, TCfg::kSmemBytes, list_occ, dev);
    return e;
  }

  static int enqueue(const Group &G, unsigned char *buf, const DeviceState &S, int dev,
                     cudaStream_t stream, int merge_per_sm) {
    const BatchInst *tab = reinterpret_cast<const BatchInst *>(buf + G.tab_off);
    // The tables stage 2 reads: the expanded offsets of an MSD group.
    const BatchInst *tab2 =
        G.msd ? reinterpret_cast<const BatchInst *>(buf + G.tab2_off) : tab;
    const int32_t count = static_cast<int32_t>(G.insts.size());
    LargeWs<K> W = ws_views<K, true>(buf + G.ws_off, G.L);
    W.lsd_min = G.lsd_min;
    const int64_t cap = tile_cap<K>();
    const unsigned cls_blocks =
        static_cast<unsigned>((G.half_entries + kClassifyWarps - 1) / kClassifyWarps);
    auto classify_on = [&](const BatchInst *t, const LargeWs<K> &w) {
      if (cudaMemsetAsync(W.ctr, 0, kCtrWords * sizeof(uint32_t), stream) != cudaSuccess)
        return false;
      classify<<<cls_blocks, (kClassifyWarps + 1) * 32, 0, stream>>>(t, count, G.half_entries,
                                                                     cap, cap / 2, w);
      return cudaGetLastError() == cudaSuccess;
    };
    const int mo = occupancy(merge, kMThreads, MS::kBytes, merge_occ, dev);
    const int64_t items = G.total_n / MergeShape<K>::T + 1;
    const int per_sm = merge_per_sm > 0 ? std::min(merge_per_sm, mo) : mo;
    const unsigned grid =
        static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(per_sm) * S.sms, items));
    auto launch_long = [&](const BatchInst *t, LargeWs<K> w) {
      BatchSpace<K> sp{t, W.tmp_keys, W.tmp_vals};
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid);
      cfg.blockDim = dim3(kMThreads);
      cfg.dynamicSmemBytes = MS::kBytes;
      cfg.stream = stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      return cudaLaunchKernelEx(&cfg, merge, sp, w, cap) == cudaSuccess;
    };

    if (G.msd) {
      // ---- MSD route, stage 1: the radix segments above the MSD threshold
      // (one pass on the top varying digit, or all their LSD passes, or none
      // for those left to stage 2), then the expanded offsets -------------------
      LargeWs<K> W1 = W;  // radix_min: the layout's, the MSD threshold
      W1.msd_stage = 1;
      if (!classify_on(tab, W1) || !launch_long(tab, W1)) return SEGSORT_ERR_CUDA;
      const size_t rj = static_cast<size_t>(G.L.max_rjobs) + 1;
      int32_t *rk = reinterpret_cast<int32_t *>(buf + G.rank_off);
      MsdBatchWs M{rk, rk + rj, rk + 2 * rj, rk + 3 * rj};
      msd_rank_batch_kernel<K><<<static_cast<unsigned>((G.L.max_rjobs + 255) / 256), 256, 0,
                                 stream>>>(W1, M);
      msd_expand_batch_kernel<K><<<static_cast<unsigned>((G.msd_entries + 255) / 256), 256, 0,
                                   stream>>>(tab, tab2, count, G.msd_entries, W1, M);
      msd_sub_batch_kernel<K><<<static_cast<unsigned>(G.L.max_rjobs), kRBuckets, 0, stream>>>(
          tab2, W1, M);
      if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
    }
    LargeWs<K> W2 = W;
    W2.radix_min = std::max<int64_t>(G.lsd_min, W.radix_min);
    if (!classify_on(tab2, W2)) return SEGSORT_ERR_CUDA;

    // Tile sort first: it forms the sorted runs the merge passes read (the
    // radix passes read the caller's buffers, which it leaves alone).
    bucket<<<static_cast<unsigned>(G.tiles), BCfg::NT, kBSmem, stream>>>(
        tab2, count, W2.half_first, W2.tmp_keys, W2.tmp_vals, W2.radix_min, W2.fallback,
        W2.ctr + kCtrFallback, W2.max_fallback);
    if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
    const int lo = occupancy(list, TCfg::NT, TCfg::kSmemBytes, list_occ, dev);
    const unsigned lgrid =
        static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(lo) * S.sms, G.tiles));
    list<<<lgrid, TCfg::NT, TCfg::kSmemBytes, stream>>>(tab2, W2.tmp_keys, W2.tmp_vals,
                                                      W2.fallback, W2.ctr + kCtrFallback,
                                                      W2.max_fallback, W2.ctr + kCtrListTicket);
    if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
    if (!launch_long(tab2, W2)) return SEGSORT_ERR_CUDA;
    return SEGSORT_OK;
  }
};

cudaError_t prepare_group(const Group &G, int dev) {
  switch (G.key_type) {
    case SEGSORT_KEY_U32: return BatchKernels<uint32_t>::prepare(dev);
    case SEGSORT_KEY_I32: return BatchKernels<int32_t>::prepare(dev);
    case SEGSORT_KEY_F32: return BatchKernels<float>::prepare(dev);
    default: return BatchKernels<uint64_t>::prepare(dev);
  }
}

int enqueue_group(const Group &G, unsigned char *buf, const DeviceState &S, int dev,
                  cudaStream_t stream, int merge_per_sm) {
  switch (G.key_type) {
    case SEGSORT_KEY_U32: return BatchKernels<uint32_t>::enqueue(G, buf, S, dev, stream, merge_per_sm);
    case SEGSORT_KEY_I32: return BatchKernels<int32_t>::enqueue(G, buf, S, dev, stream, merge_per_sm);
    case SEGSORT_KEY_F32: return BatchKernels<float>::enqueue(G, buf, S, dev, stream, merge_per_sm);
    default: return BatchKernels<uint64_t>::enqueue(G, buf, S, dev, stream, merge_per_sm);
  }
}

int prepare_all(const BatchLayout &B, int dev) {
  for (const Group &G : B.groups)
    if (prepare_group(G, dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  return SEGSORT_OK;
}

// merge_per_sm: resident merge-pass CTAs per SM (0: as many as fit).
int enqueue_all(const BatchLayout &B, unsigned char *buf, const DeviceState &S, int dev,
                cudaStream_t stream, int merge_per_sm = 0) {
  for (const Group &G : B.groups) {
    const int rc = enqueue_group(G, buf, S, dev, stream, merge_per_sm);
    if (rc != SEGSORT_OK) return rc;
  }
  return SEGSORT_OK;
}

// Class of a batch for the autotuner's cache: the key types present and the
// log2 buckets of the total keys, the largest item and the key-weighted mean
// segment length (n / nseg of each item, known on the host).
std::string batch_class(const segsort_batch_item *items, int32_t count) {
  int64_t total = 0, largest = 0;
  double weighted = 0.0;
  unsigned types = 0;
  for (int32_t i = 0; i < count; ++i) {
    const segsort_batch_item &it = items[i];
    if (it.n <= 0 || it.nseg <= 0) continue;
    total += it.n;
    largest = std::max<int64_t>(largest, it.n);
    weighted += static_cast<double>(it.n) * (static_cast<double>(it.n) / it.nseg);
    types |= 1u << it.key_type;
  }
  auto lg = [](double x) { return x >= 1.0 ? static_cast<int>(std::floor(std::log2(x))) : 0; };
  char buf[96];
  std::snprintf(buf, sizeof(buf), "t%u-n%d-max%d-len%d", types, lg(static_cast<double>(total)),
                lg(static_cast<double>(largest)), lg(total > 0 ? weighted / total : 0.0));
  return buf;
}

int current_device(int *dev, DeviceState **S) {
  if (cudaGetDevice(dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  *S = device_state(*dev);
  if (*S == nullptr || !(*S)->coop) return SEGSORT_ERR_CUDA;
  return SEGSORT_OK;
}

}  // namespace

cudaError_t batch_device_status(bool clear, uint32_t *value) {
  cudaError_t e = cudaMemcpyFromSymbol(value, g_device_status, sizeof(uint32_t));
  if (e == cudaSuccess && clear) {
    const uint32_t zero = 0;
    e = cudaMemcpyToSymbol(g_device_status, &zero, sizeof(zero));
  }
  return e;
}

}  // namespace segsort

// A plan holds one captured graph per launch shape of the merge passes (1, 2
// or 3 resident CTAs per SM); `choice` is the one launches replay.
constexpr int kPlanShapes = 3;

struct segsort_batch_plan_s {
  int dev = 0;
  void *buf = nullptr;
  size_t bytes = 0;
  cudaGraph_t graph[kPlanShapes] = {};
  cudaGraphExec_t exec[kPlanShapes] = {};
  int choice = kPlanShapes - 1;
  bool empty = false;
  std::string cls;
};

extern "C" {

int segsort_pairs_batch(const segsort_batch_item *items, int32_t count, segsort_stream_t s) {
  using namespace segsort;
  const cudaStream_t stream = reinterpret_cast<cudaStream_t>(s);
  BatchLayout B;
  int rc = build_layout(items, count, B);
  if (rc != SEGSORT_OK || B.groups.empty()) return rc;
  int dev = 0;
  DeviceState *S = nullptr;
  if ((rc = current_device(&dev, &S)) != SEGSORT_OK) return rc;
  if ((rc = prepare_all(B, dev)) != SEGSORT_OK) return rc;
  cudaMemPool_t pool = device_pool(*S, dev);
  unsigned char *buf = nullptr;
  if (pool == nullptr ||
      cudaMallocFromPoolAsync(reinterpret_cast<void **>(&buf), B.total, pool, stream) !=
          cudaSuccess) {
    cudaGetLastError();
    return SEGSORT_ERR_NO_MEMORY;
  }
  for (const Group &G : B.groups) {
    if (upload_table(G.insts, reinterpret_cast<BatchInst *>(buf + G.tab_off), stream) !=
            cudaSuccess ||
        (G.msd && upload_table(stage2_table(G, buf), reinterpret_cast<BatchInst *>(buf + G.tab2_off),
                               stream) != cudaSuccess)) {
      rc = SEGSORT_ERR_CUDA;
      break;
    }
  }
  if (rc == SEGSORT_OK) rc = enqueue_all(B, buf, *S, dev, stream);
  if (cudaFreeAsync(buf, stream) != cudaSuccess && rc == SEGSORT_OK) rc = SEGSORT_ERR_CUDA;
  return rc;
}

int segsort_batch_plan_create(const segsort_batch_item *items, int32_t count,
                              segsort_batch_plan *plan) {
  using namespace segsort;
  if (plan == nullptr) return SEGSORT_ERR_INVALID_ARG;
  *plan = nullptr;
  BatchLayout B;
  int rc = build_layout(items, count, B);
  if (rc != SEGSORT_OK) return rc;
  int dev = 0;
  DeviceState *S = nullptr;
  if ((rc = current_device(&dev, &S)) != SEGSORT_OK) return rc;
  if ((rc = prepare_all(B, dev)) != SEGSORT_OK) return rc;

  segsort_batch_plan_s *P = new (std::nothrow) segsort_batch_plan_s;
  if (P == nullptr) return SEGSORT_ERR_NO_MEMORY;
  P->dev = dev;
  P->bytes = B.total;
  cudaStream_t cs = nullptr;
  do {
    if (B.total > 0 && cudaMalloc(&P->buf, B.total) != cudaSuccess) {
      cudaGetLastError();
      rc = SEGSORT_ERR_NO_MEMORY;
      break;
    }
    unsigned char *buf = static_cast<unsigned char *>(P->buf);
    for (const Group &G : B.groups) {
      if (cudaMemcpy(buf + G.tab_off, G.insts.data(), G.insts.size() * sizeof(BatchInst),
                     cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      if (G.msd) {
        const std::vector<BatchInst> t2 = stage2_table(G, buf);
        if (cudaMemcpy(buf + G.tab2_off, t2.data(), t2.size() * sizeof(BatchInst),
                       cudaMemcpyHostToDevice) != cudaSuccess) {
          rc = SEGSORT_ERR_CUDA;
          break;
        }
      }
    }
    if (rc != SEGSORT_OK) break;
    P->empty = B.groups.empty();
    P->cls = batch_class(items, count);
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
      rc = SEGSORT_ERR_CUDA;
      break;
    }
    for (int k = 0; k < kPlanShapes && rc == SEGSORT_OK; ++k) {
      if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      rc = enqueue_all(B, buf, *S, dev, cs, k + 1);
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      if (rc == SEGSORT_OK && ce != cudaSuccess) rc = SEGSORT_ERR_CUDA;
      P->graph[k] = graph;
      if (rc == SEGSORT_OK && cudaGraphInstantiate(&P->exec[k], P->graph[k], 0) != cudaSuccess)
        rc = SEGSORT_ERR_CUDA;
    }
  } while (false);
  if (cs != nullptr) cudaStreamDestroy(cs);
  if (rc != SEGSORT_OK) {
    cudaGetLastError();
    segsort_batch_plan_destroy(P);
    return rc;
  }
  *plan = P;
  return SEGSORT_OK;
}

int segsort_batch_plan_launch(segsort_batch_plan plan, segsort_stream_t s) {
  if (plan == nullptr) return SEGSORT_ERR_INVALID_ARG;
  if (plan->empty) return SEGSORT_OK;  // nothing to sort
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != plan->dev) return SEGSORT_ERR_INVALID_ARG;
  return cudaGraphLaunch(plan->exec[plan->choice], reinterpret_cast<cudaStream_t>(s)) ==
                 cudaSuccess
             ? SEGSORT_OK
             : SEGSORT_ERR_CUDA;
}

int segsort_batch_plan_tune(segsort_batch_plan plan, segsort_stream_t s, const char *cache_path,
                            int32_t *ctas_per_sm) {
  if (plan == nullptr) return SEGSORT_ERR_INVALID_ARG;
  auto done = [&](int rc) {
    if (ctas_per_sm) *ctas_per_sm = plan->choice + 1;
    return rc;
  };
  if (plan->empty) return done(SEGSORT_OK);
  // A cached choice for this class of batch.
  if (cache_path != nullptr) {
    if (FILE *f = std::fopen(cache_path, "r")) {
      char cls[128];
      int k = 0;
      bool found = false;
      while (std::fscanf(f, "%127s %d", cls, &k) == 2) {
        if (plan->cls == cls && k >= 1 && k <= kPlanShapes) {
          plan->choice = k - 1;
          found = true;
        }
      }
      std::fclose(f);
      if (found) return done(SEGSORT_OK);
    }
  }
  // Measure every shape: one warm-up replay, then the median of three.
  const cudaStream_t stream = reinterpret_cast<cudaStream_t>(s);
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return SEGSORT_ERR_CUDA;
  }
  int rc = SEGSORT_OK;
  float best = 0.f;
  int best_k = plan->choice;
  for (int k = 0; k < kPlanShapes && rc == SEGSORT_OK; ++k) {
    float t[3];
    for (int r = -1; r < 3 && rc == SEGSORT_OK; ++r) {
      if (cudaEventRecord(a, stream) != cudaSuccess || cudaGraphLaunch(plan->exec[k], stream) != cudaSuccess ||
          cudaEventRecord(b, stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
        rc = SEGSORT_ERR_CUDA;
        break;
      }
      if (r >= 0) cudaEventElapsedTime(&t[r], a, b);
    }
    if (rc != SEGSORT_OK) break;
    std::sort(t, t + 3);
    if (k == 0 || t[1] < best) {
      best = t[1];
      best_k = k;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != SEGSORT_OK) return done(rc);
  plan->choice = best_k;
  if (cache_path != nullptr) {
    if (FILE *f = std::fopen(cache_path, "a")) {
      std::fprintf(f, "%s %d\n", plan->cls.c_str(), best_k + 1);
      std::fclose(f);
    }
  }
  return done(SEGSORT_OK);
}

size_t segsort_batch_plan_workspace_bytes(segsort_batch_plan plan) {
  return plan == nullptr ? 0 : plan->bytes;
}

void segsort_batch_plan_destroy(segsort_batch_plan plan) {
  if (plan == nullptr) return;
  for (int k = 0; k < kPlanShapes; ++k) {
    if (plan->exec[k]) cudaGraphExecDestroy(plan->exec[k]);
    if (plan->graph[k]) cudaGraphDestroy(plan->graph[k]);
  }
  if (plan->buf) cudaFree(plan->buf);
  delete plan;
}

}  // extern "C"

extern "C" size_t segsort_batch_workspace_bytes(const segsort_batch_item *items, int32_t count) {
  segsort::BatchLayout B;
  if (segsort::build_layout(items, count, B) != SEGSORT_OK) return 0;
  return B.total;
}
