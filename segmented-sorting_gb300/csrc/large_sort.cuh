// Large-segment path: segments longer than the tile capacity are sorted by a
// least-significant-digit radix sort with 8-bit digits, one scatter pass per
// digit, in the "onesweep" style: one upfront pass computes every digit
// histogram of every large segment, and each scatter pass ranks a chunk of
// keys in shared memory and learns the chunk's global digit offsets from its
// predecessors in the same segment through decoupled look-back.
//
// Kernels, in stream order:
//   large_classify  list the segments longer than CAP, zero their histograms
//   large_scan      exclusive prefix of the chunk counts of listed segments
//   large_hist      per-chunk digit histograms -> per-segment histograms
//   large_pass x P  stable scatter of one digit (P = key bits / 8);
//                   keys/vals -> tmp -> keys/vals ... (P is even, so the
//                   result ends back in the caller's buffers)
//
// It replaces the reference's large-segment driver gen_grid_kern_r2049
// (src/bb_segsort/bb_comput_l.h:1155-1284: a 2048-key block sort followed by
// log2(len/2048) global merge passes, with several synchronous device-to-host
// copies) and CUB's one-CTA-per-segment radix sort
// (lib/cub/device/dispatch/dispatch_radix_sort.cuh:323).  Every wait on
// another CTA is bounded; a wait that gives up raises kStatusTimeout.
#pragma once

#include "segsort_common.cuh"

namespace segsort {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kPassThreads = 256;  // one thread per digit in the digit loops
constexpr int kPassWarps = kPassThreads / 32;

// Keys per thread and per chunk of a scatter pass: 4096 keys for 32-bit keys,
// 2048 for 64-bit keys (the staged chunk stays under 48 KB of shared memory).
template <typename K>
struct PassShape {
  static constexpr int kItems = sizeof(K) == 4 ? 16 : 8;
  static constexpr int kChunk = kPassThreads * kItems;
};

constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagInclusive = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr int kLookbackSpinLimit = 1 << 20;  // ~0.1 s with the back-off below

enum : int {
  kCtrLarge = 0,   // number of listed segments
  kCtrChunks = 1,  // total chunks over listed segments
  kCtrHist = 2,    // ticket counter of large_hist
  kCtrPass = 3,    // ticket counters of the passes: kCtrPass + pass
  kCtrWords = 16,
};

// Device views of the large-path workspace.
template <typename K>
struct LargeWs {
  uint32_t *ctr;          // [kCtrWords]
  int32_t *list;          // [max_large] listed segment ids
  int32_t *chunk_prefix;  // [max_large + 1]
  uint32_t *hist;         // [max_large][passes][kRadix]
  uint32_t *status;       // [max_chunks][passes][kRadix] look-back words
  K *tmp_keys;            // [n]
  uint32_t *tmp_vals;     // [n]
  int32_t max_large;
  int32_t passes;
  int64_t max_chunks;
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t *>(p) = v;
}

// ---------------------------------------------------------------------------
template <typename K>
__global__ void __launch_bounds__(256)
large_classify_kernel(Offsets off, int64_t cap, LargeWs<K> ws) {
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int64_t len = 0;
  if (s < off.nseg) len = off(s + 1) - off(s);
  const bool large = len > cap;
  const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, large);
  if (ballot == 0) return;
  uint32_t base = 0;
  if (lane == 0) base = atomicAdd(&ws.ctr[kCtrLarge], __popc(ballot));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  const uint32_t li = base + __popc(ballot & lanemask_lt());
  if (large && li < static_cast<uint32_t>(ws.max_large)) {
    ws.list[li] = static_cast<int32_t>(s);
    constexpr int kChunk = PassShape<K>::kChunk;
    ws.chunk_prefix[li] = static_cast<int32_t>((len + kChunk - 1) / kChunk);
  }
  // Zero the histograms of the listed segments, one warp per segment.
  const int words = ws.passes * kRadix;
  uint32_t pending = ballot;
  while (pending) {
    const int src = __ffs(pending) - 1;
    pending &= pending - 1;
    const uint32_t l = base + __popc(ballot & ((1u << src) - 1));
    if (l >= static_cast<uint32_t>(ws.max_large)) continue;
    uint4 *h = reinterpret_cast<uint4 *>(ws.hist + static_cast<size_t>(l) * words);
    for (int i = lane; i < words / 4; i += 32) h[i] = make_uint4(0, 0, 0, 0);
  }
}

// One CTA: exclusive prefix of the chunk counts, total into ctr[kCtrChunks].
// The prefix saturates at max_chunks (the size of the look-back array): with
// well-formed offsets the total never reaches it; with overlapping malformed
// segments the chunks past it are simply not sorted.
template <typename K>
__global__ void __launch_bounds__(1024) large_scan_kernel(LargeWs<K> ws) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint64_t carry_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t nl = ws.ctr[kCtrLarge];
  if (nl > static_cast<uint32_t>(ws.max_large)) nl = ws.max_large;
  const uint64_t cap = static_cast<uint64_t>(ws.max_chunks);
  if (tid == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < nl; base += 1024) {
    const uint32_t i = base + tid;
    const uint32_t v = i < nl ? static_cast<uint32_t>(ws.chunk_prefix[i]) : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warp_sums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      warp_sums[lane] = w;
    }
    __syncthreads();
    const uint64_t carry = carry_s;
    const uint64_t incl = static_cast<uint64_t>(x) + (warp ? warp_sums[warp - 1] : 0u) + carry;
    const uint64_t excl = incl - v;
    if (i < nl) ws.chunk_prefix[i] = static_cast<int32_t>(excl < cap ? excl : cap);
    __syncthreads();
    if (tid == 1023) carry_s = incl;
    __syncthreads();
  }
  if (tid == 0) {
    const uint64_t total = carry_s < cap ? carry_s : cap;
    ws.chunk_prefix[nl] = static_cast<int32_t>(total);
    ws.ctr[kCtrChunks] = static_cast<uint32_t>(total);
  }
}

// Map a chunk ticket to its listed segment: li with prefix[li] <= t < prefix[li+1].
__device__ __forceinline__ int32_t chunk_owner(const int32_t *prefix, int32_t nl, int64_t t) {
  int32_t lo = 0, hi = nl - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Upfront histograms of every digit position; zeroes the chunk's look-back
// words for every pass.
template <typename K>
__global__ void __launch_bounds__(kPassThreads)
large_hist_kernel(const K *__restrict__ keys, Offsets off, LargeWs<K> ws) {
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  constexpr int kMaxPasses = sizeof(Bits);
  constexpr int kChunk = PassShape<K>::kChunk;
  __shared__ uint32_t h[kMaxPasses * kRadix];
  __shared__ int64_t tk_s;
  const int tid = threadIdx.x;
  const int passes = ws.passes;
  const int32_t nl = min(static_cast<int32_t>(ws.ctr[kCtrLarge]), ws.max_large);
  const int64_t total = ws.ctr[kCtrChunks];
  while (true) {
    if (tid == 0) tk_s = atomicAdd(&ws.ctr[kCtrHist], 1u);
    for (int i = tid; i < passes * kRadix; i += kPassThreads) h[i] = 0;
    __syncthreads();
    const int64_t t = tk_s;
    if (t >= total) break;
    const int32_t li = chunk_owner(ws.chunk_prefix, nl, t);
    const int64_t c = t - ws.chunk_prefix[li];
    const int64_t s = ws.list[li];
    const int64_t b = off(s), e = off(s + 1);
    const int64_t cb = b + c * kChunk;
    const int64_t ce = min(cb + kChunk, e);
    for (int64_t p = cb + tid; p < ce; p += kPassThreads) {
      const Bits x = Ord::to_bits(keys[p]);
#pragma unroll
      for (int q = 0; q < kMaxPasses; ++q)
        atomicAdd(&h[q * kRadix + static_cast<int>((x >> (q * kRadixBits)) & (kRadix - 1))], 1u);
    }
    uint32_t *st = ws.status + static_cast<size_t>(t) * passes * kRadix;
    for (int i = tid; i < passes * kRadix; i += kPassThreads) st[i] = 0;
    __syncthreads();
    uint32_t *gh = ws.hist + static_cast<size_t>(li) * passes * kRadix;
    for (int i = tid; i < passes * kRadix; i += kPassThreads) {
      const uint32_t v = h[i];
      if (v) atomicAdd(&gh[i], v);
    }
    __syncthreads();
  }
}

// Block-wide exclusive scan of one value per thread (kPassThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_tmp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tmp[warp] = x;
  __syncthreads();
  uint32_t wsum = 0;
#pragma unroll
  for (int w = 0; w < kPassWarps; ++w) wsum += (w < warp) ? warp_tmp[w] : 0u;
  __syncthreads();
  return wsum + x - v;
}

// ---------------------------------------------------------------------------
// One stable scatter pass over digit `pass` of every chunk of every listed
// segment.  Chunk tickets are taken in launch order with an atomic counter,
// so a chunk's predecessors in its segment already hold tickets (they are
// resident or finished) when it looks back at them.
template <typename K, bool PAIRS>
__global__ void __launch_bounds__(kPassThreads)
large_pass_kernel(const K *__restrict__ src_keys, const uint32_t *__restrict__ src_vals,
                  K *__restrict__ dst_keys, uint32_t *__restrict__ dst_vals, Offsets off,
                  LargeWs<K> ws, int pass) {
  using Ord = KeyOrder<K>;
  constexpr int kPassItems = PassShape<K>::kItems;
  constexpr int kChunk = PassShape<K>::kChunk;
  __shared__ uint32_t whist[kPassWarps * kRadix];  // per-warp digit counts, then prefixes
  __shared__ int32_t delta_s[kRadix];              // dst index - staged index, per digit
  __shared__ uint32_t boff_s[kRadix];              // chunk-local digit offsets
  __shared__ uint32_t warp_tmp[kPassWarps];
  __shared__ int64_t tk_s;
  __shared__ K ks[kChunk];
  __shared__ uint32_t vs[PAIRS ? kChunk : 1];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int shift = pass * kRadixBits;
  const int passes = ws.passes;
  const int32_t nl = min(static_cast<int32_t>(ws.ctr[kCtrLarge]), ws.max_large);
  const int64_t total = ws.ctr[kCtrChunks];
  const uint32_t lt = lanemask_lt();

  while (true) {
    if (tid == 0) tk_s = atomicAdd(&ws.ctr[kCtrPass + pass], 1u);
    for (int i = tid; i < kPassWarps * kRadix; i += kPassThreads) whist[i] = 0;
    __syncthreads();
    const int64_t t = tk_s;
    if (t >= total) break;
    const int32_t li = chunk_owner(ws.chunk_prefix, nl, t);
    const int64_t c = t - ws.chunk_prefix[li];
    const int64_t s = ws.list[li];
    const int64_t b = off(s), e = off(s + 1);
    const int64_t cb = b + c * kChunk;
    const int clen = static_cast<int>(min(static_cast<int64_t>(kChunk), e - cb));

    // ---- load (warp-striped) and rank within each warp, in input order ----
    K kv[kPassItems];
    uint32_t vv[kPassItems];
    uint32_t rank[kPassItems];
    const int wbase = warp * (kPassItems * 32);
#pragma unroll
    for (int j = 0; j < kPassItems; ++j) {
      const int i = wbase + j * 32 + lane;
      if (i < clen) {
        kv[j] = src_keys[cb + i];
        if constexpr (PAIRS) vv[j] = src_vals[cb + i];
      }
    }
#pragma unroll
    for (int j = 0; j < kPassItems; ++j) {
      const int i = wbase + j * 32 + lane;
      const bool valid = i < clen;
      const uint32_t d = valid ? static_cast<uint32_t>((Ord::to_bits(kv[j]) >> shift) & (kRadix - 1))
                               : static_cast<uint32_t>(kRadix);
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
      uint32_t before = 0;
      if (valid) before = whist[warp * kRadix + d];
      __syncwarp();
      if (valid && lane == 31 - __clz(peers)) whist[warp * kRadix + d] = before + __popc(peers);
      __syncwarp();
      rank[j] = before + __popc(peers & lt);
    }
    __syncthreads();

    // ---- per digit: warp prefixes, chunk total, look-back ------------------
    const int d = tid;  // kPassThreads == kRadix
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kPassWarps; ++w) {
      const uint32_t x = whist[w * kRadix + d];
      whist[w * kRadix + d] = tot;
      tot += x;
    }
    uint32_t *st = ws.status + static_cast<size_t>(t) * passes * kRadix + pass * kRadix;
    uint32_t excl = 0;
    if (c == 0) {
      st_volatile(st + d, kFlagInclusive | tot);
    } else {
      st_volatile(st + d, kFlagAggregate | tot);
      const int64_t q_first = t - c;  // the segment's first chunk (always inclusive)
      int64_t q = t - 1;
      while (true) {
        if (q < q_first) {  // unreachable: chunk q_first publishes an inclusive value
          raise_status(kStatusTimeout);
          break;
        }
        const uint32_t *qs = ws.status + static_cast<size_t>(q) * passes * kRadix + pass * kRadix;
        uint32_t v = ld_volatile(qs + d);
        int spins = 0;
        while ((v >> 30) == 0 && spins < kLookbackSpinLimit) {
          if (spins > 64) __nanosleep(64);
          ++spins;
          v = ld_volatile(qs + d);
        }
        if ((v >> 30) == 0) {
          raise_status(kStatusTimeout);
          break;
        }
        excl += v & kValueMask;
        if (v & kFlagInclusive) break;
        --q;
      }
      st_volatile(st + d, kFlagInclusive | ((excl + tot) & kValueMask));
    }
    const uint32_t boff = block_exclusive_scan(tot, warp_tmp);
    const uint32_t hcount = ws.hist[static_cast<size_t>(li) * passes * kRadix + pass * kRadix + d];
    const uint32_t dbase = block_exclusive_scan(hcount, warp_tmp);
    boff_s[d] = boff;
    delta_s[d] = static_cast<int32_t>(dbase + excl) - static_cast<int32_t>(boff);
    __syncthreads();

    // ---- scatter into shared memory in sorted-chunk order -------------------
#pragma unroll
    for (int j = 0; j < kPassItems; ++j) {
      const int i = wbase + j * 32 + lane;
      if (i < clen) {
        const uint32_t dg = static_cast<uint32_t>((Ord::to_bits(kv[j]) >> shift) & (kRadix - 1));
        const uint32_t pos = boff_s[dg] + whist[warp * kRadix + dg] + rank[j];
        ks[pos] = kv[j];
        if constexpr (PAIRS) vs[pos] = vv[j];
      }
    }
    __syncthreads();

    // ---- write runs of equal digits to their global positions --------------
    for (int i = tid; i < clen; i += kPassThreads) {
      const K k = ks[i];
      const uint32_t dg = static_cast<uint32_t>((Ord::to_bits(k) >> shift) & (kRadix - 1));
      const int64_t dst = b + i + delta_s[dg];
      // Always inside [b, e) for well-formed offsets; the check keeps
      // overlapping malformed segments from writing outside their range.
      if (dst >= b && dst < e) {
        dst_keys[dst] = k;
        if constexpr (PAIRS) dst_vals[dst] = vs[i];
      }
    }
    __syncthreads();
  }
}

}  // namespace segsort
