// Extensions around the plain sort: descending order, segmented top-k and
// 64-bit values.  Each one is the plain sort of segsort_api.cu plus short
// element-wise kernels on the same stream:
//   descending  keys are mapped in place to the complement of their order
//               bits, sorted ascending as unsigned integers (equal keys keep
//               their input order), and mapped back;
//   top-k       the sorted segments' first k elements are gathered into a
//               [nseg][k] output;
//   64-bit values  the keys are sorted with their positions as 32-bit values
//               and the 64-bit values are gathered through those positions.
#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_host.cuh"

namespace segsort {
namespace {

constexpr int kEwThreads = 256;

unsigned ew_blocks(int64_t n) { return static_cast<unsigned>((n + kEwThreads - 1) / kEwThreads); }

// keys[i] <- bits of ~order_bits(keys[i]) (forward) or back (inverse).  The
// map is a bijection, so elements outside every segment come back unchanged.
template <typename K, bool INVERSE>
__global__ void __launch_bounds__(kEwThreads) desc_map_kernel(K *keys, int64_t n) {
  using Ord = KeyOrder<K>;
  using Bits = typename Ord::Bits;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Bits *b = reinterpret_cast<Bits *>(keys) + i;
  if constexpr (INVERSE) {
    keys[i] = Ord::from_bits(static_cast<Bits>(~*b));
  } else {
    *b = static_cast<Bits>(~Ord::to_bits(keys[i]));
  }
}

__global__ void __launch_bounds__(kEwThreads) iota_kernel(uint32_t *v, int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) v[i] = static_cast<uint32_t>(i);
}

__global__ void __launch_bounds__(kEwThreads)
gather64_kernel(uint64_t *dst, const uint64_t *src, const uint32_t *idx, int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

// Output slot (s, j) of the [nseg][k] top-k matrix.
template <typename K>
__global__ void __launch_bounds__(kEwThreads)
topk_gather_kernel(const K *keys, const uint32_t *vals, Offsets off, int64_t k, K *out_keys,
                   uint32_t *out_vals, int32_t *out_counts) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= off.nseg * k) return;
  const int64_t s = t / k, j = t - s * k;
  const int64_t b = off(s), e = off(s + 1);
  const int64_t len = e > b ? e - b : 0;
  if (j == 0 && out_counts) out_counts[s] = static_cast<int32_t>(len < k ? len : k);
  if (j < len) {
    out_keys[t] = keys[b + j];
    if (out_vals) out_vals[t] = vals[b + j];
  }
}

// The plain call for key type K (vals null: keys only).
template <typename K>
int sort_typed(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg,
               cudaStream_t s) {
  segsort_stream_t st = reinterpret_cast<segsort_stream_t>(s);
  if constexpr (std::is_same_v<K, uint32_t>) {
    return vals ? segsort_pairs_u32(keys, vals, n, off, nseg, st) : segsort_keys_u32(keys, n, off, nseg, st);
  } else if constexpr (std::is_same_v<K, int32_t>) {
    return vals ? segsort_pairs_i32(keys, vals, n, off, nseg, st) : segsort_keys_i32(keys, n, off, nseg, st);
  } else if constexpr (std::is_same_v<K, float>) {
    return vals ? segsort_pairs_f32(keys, vals, n, off, nseg, st) : segsort_keys_f32(keys, n, off, nseg, st);
  } else {
    return vals ? segsort_pairs_u64(keys, vals, n, off, nseg, st) : segsort_keys_u64(keys, n, off, nseg, st);
  }
}

// The plain call on keys already mapped to unsigned order bits.
template <typename K>
int sort_as_bits(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg,
                 cudaStream_t s) {
  using Bits = typename KeyOrder<K>::Bits;
  segsort_stream_t st = reinterpret_cast<segsort_stream_t>(s);
  if constexpr (sizeof(Bits) == 4) {
    uint32_t *kb = reinterpret_cast<uint32_t *>(keys);
    return vals ? segsort_pairs_u32(kb, vals, n, off, nseg, st) : segsort_keys_u32(kb, n, off, nseg, st);
  } else {
    uint64_t *kb = reinterpret_cast<uint64_t *>(keys);
    return vals ? segsort_pairs_u64(kb, vals, n, off, nseg, st) : segsort_keys_u64(kb, n, off, nseg, st);
  }
}

// Stable descending sort: equal keys keep their input order.
template <typename K>
int desc_impl(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg,
              bool pairs, cudaStream_t s) {
  if (n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  if (n == 0 || nseg == 0) return SEGSORT_OK;
  if (keys == nullptr || off == nullptr || (pairs && vals == nullptr)) return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
  desc_map_kernel<K, false><<<ew_blocks(n), kEwThreads, 0, s>>>(keys, n);
  if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
  const int rc = sort_as_bits(keys, pairs ? vals : nullptr, n, off, nseg, s);
  // Map back even when the sort failed, so the caller's keys are intact.
  desc_map_kernel<K, true><<<ew_blocks(n), kEwThreads, 0, s>>>(keys, n);
  if (cudaGetLastError() != cudaSuccess) return SEGSORT_ERR_CUDA;
  return rc;
}

template <typename K>
int topk_impl(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg, int64_t k,
              int descending, K *out_keys, uint32_t *out_vals, int32_t *out_counts,
              cudaStream_t s) {
  if (n < 0 || nseg < 0 || k < 0) return SEGSORT_ERR_INVALID_ARG;
  if (nseg == 0 || k == 0) return SEGSORT_OK;
  if (off == nullptr || out_keys == nullptr || (out_vals != nullptr && vals == nullptr))
    return SEGSORT_ERR_INVALID_ARG;
  if (static_cast<double>(nseg) * static_cast<double>(k) >= 9.0e18) return SEGSORT_ERR_TOO_LARGE;
  int rc = SEGSORT_OK;
  if (n > 0) {
    rc = descending ? desc_impl<K>(keys, vals, n, off, nseg, vals != nullptr, s)
                    : sort_typed(keys, vals, n, off, nseg, s);
    if (rc != SEGSORT_OK) return rc;
  }
  const Offsets o{off, nseg, 0, n};
  const int64_t slots = static_cast<int64_t>(nseg) * k;
  topk_gather_kernel<K><<<ew_blocks(slots), kEwThreads, 0, s>>>(keys, vals, o, k, out_keys,
                                                                out_vals, out_counts);
  return cudaGetLastError() == cudaSuccess ? SEGSORT_OK : SEGSORT_ERR_CUDA;
}

// 64-bit values: sort (key, position) pairs, then gather the values.
template <typename K>
int v64_impl(K *keys, uint64_t *vals, int64_t n, const int32_t *off, int32_t nseg,
             cudaStream_t s) {
  if (n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  if (n == 0 || nseg == 0) return SEGSORT_OK;
  if (keys == nullptr || vals == nullptr || off == nullptr) return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  DeviceState *S = device_state(dev);
  cudaMemPool_t pool = S ? device_pool(*S, dev) : nullptr;
  const size_t idx_bytes = align256(static_cast<size_t>(n) * 4);
  unsigned char *ws = nullptr;
  if (pool == nullptr ||
      cudaMallocFromPoolAsync(reinterpret_cast<void **>(&ws), idx_bytes + static_cast<size_t>(n) * 8,
                              pool, s) != cudaSuccess) {
    cudaGetLastError();
    return SEGSORT_ERR_NO_MEMORY;
  }
  uint32_t *idx = reinterpret_cast<uint32_t *>(ws);
  uint64_t *copy = reinterpret_cast<uint64_t *>(ws + idx_bytes);
  int rc = SEGSORT_OK;
  iota_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(idx, n);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(copy, vals, static_cast<size_t>(n) * 8, cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess) {
    rc = SEGSORT_ERR_CUDA;
  }
  if (rc == SEGSORT_OK) rc = sort_typed(keys, idx, n, off, nseg, s);
  if (rc == SEGSORT_OK) {
    gather64_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(vals, copy, idx, n);
    if (cudaGetLastError() != cudaSuccess) rc = SEGSORT_ERR_CUDA;
  }
  if (cudaFreeAsync(ws, s) != cudaSuccess && rc == SEGSORT_OK) rc = SEGSORT_ERR_CUDA;
  return rc;
}

// ---------------------------------------------------------------------------
// Segmented reduce-by-key after the sort.  Positions are handled in 32-bit
// words of a bitmap: segbits marks segment starts, headbits marks run heads
// (a segment start, or a key different from the previous key), and the run
// of a head at position p is the number of heads before p, read from an
// exclusive prefix of the per-word head counts plus a popcount.
constexpr int kScanItems = 1024;  // words per block of the word-count scan

__global__ void __launch_bounds__(kEwThreads) mark_starts_kernel(Offsets off, uint32_t *segbits) {
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= off.nseg) return;
  const int64_t b = off(s), e = off(s + 1);
  if (e > b) atomicOr(&segbits[b >> 5], 1u << (b & 31));
}

// Covered positions [lo, hi) = [off(0), off(nseg)), written to the device
// (the offsets live there).
__global__ void lohi_kernel(Offsets off, uint32_t *lohi) {
  lohi[0] = static_cast<uint32_t>(off(0));
  lohi[1] = static_cast<uint32_t>(off(off.nseg));
}

// One thread per word: head bits and their count.
__global__ void __launch_bounds__(kEwThreads)
head_bits_kernel(const uint32_t *keys, const uint32_t *segbits, const uint32_t *lohi,
                 int64_t words, uint32_t *headbits, uint32_t *wcount) {
  const int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= words) return;
  const int64_t lo = lohi[0], hi = lohi[1];
  const uint32_t sb = segbits[w];
  uint32_t bits = 0;
  const int64_t p0 = w * 32;
  uint32_t prev = p0 > 0 && p0 - 1 >= lo && p0 - 1 < hi ? keys[p0 - 1] : 0u;
  for (int j = 0; j < 32; ++j) {
    const int64_t p = p0 + j;
    if (p >= hi) break;
    if (p < lo) continue;
    const uint32_t k = keys[p];
    if (((sb >> j) & 1u) || p == lo || k != prev) bits |= 1u << j;
    prev = k;
  }
  headbits[w] = bits;
  wcount[w] = static_cast<uint32_t>(__popc(bits));
}

// Exclusive scan of wcount in blocks of kScanItems words: per-block totals,
// then (one CTA) their exclusive prefix and the grand total, then the
// per-word prefix.  Counts fit uint32 (n < 2^30).
__global__ void __launch_bounds__(kEwThreads)
block_totals_kernel(const uint32_t *wcount, int64_t words, uint32_t *btotal) {
  __shared__ int warp_s[kEwThreads / 32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanItems;
  uint32_t sum = 0;
  for (int i = threadIdx.x; i < kScanItems; i += kEwThreads)
    if (base + i < words) sum += wcount[base + i];
  uint32_t tot;
  block_exclusive_add<kEwThreads>(sum, tot, warp_s);
  if (threadIdx.x == 0) btotal[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kEwThreads)
scan_totals_kernel(uint32_t *btotal, int64_t nb, uint32_t *grand) {
  __shared__ int warp_s[kEwThreads / 32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nb; b0 += kEwThreads) {
    const int64_t b = b0 + threadIdx.x;
    const uint32_t v = b < nb ? btotal[b] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_add<kEwThreads>(v, tot, warp_s);
    if (b < nb) btotal[b] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(kEwThreads)
word_prefix_kernel(const uint32_t *wcount, int64_t words, const uint32_t *bprefix,
                   uint32_t *wprefix) {
  __shared__ int warp_s[kEwThreads / 32];
  __shared__ uint32_t carry;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanItems;
  if (threadIdx.x == 0) carry = bprefix[blockIdx.x];
  __syncthreads();
  for (int i0 = 0; i0 < kScanItems; i0 += kEwThreads) {
    const int64_t w = base + i0 + threadIdx.x;
    const uint32_t v = w < words ? wcount[w] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_add<kEwThreads>(v, tot, warp_s);
    if (w < words) wprefix[w] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kEwThreads)
zero_runs_kernel(uint64_t *sums, uint32_t *counts, const uint32_t *grand) {
  const int64_t runs = *grand;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < runs;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    sums[r] = 0;
    counts[r] = 0;
  }
}

// One thread per word: keys of its heads, and its elements' values and
// counts added to their runs (one atomic per run piece of the word).
__global__ void __launch_bounds__(kEwThreads)
run_write_kernel(const uint32_t *keys, const uint32_t *vals, const uint32_t *headbits,
                 const uint32_t *wprefix, const uint32_t *lohi, int64_t words,
                 uint32_t *out_keys, uint64_t *out_sums, uint32_t *out_counts) {
  const int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= words) return;
  const int64_t lo = lohi[0], hi = lohi[1];
  const uint32_t hb = headbits[w];
  const int64_t p0 = w * 32;
  // Run of the first covered position of the word: the heads before it.
  int64_t r = static_cast<int64_t>(wprefix[w]) - 1;
  uint64_t sum = 0;
  uint32_t cnt = 0;
  for (int j = 0; j < 32; ++j) {
    const int64_t p = p0 + j;
    if (p >= hi) break;
    if (p < lo) continue;
    if ((hb >> j) & 1u) {
      if (cnt) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&out_sums[r]), sum);
        atomicAdd(&out_counts[r], cnt);
      }
      ++r;
      out_keys[r] = keys[p];
      sum = 0;
      cnt = 0;
    }
    sum += vals[p];
    ++cnt;
  }
  if (cnt && r >= 0) {
    atomicAdd(reinterpret_cast<unsigned long long *>(&out_sums[r]), sum);
    atomicAdd(&out_counts[r], cnt);
  }
}

// out_offsets[s]: run index of segment s's first element (the number of
// heads before it); the total number of runs for s = nseg and for segments
// that start at or after the covered end.
__global__ void __launch_bounds__(kEwThreads)
run_offsets_kernel(Offsets off, const uint32_t *headbits, const uint32_t *wprefix,
                   const uint32_t *lohi, const uint32_t *grand, int32_t *out_offsets) {
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s > off.nseg) return;
  const int64_t hi = lohi[1];
  const int64_t p = off(s);
  uint32_t r = *grand;
  if (s < off.nseg && p < hi) {
    const int64_t w = p >> 5;
    const uint32_t below = (1u << (p & 31)) - 1u;
    r = wprefix[w] + static_cast<uint32_t>(__popc(headbits[w] & below));
  }
  out_offsets[s] = static_cast<int32_t>(r);
}

int reduce_by_key_impl(uint32_t *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg,
                       uint32_t *out_keys, uint64_t *out_sums, uint32_t *out_counts,
                       int32_t *out_offsets, cudaStream_t s) {
  if (n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  if (nseg > 0 && (off == nullptr || out_offsets == nullptr)) return SEGSORT_ERR_INVALID_ARG;
  if (n > 0 && nseg > 0 &&
      (keys == nullptr || vals == nullptr || out_keys == nullptr || out_sums == nullptr ||
       out_counts == nullptr))
    return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
  if (nseg == 0) return SEGSORT_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  DeviceState *S = device_state(dev);
  cudaMemPool_t pool = S ? device_pool(*S, dev) : nullptr;
  const int64_t words = (n + 31) / 32 + 1;
  const int64_t nb = (words + kScanItems - 1) / kScanItems;
  const size_t wbytes = align256(static_cast<size_t>(words) * 4);
  const size_t total = 4 * wbytes + align256(static_cast<size_t>(nb) * 4) + 256;
  unsigned char *ws = nullptr;
  if (pool == nullptr ||
      cudaMallocFromPoolAsync(reinterpret_cast<void **>(&ws), total, pool, s) != cudaSuccess) {
    cudaGetLastError();
    return SEGSORT_ERR_NO_MEMORY;
  }
  uint32_t *segbits = reinterpret_cast<uint32_t *>(ws);
  uint32_t *headbits = reinterpret_cast<uint32_t *>(ws + wbytes);
  uint32_t *wcount = reinterpret_cast<uint32_t *>(ws + 2 * wbytes);
  uint32_t *wprefix = reinterpret_cast<uint32_t *>(ws + 3 * wbytes);
  uint32_t *btotal = reinterpret_cast<uint32_t *>(ws + 4 * wbytes);
  uint32_t *grand = reinterpret_cast<uint32_t *>(ws + 4 * wbytes + align256(static_cast<size_t>(nb) * 4));
  uint32_t *lohi = grand + 1;
  int rc = n > 0 ? sort_typed<uint32_t>(keys, vals, n, off, nseg, s) : SEGSORT_OK;
  const Offsets o{off, nseg, 0, n};
  if (rc == SEGSORT_OK) {
    lohi_kernel<<<1, 1, 0, s>>>(o, lohi);
    if (cudaMemsetAsync(segbits, 0, wbytes, s) != cudaSuccess) rc = SEGSORT_ERR_CUDA;
  }
  if (rc == SEGSORT_OK) {
    mark_starts_kernel<<<ew_blocks(nseg), kEwThreads, 0, s>>>(o, segbits);
    head_bits_kernel<<<ew_blocks(words), kEwThreads, 0, s>>>(keys, segbits, lohi, words, headbits,
                                                            wcount);
    block_totals_kernel<<<static_cast<unsigned>(nb), kEwThreads, 0, s>>>(wcount, words, btotal);
    scan_totals_kernel<<<1, kEwThreads, 0, s>>>(btotal, nb, grand);
    word_prefix_kernel<<<static_cast<unsigned>(nb), kEwThreads, 0, s>>>(wcount, words, btotal, wprefix);
    zero_runs_kernel<<<static_cast<unsigned>(S->sms * 4), kEwThreads, 0, s>>>(out_sums, out_counts, grand);
    run_write_kernel<<<ew_blocks(words), kEwThreads, 0, s>>>(keys, vals, headbits, wprefix, lohi,
                                                            words, out_keys, out_sums, out_counts);
    run_offsets_kernel<<<ew_blocks(static_cast<int64_t>(nseg) + 1), kEwThreads, 0, s>>>(
        o, headbits, wprefix, lohi, grand, out_offsets);
    if (cudaGetLastError() != cudaSuccess) rc = SEGSORT_ERR_CUDA;
  }
  if (cudaFreeAsync(ws, s) != cudaSuccess && rc == SEGSORT_OK) rc = SEGSORT_ERR_CUDA;
  return rc;
}

}  // namespace
}  // namespace segsort

using segsort::desc_impl;
using segsort::topk_impl;
using segsort::v64_impl;

extern "C" {

#define SEGSORT_ST(s) reinterpret_cast<cudaStream_t>(s)

int segsort_pairs_u32_desc(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           segsort_stream_t s) {
  return desc_impl<uint32_t>(k, v, n, o, ns, true, SEGSORT_ST(s));
}
int segsort_pairs_i32_desc(int32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           segsort_stream_t s) {
  return desc_impl<int32_t>(k, v, n, o, ns, true, SEGSORT_ST(s));
}
int segsort_pairs_f32_desc(float *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           segsort_stream_t s) {
  return desc_impl<float>(k, v, n, o, ns, true, SEGSORT_ST(s));
}
int segsort_pairs_u64_desc(uint64_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           segsort_stream_t s) {
  return desc_impl<uint64_t>(k, v, n, o, ns, true, SEGSORT_ST(s));
}
int segsort_keys_u32_desc(uint32_t *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return desc_impl<uint32_t>(k, nullptr, n, o, ns, false, SEGSORT_ST(s));
}
int segsort_keys_f32_desc(float *k, int64_t n, const int32_t *o, int32_t ns, segsort_stream_t s) {
  return desc_impl<float>(k, nullptr, n, o, ns, false, SEGSORT_ST(s));
}

int segsort_pairs_u32_topk(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           int64_t topk, int descending, uint32_t *ok, uint32_t *ov,
                           int32_t *counts, segsort_stream_t s) {
  return topk_impl<uint32_t>(k, v, n, o, ns, topk, descending, ok, ov, counts, SEGSORT_ST(s));
}
int segsort_pairs_f32_topk(float *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                           int64_t topk, int descending, float *ok, uint32_t *ov, int32_t *counts,
                           segsort_stream_t s) {
  return topk_impl<float>(k, v, n, o, ns, topk, descending, ok, ov, counts, SEGSORT_ST(s));
}

int segsort_pairs_u32_v64(uint32_t *k, uint64_t *v, int64_t n, const int32_t *o, int32_t ns,
                          segsort_stream_t s) {
  return v64_impl<uint32_t>(k, v, n, o, ns, SEGSORT_ST(s));
}
int segsort_pairs_i32_v64(int32_t *k, uint64_t *v, int64_t n, const int32_t *o, int32_t ns,
                          segsort_stream_t s) {
  return v64_impl<int32_t>(k, v, n, o, ns, SEGSORT_ST(s));
}
int segsort_pairs_f32_v64(float *k, uint64_t *v, int64_t n, const int32_t *o, int32_t ns,
                          segsort_stream_t s) {
  return v64_impl<float>(k, v, n, o, ns, SEGSORT_ST(s));
}
int segsort_pairs_u64_v64(uint64_t *k, uint64_t *v, int64_t n, const int32_t *o, int32_t ns,
                          segsort_stream_t s) {
  return v64_impl<uint64_t>(k, v, n, o, ns, SEGSORT_ST(s));
}

}  // extern "C"

extern "C" int segsort_pairs_u32_reduce_by_key(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o,
                                               int32_t ns, uint32_t *ok, uint64_t *sums,
                                               uint32_t *counts, int32_t *out_off,
                                               segsort_stream_t s) {
  return segsort::reduce_by_key_impl(k, v, n, o, ns, ok, sums, counts, out_off,
                                     reinterpret_cast<cudaStream_t>(s));
}
