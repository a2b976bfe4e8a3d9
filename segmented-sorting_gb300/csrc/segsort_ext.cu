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
