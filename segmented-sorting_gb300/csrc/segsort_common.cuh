// Shared device-side pieces of the segmented sort: the order-preserving key
// maps, the offsets accessor, the device status word and small helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "segsort.h"

namespace segsort {

// ---------------------------------------------------------------------------
// Order-preserving maps between a key and unsigned "order bits".  Sorting the
// bits as unsigned integers sorts the keys.  The signed rule is the sign-bit
// flip of CUB's RadixTraits::TwiddleIn (lib/cub/util_type.cuh:937-949); the
// float rule flips every bit of negative values and only the sign bit of the
// others, so -0.0 < +0.0 and NaNs order by bit pattern.
// ---------------------------------------------------------------------------
template <typename K> struct KeyOrder;

template <> struct KeyOrder<uint32_t> {
  using Bits = uint32_t;
  static __host__ __device__ __forceinline__ Bits to_bits(uint32_t k) { return k; }
  static __host__ __device__ __forceinline__ uint32_t from_bits(Bits b) { return b; }
};

template <> struct KeyOrder<int32_t> {
  using Bits = uint32_t;
  static __host__ __device__ __forceinline__ Bits to_bits(int32_t k) {
    return static_cast<uint32_t>(k) ^ 0x80000000u;
  }
  static __host__ __device__ __forceinline__ int32_t from_bits(Bits b) {
    return static_cast<int32_t>(b ^ 0x80000000u);
  }
};

template <> struct KeyOrder<float> {
  using Bits = uint32_t;
  static __device__ __forceinline__ Bits to_bits(float k) {
    uint32_t u = __float_as_uint(k);
    uint32_t mask = (u & 0x80000000u) ? 0xFFFFFFFFu : 0x80000000u;
    return u ^ mask;
  }
  static __device__ __forceinline__ float from_bits(Bits b) {
    uint32_t mask = (b & 0x80000000u) ? 0x80000000u : 0xFFFFFFFFu;
    return __uint_as_float(b ^ mask);
  }
};

template <> struct KeyOrder<uint64_t> {
  using Bits = uint64_t;
  static __host__ __device__ __forceinline__ Bits to_bits(uint64_t k) { return k; }
  static __host__ __device__ __forceinline__ uint64_t from_bits(Bits b) { return b; }
};

// ---------------------------------------------------------------------------
// Segment offsets.  off(i) for i in [0, nseg] is the begin of segment i (and
// the end of segment i-1).  CSR arrays hold nseg+1 entries; heads-only arrays
// hold nseg and the end of the last segment is n.  Every value is clamped into
// [0, n], so malformed offsets cannot address memory outside the arrays.
// ---------------------------------------------------------------------------
constexpr uint8_t kSegSkip = 0x80;    // already sorted
constexpr uint8_t kSegTmp = 0x40;     // its keys and values are in the temporary buffers
constexpr uint8_t kSegShared = 0x3F;  // leading order bits its keys share

struct Offsets {
  const int32_t *p;
  int32_t nseg;
  int32_t heads;  // 1: heads-only array of nseg entries
  int64_t n;
  // Optional per-segment flags (null for the caller's offsets): kSegSkip
  // marks a segment already sorted (one the radix passes finished before the
  // rest of the call; classify gives it no job); kSegTmp a segment whose keys
  // and values are in the temporary buffers (only the bucket kernel reads
  // them there; the result goes to the caller's buffers); the low bits the
  // number of leading order bits every key of the segment shares (a hint
  // for the bucket sort's scaling).
  const uint8_t *flags = nullptr;

  __device__ __forceinline__ int64_t operator()(int64_t i) const {
    int64_t v = (heads && i >= nseg) ? n : static_cast<int64_t>(__ldg(p + i));
    v = v < 0 ? 0 : v;
    return v > n ? n : v;
  }
};

// ---------------------------------------------------------------------------
// One instance of a batched call, as the kernels see it.  A batch is a list of
// independent (keys, values, offsets) problems of one key type sorted by one
// launch of each kernel.  Every per-instance index is instance-local; the
// *_base fields place the instance in the batch-wide arrays: its region of
// the temporary key/value buffers, its half-tile map (2 * tiles + 1 entries,
// one classify warp each) and its tile-sort CTAs.
// ---------------------------------------------------------------------------
struct BatchInst {
  void *keys;
  uint32_t *vals;
  const int32_t *offsets;
  const uint8_t *flags;  // per-segment flags (Offsets::flags) or null
  int64_t n;
  int64_t tmp_base;
  int64_t half_base;
  int64_t tile_base;
  int64_t msd_base;      // the instance's first entry in the MSD route's expansion
  int32_t nseg;
  int32_t heads;

  __device__ __forceinline__ Offsets offsets_view() const {
    return Offsets{offsets, nseg, heads, n, flags};
  }
};

// The last instance whose `field` is at or below x (instances with equal
// bases own nothing before the next one; the host drops empty instances).
__device__ __forceinline__ int32_t find_instance(const BatchInst *tab, int32_t count, int64_t x,
                                                 int64_t BatchInst::*field) {
  int32_t lo = 0, hi = count - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (tab[mid].*field <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Device status word: kernels OR error bits into it; the host reads it back
// with segsort_device_status().
// ---------------------------------------------------------------------------
enum : uint32_t {
  kStatusTimeout = 1u,
};

// One word per translation unit of the library (internal linkage); the host
// reads every unit's word.
static __device__ uint32_t g_device_status = 0;

__device__ __forceinline__ void raise_status(uint32_t bits) {
  atomicOr(&g_device_status, bits);
}

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

// Programmatic dependent launch (PTX griddepcontrol).  A kernel launched with
// programmatic stream serialization may start while the kernel before it on
// the stream is still running; pdl_wait() returns once that kernel has
// completed and its writes are visible (at once for an ordinary launch).
// pdl_trigger() lets the next such kernel start launching: it is issued at
// the start of a kernel, and a dependent launches only after every CTA of
// this grid has issued it or exited, so every CTA is resident by then.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace segsort
