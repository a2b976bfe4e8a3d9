// MSD route for the radix segments: one stable radix pass on the top digit
// that varies, then the tile sort of the sub-buckets.
//
// A radix segment (longer than the radix threshold) whose keys vary in at
// least kMsdMinDigits digit positions, and whose top varying digit leaves no
// bucket longer than kMsdMaxBucketTiles tiles, is sorted in two stages
// instead of one LSD pass per varying digit:
//   stage 1  the long-segment kernel with LargeWs::msd_stage set: the counts
//            and bucket starts as for the LSD passes, then one stable counting
//            pass on that top digit for these segments (all their passes and
//            the copy back for the other radix segments), and no merge
//            passes.  The segment is now its 256 sub-buckets in order, each
//            holding its keys in their input order, in the temporary buffers.
//   expand   (this file) the offsets of a second problem over the same keys:
//            every segment as it was, except that an MSD segment becomes its
//            sub-buckets (flagged with the order bits their keys share: the
//            digits above and at the top varying digit, which the bucket
//            sort shifts out) and a radix segment stage 1 finished is marked
//            skip.
//   stage 2  the usual launch sequence over those offsets: classify (no jobs
//            for skipped segments), the bucket route of the tile sort (it
//            reads a sub-bucket from the temporary buffers and writes it to
//            the caller's, or to the buffer the first merge pass reads for the
//            CAP-runs of a sub-bucket longer than a tile; a chunk it refuses
//            it first copies to the caller's buffers for the comparison
//            sort), the long-segment kernel (merge passes for the rest).
// For 32-bit keys that is 4 bytes per key for the counts and 16 + 16 bytes
// per pair for the pass and the tile sort, against 4 + 4 * 16 for four LSD
// passes.  The output is the stable sort of every
// segment either way (the pass is stable and the sub-buckets are sorted
// stably), so the route changes nothing in the result.
//
// The reference has no counterpart: its long segments go through merge
// passes (src/bb_segsort/bb_comput_l.h:1264-1272) or CUB's per-segment radix
// sort (src/radixseg.cu:115-124).
#pragma once

#include "radix_sort.cuh"

namespace segsort {

// Device arrays of the expansion.
struct MsdWs {
  int32_t *sub;     // [c_len + 1] the second stage's offsets (CSR)
  uint8_t *flags;   // [c_len] kSegSkip: stage 1 finished it; else the shared order bits
  int64_t c_len;    // the second stage's segments, padded with empty ones at n
  int32_t *jbeg;    // [max_rjobs] radix job begins, ascending
  int32_t *jidx;    // [max_rjobs] the job of each
  int32_t *jextra;  // [max_rjobs + 1] entries the MSD jobs before add (255 each)
};

// Segments the second stage can hold: every segment, plus 255 per radix job.
inline int64_t msd_stage2_segments(int64_t nseg, int64_t max_rjobs) {
  return nseg + (kRBuckets - 1) * max_rjobs;
}

// Thread per radix job q: its rank by begin (radix segments are non-empty
// and disjoint, so the begins differ) and the MSD jobs before it.
template <typename K>
__global__ void __launch_bounds__(256) msd_rank_kernel(LargeWs<K> ws, MsdWs M) {
  pdl_wait();     // stage 1's jobs and bucket starts
  pdl_trigger();  // the expansion may launch under this one
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q == 0 && nj == 0) M.jextra[0] = 0;
  if (q >= nj) return;
  const int32_t b = ws.rjobs[q].x;
  int32_t rank = 0, msd_before = 0;
  for (int32_t r = 0; r < nj; ++r) {
    if (__ldg(&ws.rjobs[r].x) < b) {
      ++rank;
      msd_before += (__ldg(&ws.rdigits[r]) & kRDigitMsd) != 0u;
    }
  }
  if (rank >= nj) return;  // only with malformed (overlapping) offsets
  M.jbeg[rank] = b;
  M.jidx[rank] = static_cast<int32_t>(q);
  M.jextra[rank] = (kRBuckets - 1) * msd_before;
  if (rank == nj - 1)
    M.jextra[nj] = (kRBuckets - 1) * (msd_before + ((ws.rdigits[q] & kRDigitMsd) != 0u));
}

// Thread per segment j: its entry of the second stage's offsets, at j plus
// the extra entries of the radix jobs that begin before it (an MSD
// segment's 256 entries are msd_sub_kernel's); the threads then fill the
// entries past the last segment with n (empty segments).  Every write is
// bounded by c_len, so malformed offsets cannot reach outside the arrays.
template <typename K>
__global__ void __launch_bounds__(256) msd_expand_kernel(Offsets off, LargeWs<K> ws, MsdWs M) {
  pdl_wait();     // the jobs' ranks
  pdl_trigger();  // the sub-bucket kernel may launch under this one
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t all_extra = M.jextra[nj];
  auto put = [&](int64_t at, int64_t v, uint8_t sk) {
    if (at >= 0 && at < M.c_len) {
      M.sub[at] = static_cast<int32_t>(v);
      M.flags[at] = sk;
    }
  };
  if (j < off.nseg) {
    const int64_t s = off(j), e = off(j + 1);
    int32_t lo = 0, hi = nj;  // radix jobs beginning before s
    while (lo < hi) {
      const int32_t mid = (lo + hi) >> 1;
      if (M.jbeg[mid] < s) lo = mid + 1; else hi = mid;
    }
    const int64_t base = j + M.jextra[lo];
    if (lo < nj && M.jbeg[lo] == s && e - s > ws.radix_min) {
      const uint32_t v = ws.rdigits[M.jidx[lo]];
      if (!(v & kRDigitMsd))  // stage 1 finished it, or left it to the second stage
        put(base, s, (v & kRDigitDefer) ? 0 : kSegSkip);
    } else {
      put(base, s, 0);
    }
  }
  const int64_t step = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = off.nseg + all_extra + j; i <= M.c_len; i += step) {
    if (i < M.c_len) M.flags[i] = 0;
    if (i >= 0) M.sub[i] = static_cast<int32_t>(off.n);
  }
}

// Block per radix job (by rank), thread per bucket g: entry g of an MSD
// segment, the start of its sub-bucket g, flagged with the order bits the
// sub-bucket's keys share (the digits above and at the top varying digit).
template <typename K>
__global__ void __launch_bounds__(kRBuckets) msd_sub_kernel(LargeWs<K> ws, MsdWs M) {
  pdl_wait();  // the expanded offsets
  constexpr int64_t D = sizeof(typename KeyOrder<K>::Bits);
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int32_t r = blockIdx.x;
  if (r >= nj) return;
  const int32_t q = M.jidx[r];
  const uint32_t v = ws.rdigits[q];
  if (!(v & kRDigitMsd)) return;
  const int4 jb = ws.rjobs[q];
  const int dt = 31 - __clz(v & kRDigitMask);
  const int g = threadIdx.x;
  const int64_t at = static_cast<int64_t>(jb.z) + M.jextra[r] + g;
  const uint32_t st = ws.rhist[(static_cast<int64_t>(q) * D + dt) * kRBuckets + g];
  if (at >= 0 && at < M.c_len) {
    M.sub[at] = jb.x + static_cast<int32_t>(st);
    M.flags[at] = static_cast<uint8_t>(8 * (D - dt)) | kSegTmp;
  }
}

// ---------------------------------------------------------------------------
// The batched form: one expansion per key-type group.  Jobs carry their
// instance (int4 .w) and segment (.z); every instance has its own
// second-stage offsets and flags (the stage-2 table's offsets / flags, its
// nseg the padded count c_len) and owns the expansion entries
// [msd_base, msd_base + c_len + 1) of the flat thread index.
struct MsdBatchWs {
  int32_t *jbeg;    // [max_rjobs] radix job begins, by (instance, begin)
  int32_t *jidx;    // [max_rjobs] the job of each
  int32_t *jinst;   // [max_rjobs] its instance
  int32_t *jextra;  // [max_rjobs] entries the instance's MSD jobs before it add (255 each)
};

// Thread per radix job q: its rank by (instance, begin) and the MSD jobs of
// its instance before it.
template <typename K>
__global__ void __launch_bounds__(256) msd_rank_batch_kernel(LargeWs<K> ws, MsdBatchWs M) {
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= nj) return;
  const int4 me = ws.rjobs[q];
  int32_t rank = 0, msd_before = 0;
  for (int32_t r = 0; r < nj; ++r) {
    const int32_t w = __ldg(&ws.rjobs[r].w), x = __ldg(&ws.rjobs[r].x);
    if (w < me.w || (w == me.w && x < me.x)) {
      ++rank;
      if (w == me.w) msd_before += (__ldg(&ws.rdigits[r]) & kRDigitMsd) != 0u;
    }
  }
  if (rank >= nj) return;  // only with malformed (overlapping) offsets
  M.jbeg[rank] = me.x;
  M.jidx[rank] = static_cast<int32_t>(q);
  M.jinst[rank] = me.w;
  M.jextra[rank] = (kRBuckets - 1) * msd_before;
}

// First rank in [lo, hi) whose (instance, begin) is at or above (w, x).
__device__ __forceinline__ int32_t msd_lower_bound(const MsdBatchWs &M, int32_t lo, int32_t hi,
                                                   int32_t w, int64_t x) {
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (M.jinst[mid] < w || (M.jinst[mid] == w && M.jbeg[mid] < x)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Thread per expansion entry: entry j < nseg of an instance is its segment j
// (one entry, at j plus the extra entries of the instance's MSD jobs before
// it; an MSD segment's 256 are msd_sub_batch_kernel's); the entries from
// nseg on fill the instance's padding with n.
template <typename K>
__global__ void __launch_bounds__(256)
msd_expand_batch_kernel(const BatchInst *__restrict__ tab1, const BatchInst *__restrict__ tab2,
                        int32_t count, int64_t entries, LargeWs<K> ws, MsdBatchWs M) {
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= entries) return;
  const int32_t i = find_instance(tab2, count, f, &BatchInst::msd_base);
  const BatchInst &I2 = tab2[i];
  const Offsets off = tab1[i].offsets_view();
  int32_t *sub = const_cast<int32_t *>(I2.offsets);
  uint8_t *flags = const_cast<uint8_t *>(I2.flags);
  const int64_t c_len = I2.nseg;
  const int64_t j = f - I2.msd_base;
  // The instance's jobs and the extra entries of all of its MSD jobs.
  const int32_t r0 = msd_lower_bound(M, 0, nj, i, INT64_MIN);
  const int32_t r1 = msd_lower_bound(M, r0, nj, i + 1, INT64_MIN);
  const int64_t all_extra =
      r1 > r0 ? M.jextra[r1 - 1] + (kRBuckets - 1) * ((ws.rdigits[M.jidx[r1 - 1]] & kRDigitMsd) != 0u)
              : 0;
  auto put = [&](int64_t at, int64_t v, uint8_t sk) {
    if (at >= 0 && at < c_len) {
      sub[at] = static_cast<int32_t>(v);
      flags[at] = sk;
    }
  };
  if (j < off.nseg) {
    const int64_t s = off(j), e = off(j + 1);
    const int32_t lo = msd_lower_bound(M, r0, r1, i, s);
    const int64_t base = j + (lo < r1 ? M.jextra[lo] : all_extra);
    if (lo < r1 && M.jbeg[lo] == s && e - s > ws.radix_min) {
      const uint32_t v = ws.rdigits[M.jidx[lo]];
      if (!(v & kRDigitMsd)) put(base, s, (v & kRDigitDefer) ? 0 : kSegSkip);
    } else {
      put(base, s, 0);
    }
  } else {
    const int64_t at = off.nseg + all_extra + (j - off.nseg);
    if (at <= c_len) {
      if (at < c_len) flags[at] = 0;
      if (at >= 0) sub[at] = static_cast<int32_t>(off.n);
    }
  }
}

// Block per radix job (by rank), thread per bucket g: entry g of an MSD
// segment in its instance's second-stage offsets.
template <typename K>
__global__ void __launch_bounds__(kRBuckets)
msd_sub_batch_kernel(const BatchInst *__restrict__ tab2, LargeWs<K> ws, MsdBatchWs M) {
  constexpr int64_t D = sizeof(typename KeyOrder<K>::Bits);
  const int32_t nj = min(static_cast<int32_t>(ld_volatile(&ws.ctr[kCtrRJobs])), ws.max_rjobs);
  const int32_t r = blockIdx.x;
  if (r >= nj) return;
  const int32_t q = M.jidx[r];
  const uint32_t v = ws.rdigits[q];
  if (!(v & kRDigitMsd)) return;
  const int4 jb = ws.rjobs[q];
  const BatchInst &I2 = tab2[jb.w];
  const int dt = 31 - __clz(v & kRDigitMask);
  const int g = threadIdx.x;
  const int64_t at = static_cast<int64_t>(jb.z) + M.jextra[r] + g;
  const uint32_t st = ws.rhist[(static_cast<int64_t>(q) * D + dt) * kRBuckets + g];
  if (at >= 0 && at < I2.nseg) {
    const_cast<int32_t *>(I2.offsets)[at] = jb.x + static_cast<int32_t>(st);
    const_cast<uint8_t *>(I2.flags)[at] = static_cast<uint8_t>(8 * (D - dt)) | kSegTmp;
  }
}

}  // namespace segsort
