// Long segments by merging: segments longer than the tile capacity CAP and
// at most the radix threshold (longer ones take the radix passes of
// radix_sort.cuh, which run first in the same cooperative kernel).
//
// The tile kernel has already sorted every CAP-chunk of each long segment
// (its "runs", tile_cta), so a long segment of len elements is
// ceil(len / CAP) sorted runs.  Merge pass p merges neighbouring runs of
// CAP * 2^p elements into runs twice as long; after merge_passes(len, CAP)
// passes the segment is one run.  Every pass reads and writes each key and
// value of the segments still being merged once (16 bytes per 32-bit
// key/value pair), ping-ponging between the caller's buffers and tmp; the
// tile kernel chose the buffer of the runs so that the last pass writes the
// caller's buffers.
//
// One cooperative kernel runs all passes.  A pass has two phases separated
// by a bounded grid barrier:
//   partition  one half-warp per output item (T consecutive outputs of one
//              merge) finds where the item starts in the two runs (merge
//              path, 16 probes per round over global memory);
//   merge      one CTA per item loads the two windows the item consumes into
//              shared memory, each thread merges KPT outputs from its own
//              merge-path split of the windows, and the CTA stores the item
//              with 16-byte stores.
// Ties take the earlier run first, and the runs hold stable orders, so the
// result is the stable sort of the segment.
//
// It replaces the reference's merge passes over global memory for segments
// longer than one block (src/bb_segsort/bb_comput_l.h:1155-1284: a 2048-key
// block sort followed by log2(len / 2048) merge passes, each pass driven from
// the host).
#pragma once

#include "segsort_common.cuh"
#include "tile_sort.cuh"
#include "classify.cuh"
#include "radix_sort.cuh"

namespace segsort {

// Launch shape of the merge kernel (build-time knobs; the defaults are the
// measured best on GB300).
#ifndef SEGSORT_MERGE_THREADS
#define SEGSORT_MERGE_THREADS 256
#endif
#ifndef SEGSORT_MERGE_MINB
#define SEGSORT_MERGE_MINB 3
#endif
constexpr int kMThreads = SEGSORT_MERGE_THREADS;
constexpr int kMWarps = kMThreads / 32;

// Outputs per item: kMThreads * 16 for 32-bit keys, kMThreads * 8 for 64-bit
// keys, at most one tile, so an item never spans two merges (a merge covers
// 2 * CAP * 2^p outputs).
template <typename K>
struct MergeShape {
  static constexpr int KPT = sizeof(K) == 4 ? 16 : 8;
  static constexpr int T = kMThreads * KPT;
};

template <typename K, bool PAIRS>
struct MergeSmem {
  static constexpr int T = MergeShape<K>::T;
  // Input windows with one padding slot per 8 elements: the threads of a warp
  // read them at strides near 8 during their merges, which would otherwise
  // fall on a few banks.
  static constexpr int XSLOTS = T + T / 8;
  static constexpr int OSLOTS = T + T / 32;  // output staging, one padding slot per 32
  static constexpr size_t kKeysIn = (static_cast<size_t>(XSLOTS) * sizeof(K) + 15) / 16 * 16;
  static constexpr size_t kIn = kKeysIn + (PAIRS ? static_cast<size_t>(XSLOTS) * 4 : 0);
  static constexpr size_t kOut = static_cast<size_t>(OSLOTS) * (sizeof(K) + (PAIRS ? 4 : 0));
  static constexpr size_t kBytes = (kIn + 15) / 16 * 16 + kOut;
  static __device__ __forceinline__ int xslot(int i) { return i + (i >> 3); }
  static __device__ __forceinline__ int oslot(int i) { return i + (i >> 5); }
};

// Merge-path split of diagonal d of the sorted runs A[0, la) and B[0, lb):
// how many elements of A are among the first d outputs of their merge, ties
// taken from A first.  Called by a group of W lanes (a whole warp, or the
// aligned half of one); every round probes W points of the remaining
// interval.
template <int W, typename K>
__device__ __forceinline__ int64_t group_merge_split(const K *A, int64_t la, const K *B,
                                                     int64_t lb, int64_t d) {
  static_assert(W == 16 || W == 32, "a group is a warp or half of one");
  using Ord = KeyOrder<K>;
  const int lane = threadIdx.x & 31;
  const int gl = lane & (W - 1);   // lane within the group
  const int g0 = lane & ~(W - 1);  // the group's first lane
  const unsigned mask = W == 32 ? 0xFFFFFFFFu : (0xFFFFu << g0);
  int64_t lo = d > lb ? d - lb : 0;
  int64_t hi = d < la ? d : la;
  // The split s is in [lo, hi]; A[i] <= B[d - 1 - i] holds exactly for i < s.
  while (hi > lo) {
    const int64_t span = hi - lo;
    const bool small = span <= W;
    const int64_t mid = small ? lo + gl : lo + (span * (gl + 1)) / (W + 1);
    bool pred = false;
    if (!small || gl < span) pred = Ord::to_bits(A[mid]) <= Ord::to_bits(B[d - 1 - mid]);
    const int c = __popc(__ballot_sync(mask, pred) & mask);
    if (small) {
      lo += c;
      hi = lo;
    } else {
      const long long last_true =
          __shfl_sync(mask, static_cast<long long>(mid), g0 + (c > 0 ? c - 1 : 0));
      const long long first_false =
          __shfl_sync(mask, static_cast<long long>(mid), g0 + (c < W ? c : W - 1));
      const int64_t nlo = c > 0 ? last_true + 1 : lo;
      const int64_t nhi = c < W ? first_false : hi;
      lo = nlo;
      hi = nhi;
    }
  }
  return lo;
}

// Copies R global ranges src[r][0, len[r]) into shared memory through
// put(r, i, value): 16-byte loads for the aligned middles, scalar loads for
// the unaligned ends.  Every
// load of a round is issued before the round's first shared-memory store, so
// the ranges' memory latencies overlap instead of adding up.
template <int NT, int U, int R, typename T, typename Put>
__device__ __forceinline__ void load_ranges(const T *const (&src)[R], const int (&len)[R],
                                            Put &&put) {
  constexpr int V = 16 / static_cast<int>(sizeof(T));
  const int tid = threadIdx.x;
  int head[R], nvec[R];
  int most = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    head[r] = align_head(src[r], len[r]);
    nvec[r] = (len[r] - head[r]) / V;
    most = max(most, nvec[r]);
  }
  T ends[R][2];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t0 = head[r] + nvec[r] * V;
    if (tid < head[r]) ends[r][0] = __ldcs(src[r] + tid);
    if (t0 + tid < len[r]) ends[r][1] = __ldcs(src[r] + t0 + tid);
  }
  for (int k0 = 0; k0 < most; k0 += U * NT) {
    uint4 v[R][U];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint4 *pv = reinterpret_cast<const uint4 *>(src[r] + head[r]);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + u * NT + tid;
        if (k < nvec[r]) v[r][u] = __ldcs(pv + k);
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = k0 + u * NT + tid;
        if (k < nvec[r]) {
          T e[V];
          memcpy(e, &v[r][u], 16);
#pragma unroll
          for (int c = 0; c < V; ++c) put(r, head[r] + k * V + c, e[c]);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t0 = head[r] + nvec[r] * V;
    if (tid < head[r]) put(r, tid, ends[r][0]);
    if (t0 + tid < len[r]) put(r, t0 + tid, ends[r][1]);
  }
}

// ---------------------------------------------------------------------------
// Resident CTAs per SM the registers must allow: 3 for 32-bit keys; 2 for
// 64-bit keys, whose merge at 80 registers spilled 400 bytes a thread
// (measured on GB300, 2^23 u64 pairs in segments of 2^16: 0.857 ms at 3 CTAs
// per SM with the spills, 0.797 ms at 2 without).
template <typename K>
constexpr int kMergeMinBlocks = sizeof(K) == 8 ? 2 : SEGSORT_MERGE_MINB;

// Dynamic shared memory of the long-segment kernel: the larger of the radix
// phases' and the merge passes' layouts.
template <typename K, bool PAIRS>
struct LongSmem {
  static constexpr size_t kMerge = MergeSmem<K, PAIRS>::kBytes;
  static constexpr size_t kRadix = RadixShape<K, PAIRS, kMThreads>::kBytes;
  static constexpr size_t kBytes = kMerge > kRadix ? kMerge : kRadix;
};

// The long-segment kernel: the radix phases for the segments longer than
// ws.radix_min, then the merge passes for the other segments longer than
// cap.  Cooperative launch (every CTA resident).
template <typename K, bool PAIRS, typename Space>
__global__ void __launch_bounds__(kMThreads, kMergeMinBlocks<K>)
long_segment_kernel(Space sp, LargeWs<K> ws, int64_t cap) {
  using Ord = KeyOrder<K>;
  using MS = MergeSmem<K, PAIRS>;
  constexpr int NT = kMThreads;
  constexpr int KPT = MergeShape<K>::KPT;
  constexpr int T = MergeShape<K>::T;

  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int warp_s[kMWarps];
  __shared__ uint64_t carry_s;
  __shared__ int maxp_s;

  // The MSD route's rank kernel may launch under this one (it waits for it);
  // every CTA of this cooperative grid is resident before it can.
  pdl_trigger();
  radix_phases<K, PAIRS, NT>(sp, ws, smem, warp_s);
  if (ws.msd_stage) return;  // the merge passes run after the tile sort of the sub-buckets

  const int tid = threadIdx.x;
  const int64_t G = gridDim.x;
  const int64_t nj = min(static_cast<int64_t>(ld_volatile(&ws.ctr[kCtrJobs])),
                         static_cast<int64_t>(ws.max_jobs));
  if (nj == 0) return;  // no segments for the merge passes
  const int4 *jobs = ws.jobs;
  int32_t *item_prefix = ws.item_prefix;   // [nj + 1] items before each job
  int32_t *item_job = ws.item_job;         // [items] job of each item
  uint32_t *split = ws.split;              // [items] merge-path split of its first output

  // ---- setup (CTA 0): items per job, their prefix, the most passes ---------
  if (blockIdx.x == 0) {
    if (tid == 0) {
      carry_s = 0;
      maxp_s = 0;
    }
    __syncthreads();
    const uint64_t capi = static_cast<uint64_t>(ws.max_items);
    int mp = 0;
    for (int64_t base = 0; base < nj; base += NT) {
      const int64_t j = base + tid;
      uint32_t v = 0;
      if (j < nj) {
        const int4 jb = jobs[j];
        const int64_t len = jb.y > jb.x ? jb.y - jb.x : 0;
        v = static_cast<uint32_t>((len + T - 1) / T);
        mp = max(mp, merge_passes(len, cap));
      }
      uint32_t tot;
      const uint32_t ex = block_exclusive_add<NT>(v, tot, warp_s);
      const uint64_t e64 = carry_s + ex;
      if (j < nj) item_prefix[j] = static_cast<int32_t>(e64 < capi ? e64 : capi);
      __syncthreads();
      if (tid == 0) carry_s += tot;
      __syncthreads();
    }
    atomicMax(&maxp_s, mp);
    __syncthreads();
    if (tid == 0) {
      const uint64_t total = carry_s < capi ? carry_s : capi;
      item_prefix[nj] = static_cast<int32_t>(total);
      ws.ctr[kCtrItems] = static_cast<uint32_t>(total);
      ws.ctr[kCtrPasses] = static_cast<uint32_t>(maxp_s);
    }
  }
  grid_barrier(ws.ctr);
  const int64_t total = ld_volatile(&ws.ctr[kCtrItems]);
  const int maxp = static_cast<int>(ld_volatile(&ws.ctr[kCtrPasses]));
  for (int64_t j = blockIdx.x; j < nj; j += G) {
    const int64_t p0 = item_prefix[j], p1 = item_prefix[j + 1];
    for (int64_t c = tid; c < p1 - p0; c += NT) item_job[p0 + c] = static_cast<int32_t>(j);
  }
  grid_barrier(ws.ctr);

  K *Xk = reinterpret_cast<K *>(smem);
  uint32_t *Xv = reinterpret_cast<uint32_t *>(smem + MS::kKeysIn);
  K *Ok = reinterpret_cast<K *>(smem + (MS::kIn + 15) / 16 * 16);
  uint32_t *Ov = reinterpret_cast<uint32_t *>(Ok + MS::OSLOTS);

  // Per-item descriptors written by the partition phase, so that the merge
  // phase needs one round of independent loads per item, prefetched while
  // the previous item is merged: {start of run A, la, lb, first output d0}
  // and {instance, flags: 1 = reads tmp, 2 = merges this pass}.
  int4 *desc = ws.item_desc;
  // Two descriptor slots: the CTA reads slot k & 1 for its k-th item while
  // thread 0 fills the other with the next item's descriptor.
  __shared__ int4 slot_d[2], slot_m[2];
  __shared__ uint32_t slot_s0[2], slot_s1[2];

  for (int p = 0; p < maxp; ++p) {
    const int64_t R = cap << p;  // run length this pass merges
    // ---- partition: one half-warp per item (a grid of 3 CTAs per SM has
    // more half-warps than a 2^24-pair problem has items, so no group
    // searches twice) ---------------------------------------------------------
    constexpr int kGroups = 2 * kMWarps;  // half-warps per CTA
    const int grp = tid >> 4, gl = tid & 15;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * kGroups + grp; i < total;
         i += G * kGroups) {
      const int32_t j = item_job[i];
      const int4 jb = jobs[j];
      const int64_t len = jb.y - jb.x;
      const int np = merge_passes(len, cap);
      if (p >= np) {
        if (gl == 0) desc[2 * i + 1] = make_int4(jb.w, 0, 0, 0);
        continue;
      }
      const int64_t o = (i - item_prefix[j]) * static_cast<int64_t>(T);
      const int64_t ps = o / (2 * R) * (2 * R);
      const int64_t la = min(R, len - ps);
      const int64_t lb = min(R, len - ps - la);
      const SideBuffers<K> B = sp(jb.w);
      const int from_tmp = (np - p) & 1;
      const K *src = from_tmp ? B.tmp_keys : B.keys;
      const int64_t s =
          group_merge_split<16>(src + jb.x + ps, la, src + jb.x + ps + la, lb, o - ps);
      if (gl == 0) {
        split[i] = static_cast<uint32_t>(s);
        desc[2 * i] = make_int4(static_cast<int32_t>(jb.x + ps), static_cast<int32_t>(la),
                                static_cast<int32_t>(lb), static_cast<int32_t>(o - ps));
        desc[2 * i + 1] = make_int4(jb.w, from_tmp | 2, 0, 0);
      }
    }
    grid_barrier(ws.ctr);

    // ---- merge: one CTA per item ------------------------------------------
    int4 nd = make_int4(0, 0, 0, 0), nm = make_int4(0, 0, 0, 0);
    uint32_t ns0 = 0, ns1 = 0;
    auto fetch = [&](int64_t i) {
      nd = desc[2 * i];
      nm = desc[2 * i + 1];
      ns0 = split[i];
      ns1 = i + 1 < total ? split[i + 1] : 0u;
    };
    auto publish = [&](int c) {
      slot_d[c] = nd;
      slot_m[c] = nm;
      slot_s0[c] = ns0;
      slot_s1[c] = ns1;
    };
    if (tid == 0 && blockIdx.x < total) {
      fetch(blockIdx.x);
      publish(0);
    }
    __syncthreads();
    int k = 0;
    for (int64_t i = blockIdx.x; i < total; i += G, ++k) {
      const int c = k & 1;
      const int4 dd = slot_d[c], mm = slot_m[c];
      const uint32_t s0u = slot_s0[c], s1u = slot_s1[c];
      const bool more = i + G < total;
      if (tid == 0 && more) fetch(i + G);  // in flight while this item is merged
      // Two barriers per item: after the window loads, and after the merge
      // into the staging buffer (thread 0 publishes the next descriptor
      // before it).  The next item's loads write only the windows, which no
      // thread reads once past the second barrier.
      if (mm.y & 2) {
        const int64_t la = dd.y, lb = dd.z, d0 = dd.w;
        const int64_t d1 = min(d0 + T, la + lb);
        const int64_t s0 = s0u;
        const int64_t s1 = d1 == la + lb ? la : static_cast<int64_t>(s1u);
        const int wa = static_cast<int>(s1 - s0);
        const int m = static_cast<int>(d1 - d0);
        const int wb = m - wa;
        const SideBuffers<K> B = sp(mm.x);
        const bool from_tmp = (mm.y & 1) != 0;
        const int64_t a0 = dd.x;
        const K *sk = (from_tmp ? B.tmp_keys : B.keys) + a0;
        const uint32_t *sv = PAIRS ? (from_tmp ? B.tmp_vals : B.vals) + a0 : nullptr;
        K *dk = (from_tmp ? B.keys : B.tmp_keys) + a0 + d0;
        uint32_t *dv = PAIRS ? (from_tmp ? B.vals : B.tmp_vals) + a0 + d0 : nullptr;
        // Windows: A[s0, s1) at X[0, wa), B[d0 - s0, d1 - s1) at X[wa, m)
        // (element x at slot xslot(x)).
        if (wa >= 0 && wb >= 0 && m <= T) {  // always, for well-formed offsets
          if constexpr (PAIRS && sizeof(K) == 4) {
            // 32-bit keys and values: all four windows in one round.
            const uint32_t *ku = reinterpret_cast<const uint32_t *>(sk);
            uint32_t *xk = reinterpret_cast<uint32_t *>(Xk);
            const uint32_t *src4[4] = {ku + s0, ku + la + (d0 - s0), sv + s0, sv + la + (d0 - s0)};
            const int len4[4] = {wa, wb, wa, wb};
            load_ranges<NT, 2, 4>(src4, len4, [&](int r, int x, uint32_t v) {
              const int at = MS::xslot(x + (r & 1 ? wa : 0));
              if (r < 2) xk[at] = v; else Xv[at] = v;
            });
          } else {
            const K *ks[2] = {sk + s0, sk + la + (d0 - s0)};
            const int kl[2] = {wa, wb};
            load_ranges<NT, 4, 2>(ks, kl, [&](int r, int x, K k) { Xk[MS::xslot(x + (r ? wa : 0))] = k; });
            if constexpr (PAIRS) {
              const uint32_t *vs[2] = {sv + s0, sv + la + (d0 - s0)};
              const int vl[2] = {wa, wb};
              load_ranges<NT, 4, 2>(vs, vl, [&](int r, int x, uint32_t v) {
                Xv[MS::xslot(x + (r ? wa : 0))] = v;
              });
            }
          }
          __syncthreads();
          const int dt = tid * KPT;
          if (dt < m) {
            int lo = dt > wb ? dt - wb : 0;
            int hi = dt < wa ? dt : wa;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (Ord::to_bits(Xk[MS::xslot(mid)]) <= Ord::to_bits(Xk[MS::xslot(wa + dt - 1 - mid)]))
                lo = mid + 1;
              else hi = mid;
            }
            // The heads of both windows stay in registers: one key and one
            // value read from shared memory per output.
            int ai = lo, bi = dt - lo;
            K av = Xk[MS::xslot(ai < wa ? ai : 0)];
            K bv = Xk[MS::xslot(bi < wb ? wa + bi : 0)];
            auto step = [&](int pos) {
              const bool take_a =
                  ai < wa && (bi >= wb || Ord::to_bits(av) <= Ord::to_bits(bv));
              const int x = take_a ? ai : wa + bi;
              Ok[MS::oslot(pos)] = take_a ? av : bv;
              if constexpr (PAIRS) Ov[MS::oslot(pos)] = Xv[MS::xslot(x)];
              ai += take_a;
              bi += !take_a;
              // Next head of the side just consumed (any in-range slot when
              // that side is exhausted: it is never compared again).
              const int nx = take_a ? (ai < wa ? ai : 0) : (bi < wb ? wa + bi : 0);
              const K nv = Xk[MS::xslot(nx)];
              av = take_a ? nv : av;
              bv = take_a ? bv : nv;
            };
            if (__all_sync(__activemask(), dt + KPT <= m && ai + KPT < wa && bi + KPT < wb)) {
              // For every thread of the warp: neither window can run out
              // within its KPT outputs, so no end-of-window tests (the last
              // look-ahead reads at most element wa - 1 or m - 1).  Decided
              // per warp, so warps do not diverge.
#pragma unroll
              for (int q = 0; q < KPT; ++q) {
                const int pos = dt + q;
                const bool take_a = Ord::to_bits(av) <= Ord::to_bits(bv);
                const int x = take_a ? ai : wa + bi;
                Ok[MS::oslot(pos)] = take_a ? av : bv;
                if constexpr (PAIRS) Ov[MS::oslot(pos)] = Xv[MS::xslot(x)];
                ai += take_a;
                bi += !take_a;
                const K nv = Xk[MS::xslot(take_a ? ai : wa + bi)];
                av = take_a ? nv : av;
                bv = take_a ? bv : nv;
              }
            } else if (dt + KPT <= m) {
#pragma unroll
              for (int q = 0; q < KPT; ++q) step(dt + q);
            } else {
#pragma unroll
              for (int q = 0; q < KPT; ++q)
                if (dt + q < m) step(dt + q);
            }
          }
          if (tid == 0 && more) publish(c ^ 1);
          __syncthreads();
          // Start moving the next item's windows into L2 while this one is
          // stored.
          if (more && (slot_m[c ^ 1].y & 2)) {
            const int4 nd2 = slot_d[c ^ 1], nm2 = slot_m[c ^ 1];
            const int64_t nla = nd2.y, nlb = nd2.z, nd0 = nd2.w;
            const int64_t nd1 = min(nd0 + T, nla + nlb);
            const int64_t ns0 = slot_s0[c ^ 1];
            const int64_t ns1 = nd1 == nla + nlb ? nla : static_cast<int64_t>(slot_s1[c ^ 1]);
            if (ns1 >= ns0 && nd1 - nd0 >= ns1 - ns0) {
              const SideBuffers<K> NB = sp(nm2.x);
              const bool nt = (nm2.y & 1) != 0;
              const K *nk = (nt ? NB.tmp_keys : NB.keys) + nd2.x;
              prefetch_l2<NT>(nk + ns0, ns1 - ns0);
              prefetch_l2<NT>(nk + nla + (nd0 - ns0), (nd1 - nd0) - (ns1 - ns0));
              if constexpr (PAIRS) {
                const uint32_t *nv = (nt ? NB.tmp_vals : NB.vals) + nd2.x;
                prefetch_l2<NT>(nv + ns0, ns1 - ns0);
                prefetch_l2<NT>(nv + nla + (nd0 - ns0), (nd1 - nd0) - (ns1 - ns0));
              }
            }
          }
          store_range<NT>(dk, m, [&](int x) { return Ok[MS::oslot(x)]; });
          if constexpr (PAIRS) store_range<NT>(dv, m, [&](int x) { return Ov[MS::oslot(x)]; });
          continue;
        }
      }
      if (tid == 0 && more) publish(c ^ 1);
      __syncthreads();
    }
    grid_barrier(ws.ctr);
  }
}

}  // namespace segsort
