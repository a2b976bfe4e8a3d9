// ORACLE -- test infrastructure only.  This file is the CPU checker of the
// segmented sort: the GPU library never links, loads or calls it.  It is
// imported only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline leg.
//
// It restates the reference's correctness oracle:
//   * src/mseq.cu:44-49 `segmented_sorting`: for every segment i,
//     std::stable_sort(&vec[seg[i]], &vec[seg[i+1]]) on the keys;
//   * src/bb_segsort/main.cu:152-173 `gold_segsort`: the same per-segment
//     stable sort on (key, value) pairs, comparing keys only, so equal keys
//     keep their input order and values travel with their keys.
// Keys are compared through the order-preserving unsigned bits that the GPU
// library uses (identity for unsigned keys, sign-bit flip for signed keys,
// and for floats all bits flipped when negative, else only the sign bit),
// so signed and float keys -- including -0.0/+0.0 and NaNs -- have one
// well-defined order.  Offsets follow the library's contract: CSR,
// segment i = [off[i], off[i+1]), every offset clamped into [0, n] and a
// segment whose end is below its begin treated as empty.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

namespace {

inline uint32_t bits_of(uint32_t k) { return k; }
inline uint32_t bits_of(int32_t k) { return static_cast<uint32_t>(k) ^ 0x80000000u; }
inline uint32_t bits_of(float k) {
  uint32_t u;
  std::memcpy(&u, &k, 4);
  return u ^ ((u & 0x80000000u) ? 0xFFFFFFFFu : 0x80000000u);
}
inline uint64_t bits_of(uint64_t k) { return k; }

inline int64_t clamp_off(int64_t v, int64_t n) { return v < 0 ? 0 : (v > n ? n : v); }

// One segment [b, e): stable sort of (key, value) by the key's order bits
// (src/bb_segsort/main.cu:166-167 -- stable_sort with a key-only comparator).
template <typename K>
void sort_segment(K *keys, uint32_t *vals, int64_t b, int64_t e) {
  if (e - b < 2) return;
  if (vals == nullptr) {
    // src/mseq.cu:47 -- std::stable_sort on the keys alone.
    std::stable_sort(keys + b, keys + e,
                     [](const K &x, const K &y) { return bits_of(x) < bits_of(y); });
    return;
  }
  std::vector<std::pair<K, uint32_t>> pairs;
  pairs.reserve(static_cast<size_t>(e - b));
  for (int64_t i = b; i < e; ++i) pairs.emplace_back(keys[i], vals[i]);
  std::stable_sort(pairs.begin(), pairs.end(),
                   [](const std::pair<K, uint32_t> &x, const std::pair<K, uint32_t> &y) {
                     return bits_of(x.first) < bits_of(y.first);
                   });
  for (int64_t i = b; i < e; ++i) {
    keys[i] = pairs[static_cast<size_t>(i - b)].first;
    vals[i] = pairs[static_cast<size_t>(i - b)].second;
  }
}

// Sequential loop over the segments, as src/mseq.cu:46-48.
template <typename K>
void segsort_range(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int64_t s0,
                   int64_t s1) {
  for (int64_t s = s0; s < s1; ++s) {
    const int64_t b = clamp_off(off[s], n);
    const int64_t e = clamp_off(off[s + 1], n);
    if (e > b) sort_segment(keys, vals, b, e);
  }
}

// Segments split into `threads` contiguous groups of about equal element
// count; each group is sorted by one std::thread.  Same result as the
// sequential loop (segments are independent).
template <typename K>
void segsort_mt(K *keys, uint32_t *vals, int64_t n, const int32_t *off, int32_t nseg,
                int threads) {
  if (threads <= 1 || nseg < 2) {
    segsort_range(keys, vals, n, off, 0, nseg);
    return;
  }
  std::vector<int64_t> cut(static_cast<size_t>(threads) + 1, nseg);
  cut[0] = 0;
  const int64_t first = clamp_off(off[0], n), last = clamp_off(off[nseg], n);
  const int64_t span = last > first ? last - first : 0;
  int64_t s = 0;
  for (int t = 1; t < threads; ++t) {
    const int64_t target = first + span * t / threads;
    while (s < nseg && clamp_off(off[s], n) < target) ++s;
    cut[static_cast<size_t>(t)] = s;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    const int64_t a = cut[static_cast<size_t>(t)], b = cut[static_cast<size_t>(t) + 1];
    if (b > a) pool.emplace_back([=] { segsort_range(keys, vals, n, off, a, b); });
  }
  for (auto &th : pool) th.join();
}

}  // namespace

extern "C" {

void oracle_segsort_keys_u32(uint32_t *k, int64_t n, const int32_t *o, int32_t ns, int threads) {
  segsort_mt(k, nullptr, n, o, ns, threads);
}
void oracle_segsort_keys_i32(int32_t *k, int64_t n, const int32_t *o, int32_t ns, int threads) {
  segsort_mt(k, nullptr, n, o, ns, threads);
}
void oracle_segsort_keys_f32(float *k, int64_t n, const int32_t *o, int32_t ns, int threads) {
  segsort_mt(k, nullptr, n, o, ns, threads);
}
void oracle_segsort_keys_u64(uint64_t *k, int64_t n, const int32_t *o, int32_t ns, int threads) {
  segsort_mt(k, nullptr, n, o, ns, threads);
}
void oracle_segsort_pairs_u32(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                              int threads) {
  segsort_mt(k, v, n, o, ns, threads);
}
void oracle_segsort_pairs_i32(int32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                              int threads) {
  segsort_mt(k, v, n, o, ns, threads);
}
void oracle_segsort_pairs_f32(float *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                              int threads) {
  segsort_mt(k, v, n, o, ns, threads);
}
void oracle_segsort_pairs_u64(uint64_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns,
                              int threads) {
  segsort_mt(k, v, n, o, ns, threads);
}

}  // extern "C"
