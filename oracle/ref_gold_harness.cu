// ORACLE -- test infrastructure only.  Runs the reference's own pair oracle
// `gold_segsort` (src/bb_segsort/main.cu:152-173) on one instance, so the
// C++ restatement in segsort_oracle.cpp can be pinned against it.
//
// Built by `make -C oracle ref` into the git-ignored oracle/_ref/ from the
// reference sources where they lie (the include path points into the
// reference checkout); nothing of the reference is copied here.  The
// reference file's own main() is renamed away; only its host template
// gold_segsort is called, so no GPU is needed.
//
// stdin : the reference instance text (nseg, nseg+1 offsets, n, keys)
// stdout: line 1 the keys, line 2 the values, after gold_segsort of
//         (key, value = input index) pairs with the heads-only segment
//         array the reference passes (main.cu:59-63: heads, end of last = n)
#include <cstdio>
#include <vector>

#define main reference_bb_segsort_main
#include "main.cu"
#undef main

int main() {
  unsigned nseg = 0, n = 0;
  if (std::scanf("%u", &nseg) != 1) return 1;
  std::vector<int> seg(nseg + 1);
  for (unsigned i = 0; i <= nseg; ++i)
    if (std::scanf("%d", &seg[i]) != 1) return 1;
  if (std::scanf("%u", &n) != 1) return 1;
  std::vector<unsigned> key(n), val(n);
  for (unsigned i = 0; i < n; ++i) {
    if (std::scanf("%u", &key[i]) != 1) return 1;
    val[i] = i;
  }
  // The reference passes nseg heads; the last segment ends at n.
  std::vector<int> heads(seg.begin(), seg.begin() + nseg);
  gold_segsort(key, val, static_cast<int>(n), heads, static_cast<int>(nseg));
  for (unsigned i = 0; i < n; ++i) std::printf("%u ", key[i]);
  std::printf("\n");
  for (unsigned i = 0; i < n; ++i) std::printf("%u ", val[i]);
  std::printf("\n");
  return 0;
}
