#!/bin/bash
# Copies the reference's GPU segmented sorts -- bb_segsort (src/bb_segsort/)
# and moderngpu (lib/moderngpu/) -- into the git-ignored baseline/_ref/, where
# ref_gpu_bench.cu includes them.  Run where the reference checkout is
# mounted; baseline/_ref/ then travels with the repository snapshot to the GPU
# host, where build_ref_gpu_bench.sh compiles the harness.
#
# moderngpu 2.x uses the pre-Volta shuffles (__shfl_up/__shfl_down and
# "shfl.<dir>.b32" in inline PTX, lib/moderngpu/intrinsics.hxx:122,137,170,211-212),
# which ptxas rejects for sm_70 and later; the copy gets their .sync forms.
# Their member mask is the set of lanes active at the call (activemask), not
# the full warp: moderngpu calls them inside lane-subset branches such as
# `if (tid < num_warps)` (cta_scan.hxx:98-104, cta_reduce.hxx:47-53,71-77), and
# a .sync shuffle waits for every lane its mask names, so a full-warp mask
# there waits forever for lanes that never arrive.  That is why an earlier copy
# of this shim (full-warp masks) never finished segmented_sort on GB300.
set -euo pipefail
REF=${1:-${SEGSORT_REF_DIR:-/root/reference}}
HERE="$(cd "$(dirname "$0")" && pwd)"
DST="$HERE/_ref"
rm -rf "$DST/bb_segsort" "$DST/moderngpu"
mkdir -p "$DST"
cp -r "$REF/src/bb_segsort" "$DST/bb_segsort"
cp -r "$REF/lib/moderngpu" "$DST/moderngpu"
sed -i \
  -e 's/__shfl_up(u\.x\[i\], offset, width)/__shfl_up_sync(__activemask(), u.x[i], offset, width)/' \
  -e 's/__shfl_down(u\.x\[i\], offset, width)/__shfl_down_sync(__activemask(), u.x[i], offset, width)/' \
  -e 's/"shfl\."#dir"\.b32 r0|p, %1, %2, %3;"/"{ .reg .b32 am; activemask.b32 am; shfl.sync."#dir".b32 r0|p, %1, %2, %3, am; }"/' \
  -e 's/"shfl\."#dir"\.b32 lo|p, lo, %2, %3;"/"{ .reg .b32 am; activemask.b32 am; shfl.sync."#dir".b32 lo|p, lo, %2, %3, am; }"/' \
  -e 's/"shfl\."#dir"\.b32 hi  , hi, %2, %3;"/"{ .reg .b32 am; activemask.b32 am; shfl.sync."#dir".b32 hi  , hi, %2, %3, am; }"/' \
  "$DST/moderngpu/intrinsics.hxx"
grep -c "activemask" "$DST/moderngpu/intrinsics.hxx"
