#!/bin/bash
# Copies the reference's GPU segmented sorts -- bb_segsort (src/bb_segsort/)
# and moderngpu (lib/moderngpu/) -- into the git-ignored baseline/_ref/, where
# ref_gpu_bench.cu includes them.  Run where the reference checkout is
# mounted; baseline/_ref/ then travels with the repository snapshot to the GPU
# host, where build_ref_gpu_bench.sh compiles the harness.
#
# moderngpu 2.x uses the pre-Volta shuffles (__shfl_up/__shfl_down and
# "shfl.<dir>.b32" in inline PTX, lib/moderngpu/intrinsics.hxx:122,137,170,211-212),
# which ptxas rejects for sm_70 and later; the copy gets their .sync forms with
# a full-warp mask, which is what the old forms did on a converged warp.
set -euo pipefail
REF=${1:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
DST="$HERE/_ref"
rm -rf "$DST/bb_segsort" "$DST/moderngpu"
mkdir -p "$DST"
cp -r "$REF/src/bb_segsort" "$DST/bb_segsort"
cp -r "$REF/lib/moderngpu" "$DST/moderngpu"
sed -i \
  -e 's/__shfl_up(u\.x\[i\], offset, width)/__shfl_up_sync(0xffffffffu, u.x[i], offset, width)/' \
  -e 's/__shfl_down(u\.x\[i\], offset, width)/__shfl_down_sync(0xffffffffu, u.x[i], offset, width)/' \
  -e 's/"shfl\."#dir"\.b32 r0|p, %1, %2, %3;"/"shfl.sync."#dir".b32 r0|p, %1, %2, %3, 0xffffffff;"/' \
  -e 's/"shfl\."#dir"\.b32 lo|p, lo, %2, %3;"/"shfl.sync."#dir".b32 lo|p, lo, %2, %3, 0xffffffff;"/' \
  -e 's/"shfl\."#dir"\.b32 hi  , hi, %2, %3;"/"shfl.sync."#dir".b32 hi  , hi, %2, %3, 0xffffffff;"/' \
  "$DST/moderngpu/intrinsics.hxx"
grep -c "shfl.sync\|_sync(0xffffffffu" "$DST/moderngpu/intrinsics.hxx"
