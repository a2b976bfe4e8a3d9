#!/bin/bash
# Builds baseline/ref_gpu_bench.exe (the reference GPU variants' timing
# harness) for sm_103a from baseline/_ref (see setup_ref.sh).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 --expt-relaxed-constexpr \
  --expt-extended-lambda -w -I"$HERE/_ref" -o "$HERE/ref_gpu_bench.exe" "$HERE/ref_gpu_bench.cu"
