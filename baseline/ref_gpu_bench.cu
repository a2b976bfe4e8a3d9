// Times the reference's GPU segmented sorts on this GPU, through their own
// entry points, on the equal-segment sweep of the benchmark:
//   bb    bb_segsort(keys_d, vals_d, n, d_segs, nseg)      src/bb_segsort/bb_segsort.h:35-36
//   mgpu  mgpu::segmented_sort(keys, vals, n, heads, nseg, less, context)
//         lib/moderngpu/kernel_segsort.hxx:405-415, driven as src/mergeseg.cu:118-119
//         (heads-only offsets; needs the activemask shuffle shim of setup_ref.sh)
//   cub   cub::DeviceSegmentedRadixSort::SortPairs(...)    src/radixseg.cu:121-124 (toolkit CUB)
// and, for context, the toolkit's newer cub::DeviceSegmentedSort::StablePairs
// (not a reference variant):
//   cubss cub::DeviceSegmentedSort::StableSortPairs(...)
// and the reference's prefix-trick variants, restated on the toolkit's CUB and
// Thrust: every key gets its segment index shifted past the largest key's
// most significant bit added, one global sort orders segments and keys at
// once, and the prefix is subtracted again.  Correct only while
// nseg << (msb + 1) fits 32 bits -- the reference's own inputs have 12-bit keys
// (utils/Makefile:1) -- so every line reports "prefix_overflows":
//   fixcub      max (cub::DeviceReduce::Max), add, cub::DeviceRadixSort::SortPairs,
//               subtract                               src/fixcub.cu:47-57,141-165
//   fixpasscub  the same calls, timing only the max/add and subtract passes,
//               as the reference does                  src/fixpasscub.cu:141-150,169-178
//   fixthrust   thrust::max_element, transform, thrust::sort (keys only),
//               transform                              src/fixthrust.cu:84-101
// Their temporary-storage allocations fall inside the timed region, as in the
// reference drivers (src/fixcub.cu:142,154).
//
// --bits B masks the keys to their low B bits (12: the reference's inputs).
//
// Inputs: n uint32 keys from the counter-based stream of
// segmented-sorting_gb300/instances.py (uniform_keys), values = input index,
// equal segments of each length.  Each timing brackets only the library call
// with CUDA events, as the reference drivers do (src/radixseg.cu:121-125);
// bb_segsort's own allocations fall inside its call, as in the reference
// (src/bb_segsort/bb_segsort.h:43-56).  Keys are checked sorted per segment
// after the last repetition.
//
// Build: baseline/build_ref_gpu_bench.sh (needs baseline/_ref from
// baseline/setup_ref.sh).  Output: one JSON line per (variant, length).
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_segmented_radix_sort.cuh>
#include <cub/device/device_segmented_sort.cuh>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/extrema.h>
#include <thrust/sort.h>

#include "bb_segsort/bb_segsort.h"
#include "moderngpu/kernel_segsort.hxx"

namespace {

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(1);
  }
}

__device__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// keys = top `bits` bits of splitmix64(seed * golden + i + 1):
// instances.uniform_keys(n, seed, bits)
__global__ void gen_keys(uint32_t *k, int64_t n, uint64_t seed, int bits) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) k[i] = static_cast<uint32_t>(splitmix64(seed * 0x9E3779B97F4A7C15ull + i + 1) >> (64 - bits));
}

// Segment index of every element (equal segments of len).
__global__ void segment_ids(uint32_t *s, int64_t n, int64_t len) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) s[i] = static_cast<uint32_t>(i / len);
}

// Adds (sign > 0) or subtracts the segment prefix seg << (msb(max) + 1).
__global__ void segment_prefix(uint32_t *k, const uint32_t *seg, int64_t n, const uint32_t *dmax,
                               int sign) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t m = *dmax;
    const int shift = m ? 32 - __clz(m) : 0;
    const uint32_t pre = shift < 32 ? seg[i] << shift : 0u;
    k[i] = sign > 0 ? k[i] + pre : k[i] - pre;
  }
}
__global__ void iota(uint32_t *v, int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) v[i] = static_cast<uint32_t>(i);
}
__global__ void equal_offsets(int *o, int64_t nseg, int64_t len) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i <= nseg) o[i] = static_cast<int>(i * len);
}

unsigned blocks(int64_t n) { return static_cast<unsigned>((n + 255) / 256); }

}  // namespace

int main(int argc, char **argv) {
  std::string variants = "bb,mgpu,cub,cubss,fixcub,fixpasscub,fixthrust";
  int log_n = 24, lo = 1, hi = 20, reps = 3, bits = 32;
  for (int i = 1; i + 1 < argc; i += 2) {
    const std::string a = argv[i];
    if (a == "--variants") variants = argv[i + 1];
    else if (a == "--log-n") log_n = std::atoi(argv[i + 1]);
    else if (a == "--lo") lo = std::atoi(argv[i + 1]);
    else if (a == "--hi") hi = std::atoi(argv[i + 1]);
    else if (a == "--reps") reps = std::atoi(argv[i + 1]);
    else if (a == "--bits") bits = std::atoi(argv[i + 1]);
  }
  const int64_t n = int64_t{1} << log_n;
  uint32_t *keys, *vals, *keys_out, *vals_out;
  int *offs;
  uint32_t *segs, *dmax;
  check(cudaMalloc(&segs, n * 4), "malloc");
  check(cudaMalloc(&dmax, 4), "malloc");
  check(cudaMalloc(&keys, n * 4), "malloc");
  check(cudaMalloc(&vals, n * 4), "malloc");
  check(cudaMalloc(&keys_out, n * 4), "malloc");
  check(cudaMalloc(&vals_out, n * 4), "malloc");
  check(cudaMalloc(&offs, (n + 1) * 4), "malloc");
  mgpu::standard_context_t mgpu_ctx;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  std::vector<uint32_t> host(static_cast<size_t>(n));

  auto has = [&](const char *v) { return ("," + variants + ",").find("," + std::string(v) + ",") != std::string::npos; };

  for (int lg = lo; lg <= hi; ++lg) {
    const int64_t len = int64_t{1} << lg;
    const int64_t nseg = n / len;
    equal_offsets<<<blocks(nseg + 1), 256>>>(offs, nseg, len);
    segment_ids<<<blocks(n), 256>>>(segs, n, len);
    const uint64_t seed = 1000 + lg;
    // The prefix nseg - 1 << (msb + 1) must fit 32 bits (msb of the largest
    // possible key).
    const bool overflows = static_cast<double>(nseg - 1) * std::ldexp(1.0, bits) >= 4294967296.0;
    for (const char *v : {"bb", "mgpu", "cub", "cubss", "fixcub", "fixpasscub", "fixthrust"}) {
      if (!has(v)) continue;
      const std::string var = v;
      // CUB's one-CTA-per-segment radix and moderngpu run only inside the
      // reference's own sweep (scripts/genequalseg.sh:7: at most 2^20 segments).
      if ((var == "cub" || var == "mgpu") && nseg > (int64_t{1} << 20)) {
        std::printf("{\"variant\": \"%s\", \"log_len\": %d, \"n\": %lld, \"unavailable\": "
                    "\"more than 2^20 segments, outside the reference sweep\"}\n",
                    var.c_str(), lg, static_cast<long long>(n));
        continue;
      }
      void *temp = nullptr;
      size_t temp_bytes = 0;
      if (var == "cub") {
        cub::DeviceSegmentedRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, vals, vals_out,
                                                 static_cast<int>(n), static_cast<int>(nseg),
                                                 offs, offs + 1);
        check(cudaMalloc(&temp, temp_bytes), "temp");
      } else if (var == "cubss") {
        cub::DeviceSegmentedSort::StableSortPairs(temp, temp_bytes, keys, keys_out, vals, vals_out,
                                                  static_cast<int>(n), static_cast<int>(nseg),
                                                  offs, offs + 1);
        check(cudaMalloc(&temp, temp_bytes), "temp");
      }
      std::vector<float> ms;
      const uint32_t *result = keys;
      const bool fix = var.rfind("fix", 0) == 0;
      for (int r = 0; r < reps + 1; ++r) {
        gen_keys<<<blocks(n), 256>>>(keys, n, seed, bits);
        iota<<<blocks(n), 256>>>(vals, n);
        check(cudaDeviceSynchronize(), "prepare");
        cudaEventRecord(a);
        if (fix) {
          float pass_ms = 0.f;
          void *rt = nullptr, *st = nullptr;
          size_t rb = 0, sb = 0;
          if (var == "fixthrust") {
            thrust::device_ptr<uint32_t> kp(keys);
            const uint32_t m = *thrust::max_element(thrust::device, kp, kp + n);
            check(cudaMemcpy(dmax, &m, 4, cudaMemcpyHostToDevice), "max");
            segment_prefix<<<blocks(n), 256>>>(keys, segs, n, dmax, 1);
            thrust::sort(thrust::device, kp, kp + n);
            segment_prefix<<<blocks(n), 256>>>(keys, segs, n, dmax, -1);
            result = keys;
          } else {
            cub::DeviceReduce::Max(rt, rb, keys, dmax, static_cast<int>(n));
            check(cudaMalloc(&rt, rb), "temp");
            cub::DeviceReduce::Max(rt, rb, keys, dmax, static_cast<int>(n));
            segment_prefix<<<blocks(n), 256>>>(keys, segs, n, dmax, 1);
            if (var == "fixpasscub") {
              cudaEventRecord(b);
              check(cudaEventSynchronize(b), "pre");
              cudaEventElapsedTime(&pass_ms, a, b);
            }
            cub::DeviceRadixSort::SortPairs(st, sb, keys, keys_out, vals, vals_out, static_cast<int>(n));
            check(cudaMalloc(&st, sb), "temp");
            cub::DeviceRadixSort::SortPairs(st, sb, keys, keys_out, vals, vals_out, static_cast<int>(n));
            if (var == "fixpasscub") cudaEventRecord(a);
            segment_prefix<<<blocks(n), 256>>>(keys_out, segs, n, dmax, -1);
            result = keys_out;
          }
          cudaEventRecord(b);
          check(cudaEventSynchronize(b), var.c_str());
          float t = 0;
          cudaEventElapsedTime(&t, a, b);
          if (rt) cudaFree(rt);
          if (st) cudaFree(st);
          if (r > 0) ms.push_back(t + pass_ms);
          continue;
        }
        if (var == "bb") {
          bb_segsort(keys, vals, static_cast<int>(n), offs, static_cast<int>(nseg));
          result = keys;
        } else if (var == "mgpu") {
          mgpu::segmented_sort(keys, vals, static_cast<int>(n), offs, static_cast<int>(nseg),
                               mgpu::less_t<uint32_t>(), mgpu_ctx);
          result = keys;
        } else if (var == "cub") {
          cub::DeviceSegmentedRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, vals, vals_out,
                                                   static_cast<int>(n), static_cast<int>(nseg),
                                                   offs, offs + 1);
          result = keys_out;
        } else {
          cub::DeviceSegmentedSort::StableSortPairs(temp, temp_bytes, keys, keys_out, vals,
                                                    vals_out, static_cast<int>(n),
                                                    static_cast<int>(nseg), offs, offs + 1);
          result = keys_out;
        }
        cudaEventRecord(b);
        check(cudaEventSynchronize(b), var.c_str());
        float t = 0;
        cudaEventElapsedTime(&t, a, b);
        if (r > 0) ms.push_back(t);
      }
      check(cudaMemcpy(host.data(), result, n * 4, cudaMemcpyDeviceToHost), "copy");
      bool sorted = true;
      for (int64_t i = 1; i < n && sorted; ++i)
        if (i % len != 0 && host[i - 1] > host[i]) sorted = false;
      std::sort(ms.begin(), ms.end());
      const float med = ms[ms.size() / 2];
      std::printf("{\"variant\": \"%s\", \"log_len\": %d, \"n\": %lld, \"bits\": %d, \"ms\": %.5f, "
                  "\"gkeys_s\": %.4f, \"sorted\": %s",
                  var.c_str(), lg, static_cast<long long>(n), bits, med, n / (med * 1e-3) / 1e9,
                  sorted ? "true" : "false");
      if (fix) std::printf(", \"prefix_overflows\": %s", overflows ? "true" : "false");
      if (var == "fixpasscub") std::printf(", \"timed\": \"max/add and subtract passes only\"");
      if (var == "fixthrust") std::printf(", \"values\": \"keys only\"");
      std::printf("}\n");
      std::fflush(stdout);
      if (temp) cudaFree(temp);
    }
  }
  return 0;
}
