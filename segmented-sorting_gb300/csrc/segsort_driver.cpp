// Bench driver with the reference drivers' command-line contract:
//
//   ./segsort_driver.exe [options] < instance.in
//
// Input is the reference's instance text (utils/gen_equal.cpp:108-114,
// read as in src/mseq.cu:57-67): the number of segments, the nseg+1 segment
// offsets, the number of keys, the keys.  Output, as the reference drivers:
//   ELAPSED_TIME=0  the sorted keys in the format of src/mseq.cu:27-33
//                   (a newline, every key followed by a space, a newline);
//   ELAPSED_TIME=1  one line per execution with the milliseconds of the sort
//                   call, timed with cudaEvents around the call only
//                   (src/mseq.cu:80-89), EXECUTIONS times.
// So scripts/exec.sh, scripts/test.sh, scripts/results.sh and utils/parser
// run against it unchanged.  ELAPSED_TIME and EXECUTIONS are compile-time
// defaults (as in src/Makefile:11-86) that the options below override.
//
// Options:
//   --pairs           sort (key, value) pairs with value = input index
//                     (the convention of src/radixseg.cu:89); default keys only
//   --type T          key type u32 (default), i32, f32 or u64
//   --heads           pass heads-only offsets to the *_heads entry point
//   --time / --print  force timing output / sorted-key output
//   --execs N         executions per run
//   --print-values    after the keys, print the values line (with --pairs)
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "segsort.h"

#ifndef ELAPSED_TIME
#define ELAPSED_TIME 0
#endif
#ifndef EXECUTIONS
#define EXECUTIONS 1
#endif

namespace {

void die(const char *what, const char *detail) {
  std::fprintf(stderr, "segsort_driver: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
  std::exit(1);
}

void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) die(what, cudaGetErrorString(e));
}

// Whole-stdin tokenizer (scanf is too slow for 2^25-key instances).
struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  Reader() {
    char tmp[1 << 16];
    size_t r;
    while ((r = std::fread(tmp, 1, sizeof(tmp), stdin)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    buf.push_back('\0');
  }
  const char *next() {
    while (pos < buf.size() && (buf[pos] == ' ' || buf[pos] == '\n' || buf[pos] == '\r' ||
                                buf[pos] == '\t'))
      ++pos;
    if (pos >= buf.size() - 1) return nullptr;
    const char *s = &buf[pos];
    while (pos < buf.size() && buf[pos] != ' ' && buf[pos] != '\n' && buf[pos] != '\r' &&
           buf[pos] != '\t' && buf[pos] != '\0')
      ++pos;
    return s;
  }
  long long next_int() {
    const char *s = next();
    if (!s) die("truncated input", nullptr);
    return std::strtoll(s, nullptr, 10);
  }
};

template <typename K>
K parse_key(const char *s);
template <> uint32_t parse_key<uint32_t>(const char *s) {
  return static_cast<uint32_t>(std::strtoll(s, nullptr, 10));
}
template <> int32_t parse_key<int32_t>(const char *s) {
  return static_cast<int32_t>(std::strtoll(s, nullptr, 10));
}
template <> float parse_key<float>(const char *s) { return std::strtof(s, nullptr); }
template <> uint64_t parse_key<uint64_t>(const char *s) { return std::strtoull(s, nullptr, 10); }

template <typename K> void print_key(FILE *f, K k);
template <> void print_key<uint32_t>(FILE *f, uint32_t k) { std::fprintf(f, "%u ", k); }
template <> void print_key<int32_t>(FILE *f, int32_t k) { std::fprintf(f, "%d ", k); }
template <> void print_key<float>(FILE *f, float k) { std::fprintf(f, "%.9g ", k); }
template <> void print_key<uint64_t>(FILE *f, uint64_t k) {
  std::fprintf(f, "%llu ", static_cast<unsigned long long>(k));
}

int call(uint32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns, bool heads,
         cudaStream_t s) {
  auto st = reinterpret_cast<segsort_stream_t>(s);
  if (heads) return v ? segsort_pairs_u32_heads(k, v, n, o, ns, st) : segsort_keys_u32_heads(k, n, o, ns, st);
  return v ? segsort_pairs_u32(k, v, n, o, ns, st) : segsort_keys_u32(k, n, o, ns, st);
}
int call(int32_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns, bool,
         cudaStream_t s) {
  auto st = reinterpret_cast<segsort_stream_t>(s);
  return v ? segsort_pairs_i32(k, v, n, o, ns, st) : segsort_keys_i32(k, n, o, ns, st);
}
int call(float *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns, bool, cudaStream_t s) {
  auto st = reinterpret_cast<segsort_stream_t>(s);
  return v ? segsort_pairs_f32(k, v, n, o, ns, st) : segsort_keys_f32(k, n, o, ns, st);
}
int call(uint64_t *k, uint32_t *v, int64_t n, const int32_t *o, int32_t ns, bool,
         cudaStream_t s) {
  auto st = reinterpret_cast<segsort_stream_t>(s);
  return v ? segsort_pairs_u64(k, v, n, o, ns, st) : segsort_keys_u64(k, n, o, ns, st);
}

struct Opts {
  bool pairs = false, heads = false, print_values = false;
  int timed = ELAPSED_TIME;
  int execs = EXECUTIONS;
  std::string type = "u32";
};

template <typename K>
int run(Reader &in, const Opts &opt) {
  const long long nseg = in.next_int();
  if (nseg < 0 || nseg > INT32_MAX - 1) die("bad segment count", nullptr);
  std::vector<int32_t> off(static_cast<size_t>(nseg) + 1);
  for (auto &o : off) o = static_cast<int32_t>(in.next_int());
  const long long n = in.next_int();
  if (n < 0) die("bad element count", nullptr);
  std::vector<K> keys(static_cast<size_t>(n));
  for (auto &k : keys) {
    const char *s = in.next();
    if (!s) die("truncated key list", nullptr);
    k = parse_key<K>(s);
  }
  std::vector<uint32_t> vals;
  if (opt.pairs) {
    vals.resize(static_cast<size_t>(n));
    for (size_t i = 0; i < vals.size(); ++i) vals[i] = static_cast<uint32_t>(i);
  }

  K *d_keys = nullptr;
  uint32_t *d_vals = nullptr;
  int32_t *d_off = nullptr;
  const size_t kb = sizeof(K) * static_cast<size_t>(n), vb = 4 * static_cast<size_t>(n);
  check_cuda(cudaMalloc(&d_keys, kb ? kb : 1), "cudaMalloc keys");
  if (opt.pairs) check_cuda(cudaMalloc(&d_vals, vb ? vb : 1), "cudaMalloc values");
  check_cuda(cudaMalloc(&d_off, off.size() * 4), "cudaMalloc offsets");
  // Heads-only offsets are the first nseg entries of the same array.
  check_cuda(cudaMemcpy(d_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice), "copy offsets");

  cudaStream_t stream;
  check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
  cudaEvent_t start, stop;
  check_cuda(cudaEventCreate(&start), "event");
  check_cuda(cudaEventCreate(&stop), "event");

  for (int e = 0; e < opt.execs; ++e) {
    check_cuda(cudaMemcpyAsync(d_keys, keys.data(), kb, cudaMemcpyHostToDevice, stream), "copy keys");
    if (opt.pairs)
      check_cuda(cudaMemcpyAsync(d_vals, vals.data(), vb, cudaMemcpyHostToDevice, stream), "copy values");
    check_cuda(cudaEventRecord(start, stream), "record");
    const int rc = call(d_keys, d_vals, n, d_off, static_cast<int32_t>(nseg), opt.heads, stream);
    check_cuda(cudaEventRecord(stop, stream), "record");
    if (rc != SEGSORT_OK) die("segsort call failed", segsort_error_string(rc));
    check_cuda(cudaEventSynchronize(stop), "sync");
    if (opt.timed) {
      float ms = 0.f;
      check_cuda(cudaEventElapsedTime(&ms, start, stop), "elapsed");
      std::printf("%g\n", ms);
    }
  }
  const int st = segsort_device_status(1);
  if (st != SEGSORT_OK) die("device status", segsort_error_string(st));

  if (!opt.timed) {
    std::vector<K> out(static_cast<size_t>(n));
    check_cuda(cudaMemcpy(out.data(), d_keys, kb, cudaMemcpyDeviceToHost), "copy back");
    std::fputc('\n', stdout);
    for (const K &k : out) print_key<K>(stdout, k);
    std::fputc('\n', stdout);
    if (opt.pairs && opt.print_values) {
      std::vector<uint32_t> vo(static_cast<size_t>(n));
      check_cuda(cudaMemcpy(vo.data(), d_vals, vb, cudaMemcpyDeviceToHost), "copy back");
      for (uint32_t v : vo) std::fprintf(stdout, "%u ", v);
      std::fputc('\n', stdout);
    }
  }
  cudaFree(d_keys);
  cudaFree(d_vals);
  cudaFree(d_off);
  cudaEventDestroy(start);
  cudaEventDestroy(stop);
  cudaStreamDestroy(stream);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  Opts opt;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--pairs") opt.pairs = true;
    else if (a == "--heads") opt.heads = true;
    else if (a == "--time") opt.timed = 1;
    else if (a == "--print") opt.timed = 0;
    else if (a == "--print-values") opt.print_values = true;
    else if (a == "--execs" && i + 1 < argc) opt.execs = std::atoi(argv[++i]);
    else if (a == "--type" && i + 1 < argc) opt.type = argv[++i];
    else die("unknown option", a.c_str());
  }
  if (opt.execs < 1) opt.execs = 1;
  if (opt.heads && opt.type != "u32") die("--heads supports u32 keys only", nullptr);
  Reader in;
  if (opt.type == "u32") return run<uint32_t>(in, opt);
  if (opt.type == "i32") return run<int32_t>(in, opt);
  if (opt.type == "f32") return run<float>(in, opt);
  if (opt.type == "u64") return run<uint64_t>(in, opt);
  die("unknown --type", opt.type.c_str());
  return 1;
}
