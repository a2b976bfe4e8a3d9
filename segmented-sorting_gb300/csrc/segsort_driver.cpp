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
// Binary instances (gen_instance.exe --binary) are read as well: a file that
// starts with the magic "SGSB" holds a 32-byte header (magic, version 1, key
// bytes 4 or 8, key kind 0 unsigned / 1 signed / 2 float, nseg and n as
// uint64), the nseg+1 int32 offsets, zero padding to a multiple of 8 bytes
// and the n keys, all little-endian.  When stdin is a regular file it is
// memory-mapped instead of read, and the keys are copied to the GPU straight
// from the mapping; the key type comes from the header.
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

#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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

// All of stdin: memory-mapped when it is a regular file, read otherwise.
// Text instances are tokenised from it (scanf is too slow for 2^25-key
// instances); binary instances are used in place.
struct Reader {
  std::vector<char> buf;
  const char *data = nullptr;
  size_t size = 0;
  void *map = nullptr;
  size_t pos = 0;
  Reader() {
    struct stat st;
    if (fstat(0, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
      map = mmap(nullptr, static_cast<size_t>(st.st_size), PROT_READ, MAP_PRIVATE, 0, 0);
      if (map == MAP_FAILED) map = nullptr;
      if (map) {
        data = static_cast<const char *>(map);
        size = static_cast<size_t>(st.st_size);
        return;
      }
    }
    char tmp[1 << 16];
    size_t r;
    while ((r = std::fread(tmp, 1, sizeof(tmp), stdin)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    data = buf.data();
    size = buf.size();
  }
  ~Reader() {
    if (map) munmap(map, size);
  }
  bool binary() const { return size >= 32 && std::memcmp(data, "SGSB", 4) == 0; }
  static bool space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t'; }
  // Next token as a NUL-terminated copy (tokens are short numbers).
  const char *next() {
    while (pos < size && space(data[pos])) ++pos;
    if (pos >= size) return nullptr;
    size_t len = 0;
    while (pos < size && !space(data[pos]) && data[pos] != '\0' && len + 1 < sizeof(tok))
      tok[len++] = data[pos++];
    while (pos < size && !space(data[pos]) && data[pos] != '\0') ++pos;
    tok[len] = '\0';
    return tok;
  }
  long long next_int() {
    const char *s = next();
    if (!s) die("truncated input", nullptr);
    return std::strtoll(s, nullptr, 10);
  }
  char tok[64];
};

struct BinaryHeader {
  char magic[4];
  uint32_t version, key_bytes, key_kind;
  uint64_t nseg, n;
};
static_assert(sizeof(BinaryHeader) == 32, "binary instance header is 32 bytes");

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
int sort_instance(const int32_t *off_p, long long nseg, const K *keys_p, long long n, const Opts &opt);

template <typename K>
int run(Reader &in, const Opts &opt) {
  if (in.binary()) {
    BinaryHeader h;
    std::memcpy(&h, in.data, sizeof(h));
    if (h.version != 1 || h.key_bytes != sizeof(K)) die("binary instance does not match --type", nullptr);
    if (h.nseg > static_cast<uint64_t>(INT32_MAX - 1) || h.n > (uint64_t{1} << 40))
      die("bad binary header", nullptr);
    const size_t off_at = sizeof(h), off_bytes = (h.nseg + 1) * 4;
    const size_t keys_at = (off_at + off_bytes + 7) / 8 * 8;
    if (keys_at + h.n * sizeof(K) > in.size) die("truncated binary instance", nullptr);
    return sort_instance<K>(reinterpret_cast<const int32_t *>(in.data + off_at),
                            static_cast<long long>(h.nseg),
                            reinterpret_cast<const K *>(in.data + keys_at),
                            static_cast<long long>(h.n), opt);
  }
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
  return sort_instance<K>(off.data(), nseg, keys.data(), n, opt);
}

template <typename K>
int sort_instance(const int32_t *off_p, long long nseg, const K *keys_p, long long n, const Opts &opt) {
  const std::vector<int32_t> off(off_p, off_p + nseg + 1);
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
    check_cuda(cudaMemcpyAsync(d_keys, keys_p, kb, cudaMemcpyHostToDevice, stream), "copy keys");
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
  bool type_given = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--pairs") opt.pairs = true;
    else if (a == "--heads") opt.heads = true;
    else if (a == "--time") opt.timed = 1;
    else if (a == "--print") opt.timed = 0;
    else if (a == "--print-values") opt.print_values = true;
    else if (a == "--execs" && i + 1 < argc) opt.execs = std::atoi(argv[++i]);
    else if (a == "--type" && i + 1 < argc) {
      opt.type = argv[++i];
      type_given = true;
    }
    else die("unknown option", a.c_str());
  }
  if (opt.execs < 1) opt.execs = 1;
  if (opt.heads && opt.type != "u32") die("--heads supports u32 keys only", nullptr);
  Reader in;
  if (in.binary()) {  // the key type comes from the header
    BinaryHeader h;
    std::memcpy(&h, in.data, sizeof(h));
    static const char *kinds4[] = {"u32", "i32", "f32"};
    const std::string t = h.key_bytes == 8 ? "u64" : (h.key_kind < 3 ? kinds4[h.key_kind] : "?");
    if (!type_given) opt.type = t;
    else if (opt.type != t) die("--type does not match the binary instance", t.c_str());
    if (opt.heads && opt.type != "u32") die("--heads supports u32 keys only", nullptr);
  }
  if (opt.type == "u32") return run<uint32_t>(in, opt);
  if (opt.type == "i32") return run<int32_t>(in, opt);
  if (opt.type == "f32") return run<float>(in, opt);
  if (opt.type == "u64") return run<uint64_t>(in, opt);
  die("unknown --type", opt.type.c_str());
  return 1;
}
