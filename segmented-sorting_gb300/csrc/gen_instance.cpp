// Seeded instance generator writing the reference's instance text format
// (utils/gen_equal.cpp:108-114, utils/gen_diff.cpp:63-69):
//     nseg \n off_0 ... off_nseg \n n \n key_0 ... key_{n-1} \n
//
//   gen_instance.exe equal <nseg> <segment_size> [opts]   (as utils/gen_equal.cpp)
//   gen_instance.exe diff  <nseg> <n> [opts]              (as utils/gen_diff.cpp)
//   gen_instance.exe lognormal <n> [opts]                 (uneven segments)
// Invoked through a link named equal.exe or diff.exe, the first word may be
// omitted, so scripts/genequalseg.sh and scripts/gendiffseg.sh run unchanged.
//
// Options: --binary (write the binary instance format of segsort_driver.cpp),
//          --bits B (keys uniform in [0, 2^B), default 12 as utils/Makefile:1;
//          B = 32 for the full range), --seed S (default 1), --order
//          rand|asc|desc|randminmax (utils/gen_equal.cpp:18-92),
//          --mu M --sigma S --max L --empty F (lognormal lengths).
//
// Unlike the reference, which seeds rand() with time(NULL)
// (utils/gen_equal.cpp:107), every value is a function of (seed, index):
// key i = top B bits of splitmix64(seed * 0x9E3779B97F4A7C15 + i + 1), the
// same counter-based stream the Python generator instances.py uses, so an
// instance is reproducible on every machine.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Counter-based stream: value i of stream (seed, lane).
uint64_t draw(uint64_t seed, uint64_t lane, uint64_t i) {
  return splitmix64(seed * 0x9E3779B97F4A7C15ull + lane * 0xD1B54A32D192ED03ull + i + 1);
}

double unit(uint64_t r) { return (static_cast<double>(r >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

uint64_t key_of(uint64_t seed, uint64_t i, int bits) {
  const uint64_t r = draw(seed, 0, i);
  return bits >= 64 ? r : (r >> (64 - bits));
}

void usage() {
  std::fprintf(stderr,
               "usage: gen_instance.exe equal <nseg> <segment_size> | diff <nseg> <n> | "
               "lognormal <n>  [--binary] [--bits B] [--seed S] [--order rand|asc|desc|randminmax] "
               "[--mu M] [--sigma S] [--max L] [--empty F]\n");
  std::exit(1);
}

// Binary instance (read by segsort_driver.exe): 32-byte header {"SGSB",
// version 1, key bytes, key kind 0 = unsigned, nseg, n}, nseg+1 int32
// offsets, zero padding to a multiple of 8 bytes, n little-endian keys
// (uint32 for bits <= 32, uint64 otherwise).
void emit_binary(const std::vector<int64_t> &off, const std::vector<uint64_t> &keys, int bits) {
  const uint32_t key_bytes = bits <= 32 ? 4 : 8;
  const uint32_t head[4] = {0, 1, key_bytes, 0};
  const uint64_t counts[2] = {off.size() - 1, keys.size()};
  std::fwrite("SGSB", 1, 4, stdout);
  std::fwrite(head + 1, 4, 3, stdout);
  std::fwrite(counts, 8, 2, stdout);
  std::vector<int32_t> o32(off.begin(), off.end());
  std::fwrite(o32.data(), 4, o32.size(), stdout);
  const size_t pad = (8 - (32 + o32.size() * 4) % 8) % 8;
  const char zeros[8] = {0};
  std::fwrite(zeros, 1, pad, stdout);
  if (key_bytes == 4) {
    std::vector<uint32_t> k32(keys.begin(), keys.end());
    std::fwrite(k32.data(), 4, k32.size(), stdout);
  } else {
    std::fwrite(keys.data(), 8, keys.size(), stdout);
  }
}

void emit(const std::vector<int64_t> &off, const std::vector<uint64_t> &keys) {
  std::printf("%zu\n", off.size() - 1);
  for (int64_t o : off) std::printf("%lld ", static_cast<long long>(o));
  std::printf("\n%zu\n", keys.size());
  for (uint64_t k : keys) std::printf("%llu ", static_cast<unsigned long long>(k));
  std::printf("\n");
}

}  // namespace

int main(int argc, char **argv) {
  std::vector<std::string> args(argv + 1, argv + argc);
  std::string prog = argv[0];
  const size_t slash = prog.find_last_of('/');
  if (slash != std::string::npos) prog = prog.substr(slash + 1);
  std::string mode;
  if (prog == "equal.exe") mode = "equal";
  else if (prog == "diff.exe") mode = "diff";
  if (!args.empty() && (args[0] == "equal" || args[0] == "diff" || args[0] == "lognormal")) {
    mode = args[0];
    args.erase(args.begin());
  }
  if (mode.empty()) usage();

  int bits = 12;
  uint64_t seed = 1;
  std::string order = "rand";
  bool binary = false;
  double mu = 4.0, sigma = 2.5, empty_frac = 0.01;
  int64_t max_len = int64_t{1} << 22;
  std::vector<std::string> pos;
  for (size_t i = 0; i < args.size(); ++i) {
    const std::string &a = args[i];
    auto val = [&]() -> std::string {
      if (i + 1 >= args.size()) usage();
      return args[++i];
    };
    if (a == "--binary") binary = true;
    else if (a == "--bits") bits = std::atoi(val().c_str());
    else if (a == "--seed") seed = std::strtoull(val().c_str(), nullptr, 10);
    else if (a == "--order") order = val();
    else if (a == "--mu") mu = std::atof(val().c_str());
    else if (a == "--sigma") sigma = std::atof(val().c_str());
    else if (a == "--max") max_len = std::atoll(val().c_str());
    else if (a == "--empty") empty_frac = std::atof(val().c_str());
    else pos.push_back(a);
  }
  if (bits < 1 || bits > 64) usage();

  std::vector<int64_t> off;
  int64_t n = 0;
  if (mode == "equal") {
    if (pos.size() < 2) usage();
    const int64_t nseg = std::atoll(pos[0].c_str()), size = std::atoll(pos[1].c_str());
    n = nseg * size;
    for (int64_t i = 0; i <= nseg; ++i) off.push_back(i * size);  // utils/gen_equal.cpp:13-16
  } else if (mode == "diff") {
    if (pos.size() < 2) usage();
    const int64_t nseg = std::atoll(pos[0].c_str());
    n = std::atoll(pos[1].c_str());
    if (nseg < 1 || nseg > n) usage();
    // nseg-1 distinct cut points in [1, n), sorted (utils/gen_diff.cpp:11-42).
    std::vector<uint8_t> taken(static_cast<size_t>(n), 0);
    taken[0] = 1;
    off.push_back(0);
    uint64_t i = 0;
    while (static_cast<int64_t>(off.size()) < nseg) {
      const int64_t x = static_cast<int64_t>(draw(seed, 1, i++) % static_cast<uint64_t>(n));
      if (!taken[static_cast<size_t>(x)]) {
        taken[static_cast<size_t>(x)] = 1;
        off.push_back(x);
      }
    }
    std::sort(off.begin(), off.end());
    off.push_back(n);
  } else {  // lognormal
    if (pos.empty()) usage();
    n = std::atoll(pos[0].c_str());
    std::vector<int64_t> lens;
    int64_t sum = 0;
    for (uint64_t i = 0; sum < n; ++i) {
      const double u1 = unit(draw(seed, 2, 2 * i)), u2 = unit(draw(seed, 2, 2 * i + 1));
      const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
      int64_t len = static_cast<int64_t>(std::llround(std::exp(mu + sigma * z)));
      len = std::min<int64_t>(std::max<int64_t>(len, 1), max_len);
      len = std::min(len, n - sum);
      lens.push_back(len);
      sum += len;
    }
    // Insert empty segments: segment i is followed by an empty one with
    // probability empty_frac.
    off.push_back(0);
    int64_t at = 0;
    for (size_t i = 0; i < lens.size(); ++i) {
      at += lens[i];
      off.push_back(at);
      if (unit(draw(seed, 3, i)) < empty_frac) off.push_back(at);
    }
  }

  std::vector<uint64_t> keys(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) keys[static_cast<size_t>(i)] = key_of(seed, static_cast<uint64_t>(i), bits);
  if (order == "asc") {
    std::sort(keys.begin(), keys.end());
  } else if (order == "desc") {
    std::sort(keys.begin(), keys.end(), [](uint64_t a, uint64_t b) { return a > b; });
  } else if (order == "randminmax") {
    // Each segment holds 0 and 2^bits - 1 plus random keys, shuffled
    // (utils/gen_equal.cpp:27-58).
    const uint64_t top = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    for (size_t s = 0; s + 1 < off.size(); ++s) {
      const int64_t b = off[s], e = off[s + 1];
      if (e - b >= 1) keys[static_cast<size_t>(b)] = 0;
      if (e - b >= 2) keys[static_cast<size_t>(b + 1)] = top;
      for (int64_t i = e - 1; i > b; --i) {
        const int64_t j = b + static_cast<int64_t>(draw(seed, 4, static_cast<uint64_t>(i)) %
                                                   static_cast<uint64_t>(i - b + 1));
        std::swap(keys[static_cast<size_t>(i)], keys[static_cast<size_t>(j)]);
      }
    }
  } else if (order != "rand") {
    usage();
  }
  if (binary) emit_binary(off, keys, bits);
  else emit(off, keys);
  return 0;
}
