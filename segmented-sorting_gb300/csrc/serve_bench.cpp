// Served-form benchmark: a Poisson stream of uint32 key/value segsort
// requests, served once by the continuous-batching server (segsort_server_*)
// and once by a loop that handles one request per plain call
// (copy in, segsort_pairs_u32, copy out, wait), on the same GPU.
//
//   serve_bench.exe [--requests R] [--rates 1000,5000,10000,50000]
//                   [--budget-gb 64] [--seed 7] [--lo-log 10] [--hi-log 24]
//                   [--verify-every V] [--depth 2] [--max-batch 0]
//                   [--max-batch-keys 0]
//
// V defaults to max(40, R / 200): about 200 verified requests whatever R is
// (each holds four pinned result buffers of its own).
//
// Request r: n log-uniform in [2^lo, 2^hi]; segment lengths lognormal(4, 2.5)
// clipped to [1, 2^22], summed to n, 1% empty segments inserted; keys and
// values are a slice of a pinned pool (uniform uint32 keys, values = pool
// index) at a seeded start.  Arrival times: exponential gaps at the given
// rate, from the same seed, so every rate serves the same requests.
// Latency = completion on the host minus the scheduled arrival.  Every
// verify-every'th request writes its result to a buffer of its own; those
// results are compared, bit for bit, between the served run and the
// one-request loop (each request sorted alone); the other requests write
// their results to a shared sink.  One JSON line per rate.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "segsort.h"

namespace {

using Clock = std::chrono::steady_clock;

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
uint64_t draw(uint64_t seed, uint64_t lane, uint64_t i) {
  return splitmix64(seed * 0x9E3779B97F4A7C15ull + lane * 0xD1B54A32D192ED03ull + i + 1);
}
double unit(uint64_t r) { return (static_cast<double>(r >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(1);
  }
}

template <typename T>
T *pinned(size_t count) {
  void *p = nullptr;
  check(cudaHostAlloc(&p, count * sizeof(T), cudaHostAllocDefault), "cudaHostAlloc");
  return static_cast<T *>(p);
}

// Lognormal(mu, sigma) lengths clipped to [1, max_len] summed to n (the last
// one truncated), an empty segment after each with probability empty_frac.
std::vector<int32_t> lognormal_offsets(int64_t n, uint64_t seed) {
  const double mu = 4.0, sigma = 2.5, empty_frac = 0.01;
  const int64_t max_len = int64_t{1} << 22;
  std::vector<int32_t> off{0};
  int64_t sum = 0;
  for (uint64_t i = 0; sum < n; ++i) {
    const double u1 = unit(draw(seed, 2, 2 * i)), u2 = unit(draw(seed, 2, 2 * i + 1));
    const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    int64_t len = static_cast<int64_t>(std::llround(std::exp(mu + sigma * z)));
    len = std::min<int64_t>(std::max<int64_t>(len, 1), max_len);
    len = std::min(len, n - sum);
    sum += len;
    off.push_back(static_cast<int32_t>(sum));
    if (unit(draw(seed, 3, i)) < empty_frac) off.push_back(static_cast<int32_t>(sum));
  }
  return off;
}

struct Req {
  int64_t n;
  int64_t start;  // slice of the pool
  std::vector<int32_t> off;
  int32_t *h_off;  // its place in the pinned arena of every request's offsets
  double arrival_unit;  // arrival time at rate 1 req/s (seconds)
  bool verify;
};

double pct(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const size_t i = std::min(v.size() - 1, static_cast<size_t>(std::ceil(p / 100.0 * v.size())) - 1);
  return v[i];
}

void sleep_until(Clock::time_point t) {
  const auto now = Clock::now();
  if (t > now + std::chrono::microseconds(200)) std::this_thread::sleep_until(t - std::chrono::microseconds(100));
  while (Clock::now() < t) {
  }
}

}  // namespace

int main(int argc, char **argv) {
  int64_t requests = 2000;
  std::vector<double> rates = {1000, 5000, 10000, 50000};
  double budget_gb = 64.0;
  uint64_t seed = 7;
  double lo_log = 10, hi_log = 24;
  int verify_every = 0, depth = 2, max_batch = 0, pool_log = 25;
  int64_t max_batch_keys = 0;
  for (int i = 1; i + 1 < argc; i += 2) {
    const std::string a = argv[i], v = argv[i + 1];
    if (a == "--requests") requests = std::atoll(v.c_str());
    else if (a == "--budget-gb") budget_gb = std::atof(v.c_str());
    else if (a == "--seed") seed = std::strtoull(v.c_str(), nullptr, 10);
    else if (a == "--lo-log") lo_log = std::atof(v.c_str());
    else if (a == "--hi-log") hi_log = std::atof(v.c_str());
    else if (a == "--verify-every") verify_every = std::atoi(v.c_str());
    else if (a == "--depth") depth = std::atoi(v.c_str());
    else if (a == "--max-batch") max_batch = std::atoi(v.c_str());
    else if (a == "--max-batch-keys") max_batch_keys = std::atoll(v.c_str());
    else if (a == "--pool-log") pool_log = std::atoi(v.c_str());
    else if (a == "--rates") {
      rates.clear();
      size_t p = 0;
      while (p < v.size()) {
        size_t q = v.find(',', p);
        if (q == std::string::npos) q = v.size();
        rates.push_back(std::atof(v.substr(p, q - p).c_str()));
        p = q + 1;
      }
    }
  }
  if (verify_every <= 0) verify_every = static_cast<int>(std::max<int64_t>(40, requests / 200));
  check(cudaSetDevice(0), "cudaSetDevice");

  // ---- requests ------------------------------------------------------------
  const int64_t pool_n = int64_t{1} << pool_log;
  uint32_t *pool_k = pinned<uint32_t>(pool_n), *pool_v = pinned<uint32_t>(pool_n);
  for (int64_t i = 0; i < pool_n; ++i) {
    pool_k[i] = static_cast<uint32_t>(draw(seed, 0, i) >> 32);
    pool_v[i] = static_cast<uint32_t>(i);
  }
  std::vector<Req> reqs(requests);
  double t = 0.0;
  int64_t total_keys = 0, max_n = 0;
  for (int64_t r = 0; r < requests; ++r) {
    Req &q = reqs[r];
    const double u = unit(draw(seed, 8, 3 * r));
    q.n = std::min<int64_t>(pool_n, static_cast<int64_t>(std::llround(std::exp2(lo_log + (hi_log - lo_log) * u))));
    q.start = static_cast<int64_t>(draw(seed, 8, 3 * r + 1) % static_cast<uint64_t>(pool_n - q.n + 1));
    q.off = lognormal_offsets(q.n, seed * 100003 + r);
    t += -std::log(unit(draw(seed, 9, r)));
    q.arrival_unit = t;
    q.verify = verify_every > 0 && r % verify_every == 0;
    total_keys += q.n;
    max_n = std::max(max_n, q.n);
  }
  // Every request's offsets in one pinned arena (one allocation, however
  // many requests).
  size_t arena_n = 0;
  for (const Req &q : reqs) arena_n += q.off.size();
  int32_t *arena = pinned<int32_t>(arena_n);
  size_t at = 0;
  for (Req &q : reqs) {
    q.h_off = arena + at;
    std::memcpy(q.h_off, q.off.data(), q.off.size() * 4);
    at += q.off.size();
  }
  uint32_t *sink_k = pinned<uint32_t>(max_n), *sink_v = pinned<uint32_t>(max_n);
  std::vector<uint32_t *> out_srv_k(requests, nullptr), out_srv_v(requests, nullptr);
  std::vector<uint32_t *> out_pl_k(requests, nullptr), out_pl_v(requests, nullptr);
  for (int64_t r = 0; r < requests; ++r) {
    if (!reqs[r].verify) continue;
    out_srv_k[r] = pinned<uint32_t>(reqs[r].n);
    out_srv_v[r] = pinned<uint32_t>(reqs[r].n);
    out_pl_k[r] = pinned<uint32_t>(reqs[r].n);
    out_pl_v[r] = pinned<uint32_t>(reqs[r].n);
  }

  // ---- plain loop resources ---------------------------------------------------
  cudaStream_t st;
  check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
  uint32_t *dk, *dv;
  int32_t *doff;
  size_t max_off = 0;
  for (const Req &q : reqs) max_off = std::max(max_off, q.off.size());
  check(cudaMalloc(&dk, max_n * 4), "malloc");
  check(cudaMalloc(&dv, max_n * 4), "malloc");
  check(cudaMalloc(&doff, max_off * 4), "malloc");

  auto plain_one = [&](int64_t r, uint32_t *ok, uint32_t *ov) {
    const Req &q = reqs[r];
    const int32_t nseg = static_cast<int32_t>(q.off.size() - 1);
    check(cudaMemcpyAsync(dk, pool_k + q.start, q.n * 4, cudaMemcpyHostToDevice, st), "h2d");
    check(cudaMemcpyAsync(dv, pool_v + q.start, q.n * 4, cudaMemcpyHostToDevice, st), "h2d");
    check(cudaMemcpyAsync(doff, q.h_off, q.off.size() * 4, cudaMemcpyHostToDevice, st), "h2d");
    const int rc = segsort_pairs_u32(dk, dv, q.n, doff, nseg, st);
    if (rc != SEGSORT_OK) {
      std::fprintf(stderr, "segsort_pairs_u32: %s\n", segsort_error_string(rc));
      std::exit(1);
    }
    check(cudaMemcpyAsync(ok, dk, q.n * 4, cudaMemcpyDeviceToHost, st), "d2h");
    check(cudaMemcpyAsync(ov, dv, q.n * 4, cudaMemcpyDeviceToHost, st), "d2h");
    check(cudaStreamSynchronize(st), "sync");
  };
  // warm-up: pool, kernels, attributes
  for (int64_t r = 0; r < std::min<int64_t>(requests, 8); ++r) plain_one(r, sink_k, sink_v);

  const size_t budget = static_cast<size_t>(budget_gb * 1073741824.0);
  for (double rate : rates) {
    // ---- served ---------------------------------------------------------------
    segsort_server srv = nullptr;
    int rc = segsort_server_create(budget, max_batch_keys, max_batch, depth, &srv);
    if (rc != SEGSORT_OK) {
      std::fprintf(stderr, "segsort_server_create: %s\n", segsort_error_string(rc));
      return 1;
    }
    std::vector<uint64_t> tickets(requests);
    std::vector<double> late(requests);
    const Clock::time_point t0 = Clock::now() + std::chrono::milliseconds(5);
    for (int64_t r = 0; r < requests; ++r) {
      const Req &q = reqs[r];
      const Clock::time_point at =
          t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(q.arrival_unit / rate));
      sleep_until(at);
      late[r] = std::chrono::duration<double, std::milli>(Clock::now() - at).count();
      rc = segsort_server_submit(srv, pool_k + q.start, pool_v + q.start, q.n, q.h_off,
                                 static_cast<int32_t>(q.off.size() - 1),
                                 q.verify ? out_srv_k[r] : sink_k, q.verify ? out_srv_v[r] : sink_v,
                                 &tickets[r]);
      if (rc != SEGSORT_OK) {
        std::fprintf(stderr, "segsort_server_submit: %s\n", segsort_error_string(rc));
        return 1;
      }
    }
    std::vector<double> lat_srv(requests);
    for (int64_t r = 0; r < requests; ++r) {
      double ms = 0;
      rc = segsort_server_wait(srv, tickets[r], &ms);
      if (rc != SEGSORT_OK) {
        std::fprintf(stderr, "request %lld: %s\n", static_cast<long long>(r), segsort_error_string(rc));
        return 1;
      }
      lat_srv[r] = ms + late[r];
    }
    const double srv_span = std::chrono::duration<double>(Clock::now() - t0).count();
    segsort_server_stats ss;
    segsort_server_get_stats(srv, &ss);
    segsort_server_destroy(srv);
    const int dstat = segsort_device_status(1);

    // ---- one request per plain call -------------------------------------------
    std::vector<double> lat_pl(requests);
    const Clock::time_point t1 = Clock::now() + std::chrono::milliseconds(5);
    for (int64_t r = 0; r < requests; ++r) {
      const Req &q = reqs[r];
      const Clock::time_point at =
          t1 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(q.arrival_unit / rate));
      sleep_until(at);
      plain_one(r, q.verify ? out_pl_k[r] : sink_k, q.verify ? out_pl_v[r] : sink_v);
      lat_pl[r] = std::chrono::duration<double, std::milli>(Clock::now() - at).count();
    }
    const double pl_span = std::chrono::duration<double>(Clock::now() - t1).count();

    int64_t verified = 0;
    bool identical = true;
    for (int64_t r = 0; r < requests; ++r) {
      if (!reqs[r].verify) continue;
      ++verified;
      const size_t b = reqs[r].n * 4;
      if (std::memcmp(out_srv_k[r], out_pl_k[r], b) != 0 || std::memcmp(out_srv_v[r], out_pl_v[r], b) != 0)
        identical = false;
      std::memset(out_srv_k[r], 0, b);  // the next rate must write them again
      std::memset(out_srv_v[r], 0, b);
    }
    auto jl = [&](const char *name, const std::vector<double> &lat, double span) {
      std::printf("\"%s\": {\"p50_ms\": %.4f, \"p99_ms\": %.4f, \"p999_ms\": %.4f, \"mean_ms\": %.4f, "
                  "\"gkeys_s\": %.4f, \"span_s\": %.4f}",
                  name, pct(lat, 50), pct(lat, 99), pct(lat, 99.9),
                  [&] { double s = 0; for (double x : lat) s += x; return s / lat.size(); }(),
                  total_keys / span / 1e9, span);
    };
    std::printf("{\"rate_req_s\": %.0f, \"requests\": %lld, \"keys\": %lld, ", rate,
                static_cast<long long>(requests), static_cast<long long>(total_keys));
    jl("served", lat_srv, srv_span);
    std::printf(", ");
    jl("plain", lat_pl, pl_span);
    std::printf(", \"depth\": %d, \"max_batch_keys\": %lld", depth,
                static_cast<long long>(max_batch_keys ? max_batch_keys : (int64_t{1} << 26)));
    std::printf(", \"batches\": %lld, \"max_batch\": %lld, \"mean_batch\": %.2f, \"peak_gb\": %.3f, "
                "\"budget_gb\": %.1f, \"budget_waits\": %lld, \"max_submit_late_ms\": %.4f, "
                "\"verified\": %lld, \"identical\": %s, \"device_status\": %d}\n",
                static_cast<long long>(ss.batches), static_cast<long long>(ss.max_batch),
                ss.batches ? static_cast<double>(ss.requests) / ss.batches : 0.0,
                ss.peak_bytes / 1073741824.0, budget_gb, static_cast<long long>(ss.budget_waits),
                *std::max_element(late.begin(), late.end()), static_cast<long long>(verified),
                identical ? "true" : "false", dstat);
    std::fflush(stdout);
    if (!identical || dstat != SEGSORT_OK || ss.status != SEGSORT_OK) return 2;
  }
  return 0;
}
