// Served form: a continuous-batching request server (segsort_server_*).
//
// Host side only; the device work is the batched sort of segsort_batch.cu.
// submit() queues a request (host buffers) and returns at once.  One worker
// thread per server forms batches: it admits queued requests in arrival order
// while their device footprint fits the HBM budget beside the requests in
// flight, and launches the batch as a three-stage pipeline on three streams:
//     copies in (s_in) -> one batched sort (s_sort) -> copies out (s_out)
// tied by events, so the copies of one batch overlap the sort of another.
// At most `depth` batches are between admission and the end of their sort;
// requests that arrive meanwhile wait in the queue and join the next batch,
// which is what coalesces them under load; a batch closes at max_batch_keys
// keys so that one batch's sort overlaps the next one's copies.  Stream callbacks (no CUDA calls
// inside) report the end of each sort and of each batch's copies out; the
// latter completes the batch's requests and releases their budget.
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "segsort.h"
#include "segsort_host.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  const uint32_t *h_keys, *h_vals;
  const int32_t *h_offsets;
  int64_t n;
  int32_t nseg;
  uint32_t *h_keys_out, *h_vals_out;
  size_t bytes;  // device footprint charged against the budget
  Clock::time_point t_submit, t_done;
  bool done = false;
  bool collected = false;  // segsort_server_wait has returned for it
  int status = SEGSORT_OK;
};

// Default batch size limit: 2^26 keys, a few milliseconds of sorting.
constexpr int64_t kDefaultBatchKeys = int64_t{1} << 26;

size_t a256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Device bytes of one request's buffers in a batch.
size_t buffer_bytes(int64_t n, int32_t nseg) {
  return 2 * a256(static_cast<size_t>(n) * 4) + a256((static_cast<size_t>(nseg) + 1) * 4);
}

// Footprint charged at admission: the request's buffers plus an upper bound
// of its share of the batch workspace (the workspace of a problem one tile
// larger, which covers the per-instance half-tile map, table entry and
// rounding of the batch layout).
size_t footprint(int64_t n, int32_t nseg) {
  return buffer_bytes(n, nseg) + segsort_workspace_bytes(n + 4097, 1, 4, 4) + 8192;
}

}  // namespace

struct segsort_server_s {
  int dev = 0;
  size_t budget = 0;
  int64_t max_batch_keys = 0;
  int max_batch = 0;
  int depth = 2;
  cudaStream_t s_in = nullptr, s_sort = nullptr, s_out = nullptr;
  cudaEvent_t ev_in = nullptr, ev_sorted = nullptr;

  std::mutex mu;
  std::condition_variable cv;
  // Requests by ticket, from ticket `base` on: a request leaves the front
  // once it is done and its wait has returned, so a long-running server
  // holds only the requests still in flight or not yet waited for.  The
  // deque keeps references to the others stable.
  std::deque<Request> reqs;
  uint64_t base = 0;
  std::deque<uint64_t> queue;    // submitted, not admitted
  uint64_t completed = 0;
  size_t in_flight = 0;          // admitted bytes not yet released
  uint64_t released = 0;         // release generation
  int pipeline = 0;              // batches admitted whose sort has not ended
  bool stop = false;
  segsort_server_stats stats = {};
  std::thread worker;
};

namespace {

struct BatchRecord {
  segsort_server_s *S;
  std::vector<uint64_t> tickets;
  size_t bytes;
};

void CUDART_CB on_sorted(void *p) {
  segsort_server_s *S = static_cast<segsort_server_s *>(p);
  std::lock_guard<std::mutex> lk(S->mu);
  --S->pipeline;
  S->cv.notify_all();
}

void CUDART_CB on_done(void *p) {
  std::unique_ptr<BatchRecord> B(static_cast<BatchRecord *>(p));
  segsort_server_s *S = B->S;
  const Clock::time_point now = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  for (uint64_t t : B->tickets) {
    Request &r = S->reqs[t - S->base];
    r.t_done = now;
    r.done = true;
    S->stats.keys += r.n;
  }
  S->stats.requests += static_cast<int64_t>(B->tickets.size());
  S->completed += B->tickets.size();
  S->in_flight -= B->bytes;
  ++S->released;
  S->cv.notify_all();
}

// Enqueues one batch: copies in, batched sort, copies out, callbacks.  The
// request fields it reads were fixed at submission.  *sorted_cb is set once
// the end-of-sort callback is enqueued; on failure the streams are drained
// and the batch buffer freed before returning.
int launch_batch(segsort_server_s *S, const std::vector<Request *> &rs, BatchRecord *rec,
                 bool *sorted_cb) {
  *sorted_cb = false;
  size_t total = 0;
  for (const Request *r : rs) total += buffer_bytes(r->n, r->nseg);
  const int dev = S->dev;
  segsort::DeviceState *DS = segsort::device_state(dev);
  cudaMemPool_t pool = DS ? segsort::device_pool(*DS, dev) : nullptr;
  unsigned char *d = nullptr;
  if (pool == nullptr ||
      cudaMallocFromPoolAsync(reinterpret_cast<void **>(&d), total, pool, S->s_in) != cudaSuccess) {
    cudaGetLastError();
    return SEGSORT_ERR_NO_MEMORY;
  }
  auto fail = [&](int rc) {
    cudaGetLastError();
    cudaStreamSynchronize(S->s_in);
    cudaStreamSynchronize(S->s_sort);
    cudaStreamSynchronize(S->s_out);
    cudaFreeAsync(d, S->s_out);
    cudaStreamSynchronize(S->s_out);
    cudaGetLastError();
    return rc;
  };
  std::vector<segsort_batch_item> items(rs.size());
  std::vector<unsigned char *> dk(rs.size());
  size_t off = 0;
  for (size_t i = 0; i < rs.size(); ++i) {
    const Request &r = *rs[i];
    const size_t kb = static_cast<size_t>(r.n) * 4;
    unsigned char *k = d + off, *v = k + a256(kb), *o = v + a256(kb);
    off += buffer_bytes(r.n, r.nseg);
    dk[i] = k;
    if (kb > 0 && (cudaMemcpyAsync(k, r.h_keys, kb, cudaMemcpyHostToDevice, S->s_in) != cudaSuccess ||
                   cudaMemcpyAsync(v, r.h_vals, kb, cudaMemcpyHostToDevice, S->s_in) != cudaSuccess))
      return fail(SEGSORT_ERR_CUDA);
    if (r.nseg > 0 && cudaMemcpyAsync(o, r.h_offsets, (static_cast<size_t>(r.nseg) + 1) * 4,
                                      cudaMemcpyHostToDevice, S->s_in) != cudaSuccess)
      return fail(SEGSORT_ERR_CUDA);
    items[i] = segsort_batch_item{SEGSORT_KEY_U32, 0, k, reinterpret_cast<uint32_t *>(v), r.n,
                                  reinterpret_cast<const int32_t *>(o), r.nseg, 0};
  }
  if (cudaEventRecord(S->ev_in, S->s_in) != cudaSuccess ||
      cudaStreamWaitEvent(S->s_sort, S->ev_in, 0) != cudaSuccess)
    return fail(SEGSORT_ERR_CUDA);
  // A batch of one request is a plain call (the same kernels without the
  // batch's table upload and per-group launches; at low load most batches
  // hold one request).
  const int rc =
      items.size() == 1
          ? segsort_pairs_u32(static_cast<uint32_t *>(items[0].d_keys), items[0].d_vals,
                              items[0].n, items[0].d_offsets, items[0].nseg, S->s_sort)
          : segsort_pairs_batch(items.data(), static_cast<int32_t>(items.size()), S->s_sort);
  if (rc != SEGSORT_OK) return fail(rc);
  // The copies out wait for the sort, not for the host callback after it
  // (a host function holds its stream until it returns).
  if (cudaEventRecord(S->ev_sorted, S->s_sort) != cudaSuccess ||
      cudaStreamWaitEvent(S->s_out, S->ev_sorted, 0) != cudaSuccess)
    return fail(SEGSORT_ERR_CUDA);
  if (cudaLaunchHostFunc(S->s_sort, on_sorted, S) != cudaSuccess) return fail(SEGSORT_ERR_CUDA);
  *sorted_cb = true;
  for (size_t i = 0; i < rs.size(); ++i) {
    const Request &r = *rs[i];
    const size_t kb = static_cast<size_t>(r.n) * 4;
    if (kb > 0 &&
        (cudaMemcpyAsync(r.h_keys_out, dk[i], kb, cudaMemcpyDeviceToHost, S->s_out) != cudaSuccess ||
         cudaMemcpyAsync(r.h_vals_out, dk[i] + a256(kb), kb, cudaMemcpyDeviceToHost, S->s_out) !=
             cudaSuccess))
      return fail(SEGSORT_ERR_CUDA);
  }
  if (cudaFreeAsync(d, S->s_out) != cudaSuccess) return fail(SEGSORT_ERR_CUDA);
  if (cudaLaunchHostFunc(S->s_out, on_done, rec) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamSynchronize(S->s_out);
    return SEGSORT_ERR_CUDA;
  }
  return SEGSORT_OK;
}

void worker_loop(segsort_server_s *S) {
  cudaSetDevice(S->dev);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true) {
    S->cv.wait(lk, [&] { return S->stop || (!S->queue.empty() && S->pipeline < S->depth); });
    if (S->queue.empty()) {
      if (S->stop) break;
      continue;
    }
    // Admission: arrival order, while the budget allows.
    std::vector<Request *> take;
    std::unique_ptr<BatchRecord> rec(new BatchRecord{S, {}, 0});
    bool deferred = false;  // the oldest queued request did not fit the budget
    int64_t keys = 0;
    while (!S->queue.empty() &&
           (S->max_batch <= 0 || static_cast<int>(take.size()) < S->max_batch)) {
      Request &r = S->reqs[S->queue.front() - S->base];
      // A batch closes once it holds max_batch_keys keys, so that the copies
      // of the next batch overlap its sort instead of waiting behind it.
      if (!take.empty() && keys + r.n > S->max_batch_keys) break;
      if (S->in_flight + rec->bytes + r.bytes > S->budget) {
        deferred = true;
        break;
      }
      rec->bytes += r.bytes;
      keys += r.n;
      rec->tickets.push_back(S->queue.front());
      take.push_back(&r);
      S->queue.pop_front();
    }
    if (deferred) ++S->stats.budget_waits;
    if (take.empty()) {  // the oldest request waits for memory to be released
      const uint64_t gen = S->released;
      S->cv.wait(lk, [&] { return S->released != gen; });
      continue;
    }
    S->in_flight += rec->bytes;
    if (static_cast<int64_t>(S->in_flight) > S->stats.peak_bytes)
      S->stats.peak_bytes = static_cast<int64_t>(S->in_flight);
    ++S->pipeline;
    ++S->stats.batches;
    if (static_cast<int64_t>(take.size()) > S->stats.max_batch)
      S->stats.max_batch = static_cast<int64_t>(take.size());
    lk.unlock();
    BatchRecord *raw = rec.release();
    bool sorted_cb = false;
    const int rc = launch_batch(S, take, raw, &sorted_cb);
    lk.lock();
    if (rc != SEGSORT_OK) {
      // Nothing of this batch completes on the device: fail its requests
      // here.  Work already enqueued for it finishes on its streams.
      cudaGetLastError();
      if (S->stats.status == SEGSORT_OK) S->stats.status = rc;
      const Clock::time_point now = Clock::now();
      for (uint64_t t : raw->tickets) {
        Request &r = S->reqs[t - S->base];
        r.status = rc;
        r.done = true;
        r.t_done = now;
      }
      S->completed += raw->tickets.size();
      S->in_flight -= raw->bytes;
      ++S->released;
      if (!sorted_cb) --S->pipeline;  // otherwise the end-of-sort callback does it
      delete raw;
      S->cv.notify_all();
    }
  }
}

}  // namespace

extern "C" {

int segsort_server_create(size_t budget_bytes, int64_t max_batch_keys, int32_t max_batch,
                          int32_t depth, segsort_server *server) {
  if (server == nullptr) return SEGSORT_ERR_INVALID_ARG;
  *server = nullptr;
  if (budget_bytes == 0 || max_batch_keys < 0 || max_batch < 0 || depth < 0 || depth > 8)
    return SEGSORT_ERR_INVALID_ARG;
  std::unique_ptr<segsort_server_s> S(new (std::nothrow) segsort_server_s);
  if (!S) return SEGSORT_ERR_NO_MEMORY;
  S->budget = budget_bytes;
  S->max_batch_keys = max_batch_keys == 0 ? kDefaultBatchKeys : max_batch_keys;
  S->max_batch = max_batch;
  S->depth = depth == 0 ? 2 : depth;
  if (cudaGetDevice(&S->dev) != cudaSuccess) return SEGSORT_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&S->s_in, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&S->s_sort, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&S->s_out, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&S->ev_in, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&S->ev_sorted, cudaEventDisableTiming) != cudaSuccess) {
    if (S->s_in) cudaStreamDestroy(S->s_in);
    if (S->s_sort) cudaStreamDestroy(S->s_sort);
    if (S->s_out) cudaStreamDestroy(S->s_out);
    if (S->ev_in) cudaEventDestroy(S->ev_in);
    if (S->ev_sorted) cudaEventDestroy(S->ev_sorted);
    return SEGSORT_ERR_CUDA;
  }
  segsort_server_s *raw = S.release();
  raw->worker = std::thread(worker_loop, raw);
  *server = raw;
  return SEGSORT_OK;
}

int segsort_server_submit(segsort_server S, const uint32_t *h_keys, const uint32_t *h_vals,
                          int64_t n, const int32_t *h_offsets, int32_t nseg,
                          uint32_t *h_keys_out, uint32_t *h_vals_out, uint64_t *ticket) {
  if (S == nullptr || ticket == nullptr || n < 0 || nseg < 0) return SEGSORT_ERR_INVALID_ARG;
  if (n > 0 && (h_keys == nullptr || h_vals == nullptr || h_keys_out == nullptr ||
                h_vals_out == nullptr))
    return SEGSORT_ERR_INVALID_ARG;
  if (nseg > 0 && h_offsets == nullptr) return SEGSORT_ERR_INVALID_ARG;
  if (n >= (int64_t{1} << 30)) return SEGSORT_ERR_TOO_LARGE;
  Request r;
  r.h_keys = h_keys;
  r.h_vals = h_vals;
  r.h_offsets = h_offsets;
  r.n = n;
  r.nseg = nseg;
  r.h_keys_out = h_keys_out;
  r.h_vals_out = h_vals_out;
  r.bytes = footprint(n, nseg);
  if (r.bytes > S->budget) return SEGSORT_ERR_TOO_LARGE;
  r.t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) return SEGSORT_ERR_INVALID_ARG;
  *ticket = S->base + S->reqs.size();
  S->reqs.push_back(r);
  S->queue.push_back(*ticket);
  S->cv.notify_all();
  return SEGSORT_OK;
}

int segsort_server_wait(segsort_server S, uint64_t ticket, double *latency_ms) {
  if (S == nullptr) return SEGSORT_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  if (ticket < S->base || ticket >= S->base + S->reqs.size() ||
      S->reqs[ticket - S->base].collected)
    return SEGSORT_ERR_INVALID_ARG;  // unknown, or already waited for
  S->cv.wait(lk, [&] { return S->reqs[ticket - S->base].done; });
  Request &r = S->reqs[ticket - S->base];
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
  const int status = r.status;
  r.collected = true;
  while (!S->reqs.empty() && S->reqs.front().done && S->reqs.front().collected) {
    S->reqs.pop_front();
    ++S->base;
  }
  return status;
}

int segsort_server_drain(segsort_server S) {
  if (S == nullptr) return SEGSORT_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv.wait(lk, [&] { return S->completed == S->base + S->reqs.size(); });
  return S->stats.status;
}

int segsort_server_get_stats(segsort_server S, segsort_server_stats *stats) {
  if (S == nullptr || stats == nullptr) return SEGSORT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  *stats = S->stats;
  return SEGSORT_OK;
}

void segsort_server_destroy(segsort_server S) {
  if (S == nullptr) return;
  segsort_server_drain(S);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  cudaStreamSynchronize(S->s_out);
  cudaStreamDestroy(S->s_in);
  cudaStreamDestroy(S->s_sort);
  cudaStreamDestroy(S->s_out);
  cudaEventDestroy(S->ev_in);
  cudaEventDestroy(S->ev_sorted);
  delete S;
}

}  // extern "C"
