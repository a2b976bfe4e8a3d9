/*
 * segsort.h -- C ABI of the GB300 (sm_103a) segmented sort.
 *
 * Every entry point sorts, independently and stably, each segment
 * [offsets[i], offsets[i+1]) of a device array of keys (and, for the
 * `pairs` forms, the uint32 values that travel with them).  The sort is in
 * place: on return the input buffers hold the result, as with
 * bb_segsort (src/bb_segsort/bb_segsort.h:175-178 copies the result back
 * into keys_d/vals_d).  Elements outside every segment are not touched.
 *
 * Order.  Keys are compared through an order-preserving map to unsigned
 * bits: unsigned keys as-is, signed keys with the sign bit flipped, float
 * keys with all bits flipped when the sign bit is set and only the sign
 * bit flipped otherwise.  So -0.0f sorts before +0.0f, and NaNs sort by
 * their bit pattern (negative NaNs first, positive NaNs last).  Equal keys
 * keep their input order (stable), which is what the reference's oracle
 * std::stable_sort gives (src/mseq.cu:44-49, src/bb_segsort/main.cu:152-173).
 *
 * Offsets.  `d_offsets` is a device array of nseg+1 int32 CSR offsets:
 * segment i is [d_offsets[i], d_offsets[i+1]).  They must be
 * non-decreasing and lie in [0, n]; the kernels clamp every offset into
 * [0, n] and treat a segment whose end is below its begin as empty, so a
 * malformed array cannot make them touch memory outside [0, n).  The
 * `_heads` forms take nseg segment heads instead, the last segment ending
 * at n (the bb_segsort and moderngpu convention,
 * src/bb_segsort/bb_segsort.h:35-36, lib/moderngpu/kernel_segsort.hxx:405-415).
 *
 * Asynchrony.  Every call is asynchronous on `stream` and makes no host
 * synchronisation.  Temporary storage comes either from the caller (the
 * `_ws` forms, sized by segsort_workspace_bytes) or from a library-owned
 * stream-ordered memory pool (cudaMallocFromPoolAsync / cudaFreeAsync on
 * `stream`).  Calls on different streams may run concurrently.
 *
 * Errors.  0 on success, a negative SEGSORT_ERR_* code otherwise.  No
 * call throws or exits.  A device-side failure (a bounded wait in a
 * kernel that gave up) cannot be returned by an asynchronous call; it is
 * recorded on the device and read back by segsort_device_status().
 *
 * Limits.  n < 2^30 elements per call; offsets are int32.
 */
#ifndef SEGSORT_H_
#define SEGSORT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; a null pointer is the legacy default stream. */
struct CUstream_st;
typedef struct CUstream_st *segsort_stream_t;

#define SEGSORT_OK 0
#define SEGSORT_ERR_INVALID_ARG (-1) /* null pointer, n < 0, nseg < 0, ...   */
#define SEGSORT_ERR_CUDA (-2)        /* a CUDA runtime call or launch failed */
#define SEGSORT_ERR_TIMEOUT (-3)     /* a bounded device wait gave up        */
#define SEGSORT_ERR_NO_MEMORY (-4)   /* the workspace could not be allocated */
#define SEGSORT_ERR_TOO_LARGE (-5)   /* n or a segment exceeds the limits    */
#define SEGSORT_ERR_WORKSPACE (-6)   /* caller workspace too small/unaligned */

/* ------------------------------------------------------------------------
 * Keys only.
 * Replaces the keys-only CPU path `segmented_sorting(uint* vec, uint* seg,
 * int number_of_segments)` (src/mseq.cu:44-49), which runs std::stable_sort
 * on every [seg[i], seg[i+1]).
 * ---------------------------------------------------------------------- */
int segsort_keys_u32(uint32_t *d_keys, int64_t n, const int32_t *d_offsets,
                     int32_t nseg, segsort_stream_t stream);
int segsort_keys_i32(int32_t *d_keys, int64_t n, const int32_t *d_offsets,
                     int32_t nseg, segsort_stream_t stream);
int segsort_keys_f32(float *d_keys, int64_t n, const int32_t *d_offsets,
                     int32_t nseg, segsort_stream_t stream);
int segsort_keys_u64(uint64_t *d_keys, int64_t n, const int32_t *d_offsets,
                     int32_t nseg, segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Key/value pairs (uint32 values, moved with their keys).
 * Replaces cub::DeviceSegmentedRadixSort::SortPairs(d_temp, temp_bytes,
 * keys_in, keys_out, vals_in, vals_out, n, nseg, d_seg, d_seg + 1) as called
 * in src/radixseg.cu:121-124 (signature at
 * lib/cub/device/device_segmented_radix_sort.cuh:140-155): the same CSR
 * offsets (begin = d_offsets, end = d_offsets + 1), in place instead of
 * double-buffered, stable, and without the two-phase temp-storage query.
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                      const int32_t *d_offsets, int32_t nseg,
                      segsort_stream_t stream);
int segsort_pairs_i32(int32_t *d_keys, uint32_t *d_vals, int64_t n,
                      const int32_t *d_offsets, int32_t nseg,
                      segsort_stream_t stream);
int segsort_pairs_f32(float *d_keys, uint32_t *d_vals, int64_t n,
                      const int32_t *d_offsets, int32_t nseg,
                      segsort_stream_t stream);
int segsort_pairs_u64(uint64_t *d_keys, uint32_t *d_vals, int64_t n,
                      const int32_t *d_offsets, int32_t nseg,
                      segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Heads-only offsets: d_heads[nseg], segment i = [d_heads[i], d_heads[i+1])
 * and the last segment ends at n.
 * Replaces `int bb_segsort(K *keys_d, T *vals_d, int n, int *d_segs,
 * int length)` (src/bb_segsort/bb_segsort.h:35-36) and
 * `mgpu::segmented_sort(keys, vals, count, segments, num_segments, comp,
 * context)` (lib/moderngpu/kernel_segsort.hxx:405-415; driven from
 * src/mergeseg.cu:79-90,118-119 with heads only).  Unlike bb_segsort the
 * result is stable and the call returns 0 on success (bb_segsort returns 1).
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32_heads(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                            const int32_t *d_heads, int32_t nseg,
                            segsort_stream_t stream);
int segsort_keys_u32_heads(uint32_t *d_keys, int64_t n, const int32_t *d_heads,
                           int32_t nseg, segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Caller-provided workspace.  segsort_workspace_bytes() is an upper bound
 * for any offsets array with these n / nseg / key and value widths
 * (key_bytes 4 or 8, val_bytes 0 or 4).  The workspace must be 256-byte
 * aligned device memory of at least that size; it is used asynchronously
 * on `stream` and may be reused once the call's work on `stream` is done.
 * These replace the two-phase `d_temp_storage == NULL` size query of
 * lib/cub/device/device_segmented_radix_sort.cuh:140-155.
 * ---------------------------------------------------------------------- */
size_t segsort_workspace_bytes(int64_t n, int32_t nseg, int key_bytes,
                               int val_bytes);
int segsort_pairs_u32_ws(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                         const int32_t *d_offsets, int32_t nseg,
                         void *d_workspace, size_t workspace_bytes,
                         segsort_stream_t stream);
int segsort_keys_u32_ws(uint32_t *d_keys, int64_t n, const int32_t *d_offsets,
                        int32_t nseg, void *d_workspace,
                        size_t workspace_bytes, segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Allocation-free form of segsort_pairs_u32.  No counterpart in the
 * reference, whose drivers allocate device memory around every call
 * (src/radixseg.cu:98-120, src/bb_segsort/bb_segsort.h:43-56).
 *
 * For callers that cannot allocate device memory where they sort: code whose
 * device memory belongs to another allocator that already holds the device
 * (a framework's caching allocator), real-time loops that must not block in,
 * or fail on, an allocation once running, and code that must not fail with
 * out-of-memory in mid-run.  The temporary storage is a fixed scratch array
 * that is part of the library's device code, sized for n up to
 * SEGSORT_NOALLOC_MAX_N uint32 key/value pairs (about 10 MiB); every GPU
 * that loads the library holds it until the process exits.  The call makes
 * no cudaMalloc, cudaFree or other allocating call.
 *
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  All calls share the one array, and every call
 * clears what it needs at its start: calls that overlap on the GPU (other
 * streams, or other host threads without ordering) race and corrupt each
 * other's results, so order them on one stream.  n > SEGSORT_NOALLOC_MAX_N
 * returns SEGSORT_ERR_TOO_LARGE before touching the GPU.
 * ---------------------------------------------------------------------- */
#define SEGSORT_NOALLOC_MAX_N 1048576
int segsort_pairs_u32_noalloc(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                              const int32_t *d_offsets, int32_t nseg,
                              segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Descending order, stable: equal keys keep their input order.  Replaces
 * cub::DeviceSegmentedRadixSort::SortPairsDescending
 * (lib/cub/device/device_segmented_radix_sort.cuh:338).  The keys are mapped
 * in place to the complement of their order bits, sorted ascending and
 * mapped back (two extra element-wise passes over the keys).
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32_desc(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg,
                           segsort_stream_t stream);
int segsort_pairs_i32_desc(int32_t *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg,
                           segsort_stream_t stream);
int segsort_pairs_f32_desc(float *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg,
                           segsort_stream_t stream);
int segsort_pairs_u64_desc(uint64_t *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg,
                           segsort_stream_t stream);
int segsort_keys_u32_desc(uint32_t *d_keys, int64_t n, const int32_t *d_offsets,
                          int32_t nseg, segsort_stream_t stream);
int segsort_keys_f32_desc(float *d_keys, int64_t n, const int32_t *d_offsets,
                          int32_t nseg, segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Segmented top-k (no reference counterpart).  Sorts every segment in place
 * (ascending, or stable descending when `descending` is non-zero), then
 * writes its first min(k, len) keys -- and values, when d_out_vals is not
 * null -- to row s of the [nseg][k] outputs, and min(k, len) to
 * d_out_counts[s] when d_out_counts is not null.  Output slots past a row's
 * count are not written.
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32_topk(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg, int64_t k,
                           int descending, uint32_t *d_out_keys,
                           uint32_t *d_out_vals, int32_t *d_out_counts,
                           segsort_stream_t stream);
int segsort_pairs_f32_topk(float *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg, int64_t k,
                           int descending, float *d_out_keys, uint32_t *d_out_vals,
                           int32_t *d_out_counts, segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * 64-bit values (the reference's bb_segsort instances carry double values,
 * src/bb_segsort/main.cu:68-72).  The keys are sorted with their positions
 * as 32-bit values, then the 64-bit values are gathered through those
 * positions (workspace: 12 bytes per element from the library's pool).
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32_v64(uint32_t *d_keys, uint64_t *d_vals, int64_t n,
                          const int32_t *d_offsets, int32_t nseg,
                          segsort_stream_t stream);
int segsort_pairs_i32_v64(int32_t *d_keys, uint64_t *d_vals, int64_t n,
                          const int32_t *d_offsets, int32_t nseg,
                          segsort_stream_t stream);
int segsort_pairs_f32_v64(float *d_keys, uint64_t *d_vals, int64_t n,
                          const int32_t *d_offsets, int32_t nseg,
                          segsort_stream_t stream);
int segsort_pairs_u64_v64(uint64_t *d_keys, uint64_t *d_vals, int64_t n,
                          const int32_t *d_offsets, int32_t nseg,
                          segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Segmented reduce-by-key (no reference counterpart; the step after the sort
 * in typical pipelines).  Sorts every segment ascending in place, then, for
 * every run of equal keys inside a segment, in segment order: its key in
 * d_out_keys, the sum of its values (64-bit, no overflow) in d_out_sums and
 * its length in d_out_counts; d_out_offsets[s] (nseg + 1 entries) is the
 * index of segment s's first run, d_out_offsets[nseg] the number of runs.
 * The three run arrays need room for n runs.
 * ---------------------------------------------------------------------- */
int segsort_pairs_u32_reduce_by_key(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                                    const int32_t *d_offsets, int32_t nseg,
                                    uint32_t *d_out_keys, uint64_t *d_out_sums,
                                    uint32_t *d_out_counts, int32_t *d_out_offsets,
                                    segsort_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched form: many independent instances, each with its own keys, uint32
 * values and offsets, sorted by one launch of each kernel per key type
 * instead of one sequence of launches per instance.  No counterpart in the
 * reference, which sorts one instance per program; it replaces the
 * reference's launch loops over streams (src/newthrust.cu:137-157) and its
 * per-bin streams (src/bb_segsort/bb_segsort.h:60-61) as the way to keep the
 * GPU busy with many small problems.
 *
 * Every item is the argument list of one segsort_pairs_<type> call
 * (heads = 1: the segsort_pairs_u32_heads convention).  Items must not
 * overlap in memory.  The result of every item is bit for bit the result of
 * its own plain call.  Limits: each item n < 2^30, and the items of one key
 * type together fewer than 2^31 elements (SEGSORT_ERR_TOO_LARGE).
 * ---------------------------------------------------------------------- */
#define SEGSORT_KEY_U32 0
#define SEGSORT_KEY_I32 1
#define SEGSORT_KEY_F32 2
#define SEGSORT_KEY_U64 3

typedef struct segsort_batch_item {
  int32_t key_type; /* SEGSORT_KEY_*                               */
  int32_t heads;    /* 1: d_offsets holds nseg heads, end = n       */
  void *d_keys;     /* n keys of key_type                           */
  uint32_t *d_vals; /* n values                                     */
  int64_t n;
  const int32_t *d_offsets;
  int32_t nseg;
  int32_t reserved; /* 0                                            */
} segsort_batch_item;

/* One-shot: enqueues the batch on `stream` (workspace from the library's
 * pool, no host synchronisation). */
int segsort_pairs_batch(const segsort_batch_item *items, int32_t count,
                        segsort_stream_t stream);

/* Plan: validates the items once, allocates the workspace, and captures the
 * whole batch into one CUDA graph.  Each launch replays the graph on
 * `stream`: it sorts whatever the items' buffers hold at that time, at the
 * same addresses.  Launches of one plan must not overlap (they share its
 * workspace): order them on one stream. */
typedef struct segsort_batch_plan_s *segsort_batch_plan;
int segsort_batch_plan_create(const segsort_batch_item *items, int32_t count,
                              segsort_batch_plan *plan);
int segsort_batch_plan_launch(segsort_batch_plan plan, segsort_stream_t stream);
/* Autotuner: picks the launch shape of the plan's merge passes (1, 2 or 3
 * resident CTAs per SM) by replaying the plan four times per shape on
 * `stream` (the items' buffers are sorted by it, as by a launch) and keeping
 * the fastest.  With cache_path given, the choice is looked up first in, and
 * after a measurement appended to, that text file, keyed by the class of the
 * batch (key types present; log2 of the total keys, the largest item and the
 * key-weighted mean segment length).  *ctas_per_sm (optional) receives the
 * choice.  Untuned plans use 3. */
int segsort_batch_plan_tune(segsort_batch_plan plan, segsort_stream_t stream,
                            const char *cache_path, int32_t *ctas_per_sm);
size_t segsort_batch_plan_workspace_bytes(segsort_batch_plan plan);
void segsort_batch_plan_destroy(segsort_batch_plan plan);

/* Device bytes one segsort_pairs_batch call on these items takes from the
 * library's pool (tables and workspace); 0 when the items are invalid or
 * hold nothing to sort. */
size_t segsort_batch_workspace_bytes(const segsort_batch_item *items, int32_t count);

/* ------------------------------------------------------------------------
 * Served form: a continuous-batching request server on the current device.
 * No counterpart in the reference (its programs sort one instance read from
 * stdin, src/mseq.cu:57-67).
 *
 * Requests are uint32 key/value sorts whose inputs and outputs live in host
 * memory (pin it, e.g. cudaHostAlloc, for copies that overlap the sorts).
 * submit() only queues the request and returns a ticket.  A worker thread
 * admits queued requests in arrival order while their device footprint
 * (keys, values, offsets and sort workspace) fits the HBM budget next to the
 * requests already in flight, coalesces every admitted request into one
 * batched sort (segsort_pairs_batch), and keeps up to `depth` batches in the
 * pipeline: the copies in of the next batch and the copies out of the last
 * one overlap the current sort.  Requests that arrive while a batch runs join
 * the next one.  A request whose footprint alone exceeds the budget is refused
 * (SEGSORT_ERR_TOO_LARGE).  The result of every request is bit for bit the
 * result of its own plain call.
 * ---------------------------------------------------------------------- */
typedef struct segsort_server_s *segsort_server;
typedef struct segsort_server_stats {
  int64_t requests;         /* completed requests                         */
  int64_t batches;          /* batched sorts launched                     */
  int64_t keys;             /* keys of the completed requests             */
  int64_t max_batch;        /* most requests coalesced into one batch     */
  int64_t peak_bytes;       /* highest admitted device footprint          */
  int64_t budget_waits;     /* admissions that left the oldest queued
                               request waiting for memory to be released  */
  int32_t status;           /* first error of the worker, SEGSORT_OK      */
  int32_t reserved;
} segsort_server_stats;

/* budget_bytes: device bytes the in-flight requests may hold;
 * max_batch_keys: a batch closes once it holds this many keys (0: 2^26;
 * a single larger request still forms a batch of its own); max_batch: most
 * requests per batch (0: no limit); depth: batches in the pipeline (1..8,
 * 0: 2). */
int segsort_server_create(size_t budget_bytes, int64_t max_batch_keys, int32_t max_batch,
                          int32_t depth, segsort_server *server);
int segsort_server_submit(segsort_server server, const uint32_t *h_keys,
                          const uint32_t *h_vals, int64_t n, const int32_t *h_offsets,
                          int32_t nseg, uint32_t *h_keys_out, uint32_t *h_vals_out,
                          uint64_t *ticket);
/* Blocks until the request is done; *latency_ms (optional) = completion
 * minus submission, host steady clock.  Wait once per ticket: the server
 * keeps a request's record until its wait returns (a second wait on the
 * ticket returns SEGSORT_ERR_INVALID_ARG), so a long-running server holds
 * only the requests still in flight or not yet waited for. */
int segsort_server_wait(segsort_server server, uint64_t ticket, double *latency_ms);
/* Blocks until every submitted request is done. */
int segsort_server_drain(segsort_server server);
int segsort_server_get_stats(segsort_server server, segsort_server_stats *stats);
/* Drains, stops the worker and frees the server. */
void segsort_server_destroy(segsort_server server);

/* ------------------------------------------------------------------------
 * Diagnostics.
 * segsort_device_status() synchronises the current device, returns
 * SEGSORT_OK or the first device-side error recorded since the last clear
 * (SEGSORT_ERR_TIMEOUT when a bounded wait gave up), and clears it when
 * `clear` is non-zero.  There is no counterpart in the reference, whose
 * drivers only print cudaGetLastError (src/radixseg.cu:127-132).
 * ---------------------------------------------------------------------- */
int segsort_device_status(int clear);
const char *segsort_error_string(int code);
int segsort_version(void);

/* The library's own stream-ordered pool on the current device: *created = 1
 * once the first call that allocates from it has created it (0 before), and
 * *used = the bytes its allocations hold right now (cudaMemPoolAttrUsedMemCurrent;
 * 0 when idle, since every call frees what it takes on its stream).  A
 * diagnostic, e.g. to show that the allocation-free entry point never
 * creates the pool.  No counterpart in the reference. */
int segsort_pool_bytes(int *created, uint64_t *used);

/* Run-time tuning parameters, process-wide (no counterpart in the reference,
 * whose variants fix their thresholds at compile time, e.g. the bin bounds
 * of src/bb_segsort/bb_bin.h:54-100).
 *   SEGSORT_PARAM_RADIX_MIN_32 / _64: segments longer than this many keys
 *     (32-bit / 64-bit keys) are sorted by LSD radix passes; shorter long
 *     segments by merge passes over tile-sorted runs.  At least 4096.
 *   SEGSORT_PARAM_STREAM_MAX_AVG: problems whose average segment (n / nseg)
 *     is at most this long take the streamed short-segment tile kernel.
 *   SEGSORT_PARAM_BUCKET_MIN_AVG: other problems whose average segment is at
 *     least this long take the bucket route of the tile sort (a bucket sort
 *     by key value per chunk, the comparison sort for the chunks it
 *     refuses); 0 turns the route off.
 *   SEGSORT_PARAM_MSD: 1 (default) or 0.  With 1, a call whose average
 *     segment is longer than the radix threshold, in the library's own
 *     workspace, sorts its radix segments whose keys vary in at least three
 *     8-bit digits by one radix pass on the top varying digit and then the
 *     tile sort of the 256 sub-buckets, instead of one pass per digit.
 *   SEGSORT_PARAM_TINY_MAX_AVG: problems whose average segment is at most this
 *     long (and at most the streamed-tile threshold) take the tiny route: a
 *     network sort of chunks of segments of at most 8 keys, the comparison sort
 *     for the other chunks; 0 turns it off.
 * A change applies to calls made after it; batch plans keep the values they
 * were created with.  SEGSORT_ERR_INVALID_ARG for an unknown parameter or a
 * value out of range. */
#define SEGSORT_PARAM_RADIX_MIN_32 1
#define SEGSORT_PARAM_RADIX_MIN_64 2
#define SEGSORT_PARAM_STREAM_MAX_AVG 3
#define SEGSORT_PARAM_BUCKET_MIN_AVG 4
#define SEGSORT_PARAM_MSD 5
#define SEGSORT_PARAM_TINY_MAX_AVG 6
int segsort_set_param(int param, int64_t value);
int segsort_get_param(int param, int64_t *value);

/* Autotuner of plain calls (no counterpart in the reference).
 * segsort_tune_pairs_u32 sorts the given problem like segsort_pairs_u32, but
 * first measures it -- on copies of the inputs, each route timed three times
 * after one untimed call -- under candidate routes: the radix threshold
 * (4096, 2^15, 2^17, off), the streamed-tile kernel (never, always), the
 * long-segment kernel's resident CTAs per SM (1, 2, all), the bucket-route
 * threshold (off, 64, 256) and the MSD route (the other setting), one after
 * the other, keeping a candidate that is at least 2% faster.  The chosen
 * route is returned (optional outputs: its first three fields), recorded for
 * the problem's class in this process, and appended to cache_path (optional)
 * as a line
 *   plain k<key bytes> n<log2 n> len<log2 (n / nseg)> <radix> <stream> <ctas> <bucket> <msd>
 * (a line without the last two fields loads them at their defaults, 128 and
 * 1).  Later plain calls of that class (any key type of the same width) take the
 * recorded route.  segsort_tune_load reads such lines from a file into the
 * process's table (returns how many, or SEGSORT_ERR_INVALID_ARG when the
 * file cannot be read; lines of other formats are skipped);
 * segsort_tune_clear empties it; segsort_tune_lookup returns 1 and the
 * route recorded for a class, 0 when there is none.  The tuner synchronises
 * `stream` and allocates from the library's pool; the others are host-only. */
int segsort_tune_pairs_u32(uint32_t *d_keys, uint32_t *d_vals, int64_t n,
                           const int32_t *d_offsets, int32_t nseg, segsort_stream_t stream,
                           const char *cache_path, int64_t *radix_min,
                           int64_t *stream_max_avg, int32_t *merge_ctas_per_sm);
int segsort_tune_load(const char *cache_path);
void segsort_tune_clear(void);
int segsort_tune_lookup(int key_bytes, int64_t n, int32_t nseg, int64_t *radix_min,
                        int64_t *stream_max_avg, int32_t *merge_ctas_per_sm);

/* Self-test of the bounded device waits (no counterpart in the reference).
 * Launches a small kernel on a stream of its own whose wait can never
 * complete -- which = 0: a grid barrier that one of its two CTAs never
 * reaches; 1: an mbarrier phase expecting bytes that no copy supplies; 2: a
 * radix look-back on a tile that never publishes -- with a spin limit of a
 * few milliseconds.  The kernel gives up, records SEGSORT_ERR_TIMEOUT for
 * segsort_device_status() and returns; this call returns SEGSORT_OK once it
 * has finished.  No GPU fault is involved. */
int segsort_selftest_wait_timeout(int which);

/* Phase timing for benchmarks.  While enabled, every sort call records CUDA
 * events on its own stream around its tile-sort kernel and around its
 * large-segment kernels (a few microseconds of host work per call, no
 * device synchronisation).  segsort_profile_read() waits for the recorded
 * events, adds up their elapsed times and launch counts since the last
 * reset, and resets them when `reset` is non-zero.  No counterpart in the
 * reference, which times whole driver calls only (src/radixseg.cu:121-137). */
int segsort_profile_enable(int on);
int segsort_profile_read(double *tile_ms, double *large_ms, int64_t *tile_launches,
                         int64_t *large_launches, int reset);

#ifdef __cplusplus
}
#endif

#endif /* SEGSORT_H_ */
