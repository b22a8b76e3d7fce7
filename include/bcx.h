/*
 * bcx.h -- C ABI of libbcx, the GB300 (sm_103a) data-parallel core behind the
 * boost::compute algorithm headers.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns
 * a bcx_status.  Status values equal the OpenCL cl_int error codes wherever an
 * OpenCL counterpart exists, so a header can rethrow them unchanged as
 * boost::compute::opencl_error(status).
 *
 * Calling convention (mirrors the reference's queue-ordered algorithms,
 * include/boost/compute/command_queue.hpp:1403-1495):
 *   - all compute calls are asynchronous on the given stream (a cudaStream_t;
 *     NULL = the legacy default stream) and return once work is enqueued;
 *   - device pointers are raw CUDA device (or managed) pointers;
 *   - temporary storage follows a query/run pair: pass temp == NULL with a
 *     non-NULL temp_bytes to receive the size needed, then call again with
 *     temp pointing at that many bytes of device memory.  Passing
 *     temp == NULL and temp_bytes == NULL lets the library take the temporary
 *     from a stream-ordered pool (cudaMallocAsync) and release it on the
 *     stream after the work (the reference allocates temporaries per call,
 *     algorithm/detail/radix_sort.hpp:333-336);
 *   - no C++ exception crosses this ABI; bcx_last_error_string() describes the
 *     last failure on the calling thread.
 */
#ifndef BCX_H
#define BCX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int bcx_status;
typedef void *bcx_stream; /* a cudaStream_t */

/* ---- status codes ------------------------------------------------------ */
#define BCX_SUCCESS                   0
#define BCX_DEVICE_NOT_FOUND         -1   /* CL_DEVICE_NOT_FOUND */
#define BCX_MEM_ALLOCATION_FAILURE   -4   /* CL_MEM_OBJECT_ALLOCATION_FAILURE */
#define BCX_OUT_OF_RESOURCES         -5   /* CL_OUT_OF_RESOURCES (CUDA runtime error) */
#define BCX_BUILD_PROGRAM_FAILURE   -11   /* CL_BUILD_PROGRAM_FAILURE (NVRTC) */
#define BCX_INVALID_VALUE           -30   /* CL_INVALID_VALUE */
#define BCX_INVALID_KERNEL_NAME     -46   /* CL_INVALID_KERNEL_NAME */
#define BCX_INVALID_BUFFER_SIZE     -61   /* CL_INVALID_BUFFER_SIZE */
#define BCX_DEVICE_TIMEOUT        -9001   /* a bounded device-side wait gave up */
#define BCX_UNSUPPORTED           -9002   /* dtype/op combination not provided */

/* ---- element types (the radix-sortable fundamentals of
 *      algorithm/detail/radix_sort.hpp:41-47) ------------------------------ */
typedef enum {
    BCX_CHAR = 0, BCX_UCHAR = 1, BCX_SHORT = 2, BCX_USHORT = 3,
    BCX_INT = 4, BCX_UINT = 5, BCX_LONG = 6, BCX_ULONG = 7,
    BCX_FLOAT = 8, BCX_DOUBLE = 9
} bcx_dtype;

/* ---- built-in binary functors (functional/operator.hpp:57-92,
 *      functional/integer.hpp:24-25) -------------------------------------- */
typedef enum {
    BCX_PLUS = 0, BCX_MULTIPLIES = 1, BCX_MIN = 2, BCX_MAX = 3,
    BCX_BIT_AND = 4, BCX_BIT_OR = 5, BCX_BIT_XOR = 6,
    BCX_MINUS = 7, BCX_DIVIDES = 8, BCX_MODULUS = 9
} bcx_op;

/* ---- built-in unary functors used by transform (functional/math.hpp,
 *      functional/operator.hpp) ------------------------------------------- */
typedef enum {
    BCX_IDENTITY = 0, BCX_NEGATE = 1, BCX_ABS = 2, BCX_SQRT = 3,
    BCX_LOGICAL_NOT = 4, BCX_BIT_NOT = 5
} bcx_unary_op;

/* ---- runtime (replaces system.hpp / device.hpp / command_queue.hpp /
 *      buffer.hpp for the hot path) --------------------------------------- */

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
bcx_status bcx_get_version(int *version);
/* Text of the last failure on the calling thread ("" if none). */
const char *bcx_last_error_string(void);
/* system::devices() count -- system.hpp:181 */
bcx_status bcx_device_count(int *count);
/* Make `device` current for this thread (context selection, system.hpp:235-298). */
bcx_status bcx_set_device(int device);
/* device::name(), compute_units(), global_memory_size() -- device.hpp */
bcx_status bcx_device_info(int device, char *name, size_t name_len,
                           int *compute_units, size_t *global_mem_bytes);
/* command_queue(context, device) -- command_queue.hpp:78 */
bcx_status bcx_stream_create(bcx_stream *stream);
bcx_status bcx_stream_destroy(bcx_stream stream);
/* command_queue::finish() -- command_queue.hpp:1564 */
bcx_status bcx_stream_synchronize(bcx_stream stream);
/* Events: a marker recorded on a stream, completed when all work queued
 * before it has finished; timing is enabled.  They replace the OpenCL events
 * behind event.hpp (wait() :213, status() :173, duration via
 * clGetEventProfilingInfo :202) and command_queue::enqueue_marker (:1622) /
 * enqueue_barrier(wait_list) (:1601). */
typedef void *bcx_event; /* a cudaEvent_t */
bcx_status bcx_event_create(bcx_event *event);
bcx_status bcx_event_destroy(bcx_event event);
/* enqueue_marker: record `event` at the current end of `stream`. */
bcx_status bcx_event_record(bcx_event event, bcx_stream stream);
/* event::wait(): block the calling thread until the event has completed. */
bcx_status bcx_event_synchronize(bcx_event event);
/* event::status(): *complete = 1 when the event has completed, else 0. */
bcx_status bcx_event_query(bcx_event event, int *complete);
/* Milliseconds between two completed events recorded on the device. */
bcx_status bcx_event_elapsed_ms(bcx_event start, bcx_event end, float *ms);
/* enqueue_barrier(wait_list): later work on `stream` waits for `event`
 * (on the device; the host does not block). */
bcx_status bcx_stream_wait_event(bcx_stream stream, bcx_event event);
/* buffer(context, size) -- buffer.hpp; freed by bcx_free */
bcx_status bcx_malloc(void **ptr, size_t bytes);
bcx_status bcx_free(void *ptr);
/* Temporaries of one algorithm call, in stream order: the reference creates
 * each call's temporary buffers and releases them when the call returns
 * (detail/scan_on_gpu.hpp:216, detail/radix_sort.hpp:333-336); here they come
 * from the device's stream-ordered pool and are released in stream order, so
 * neither call blocks the host. */
bcx_status bcx_malloc_async(void **ptr, size_t bytes, bcx_stream stream);
bcx_status bcx_free_async(void *ptr, bcx_stream stream);
/* Host memory used in place as a buffer (buffer with CL_MEM_USE_HOST_PTR,
 * buffer.hpp:60-90; the storage of mapped_view, container/mapped_view.hpp:
 * 44-120): `bytes` of host memory at `host` are page-locked and mapped into the
 * device's address space, and *device_ptr is the address kernels use (on a
 * Grace host the GPU reads it over the CPU-GPU link).  read_only != 0 for
 * memory the device only reads.  Registrations of the same address are
 * counted; bcx_host_unregister releases one. */
bcx_status bcx_host_register(void *host, size_t bytes, int read_only, void **device_ptr);
bcx_status bcx_host_unregister(void *host);
/* Page-locked host memory (allocator/pinned_allocator.hpp). */
bcx_status bcx_malloc_host(void **ptr, size_t bytes);
bcx_status bcx_free_host(void *ptr);
/* enqueue_copy_buffer / enqueue_read_buffer / enqueue_write_buffer
 * (command_queue.hpp:400-700), direction inferred from the pointers. */
bcx_status bcx_memcpy_async(void *dst, const void *src, size_t bytes, bcx_stream stream);
/* enqueue_fill_buffer with a byte pattern (command_queue.hpp:1250). */
bcx_status bcx_memset_async(void *dst, int byte_value, size_t bytes, bcx_stream stream);
/* Synchronizes `stream`, then reports and clears any bounded device-side wait
 * that expired in this library's kernels since the last check
 * (BCX_DEVICE_TIMEOUT), or BCX_SUCCESS. */
bcx_status bcx_device_error_check(bcx_stream stream);
/* Test hook for failure detection (no counterpart in the reference, which
 * reports errors through exceptions only, exception/opencl_error.hpp:30):
 * runs one of the library's bounded device-side waits -- which = 0 the
 * onesweep digit look-back, 1 the scan tile look-back, 2 the bulk-copy
 * mbarrier wait -- against a status word or barrier that nothing publishes,
 * giving up after `polls` polls (1 .. 2^20).  The kernel returns normally and
 * the next bcx_device_error_check reports BCX_DEVICE_TIMEOUT. */
bcx_status bcx_debug_expire_wait(bcx_stream stream, int which, unsigned polls);

/* ---- sort ---------------------------------------------------------------
 * Radix path of detail::radix_sort / radix_sort_by_key
 * (algorithm/detail/radix_sort.hpp:253-462).  Keys are ordered by the
 * reference's radix() key transform (radix_sort.hpp:100-127) and the sort is
 * stable, so equal keys keep their input order and values follow their keys.
 * In place on `keys` (and `values`); any n. value_bytes in {1,2,4,8,16}. */
bcx_status bcx_radix_sort_keys(bcx_stream stream, bcx_dtype key_type, void *keys,
                               size_t n, int descending,
                               void *temp, size_t *temp_bytes);
bcx_status bcx_radix_sort_pairs(bcx_stream stream, bcx_dtype key_type,
                                size_t value_bytes, void *keys, void *values,
                                size_t n, int descending,
                                void *temp, size_t *temp_bytes);
/* Public compute::sort / sort_by_key dispatch for less<T> (descending = 0) and
 * greater<T> (descending = 1): sort.hpp:34-80 (n < 2 nothing, n <= 32 serial
 * insertion sort with the comparator, else radix) and sort_by_key.hpp:33-83
 * (n < 32 serial insertion sort by key, else radix). */
bcx_status bcx_sort_keys(bcx_stream stream, bcx_dtype key_type, void *keys,
                         size_t n, int descending,
                         void *temp, size_t *temp_bytes);
bcx_status bcx_sort_pairs(bcx_stream stream, bcx_dtype key_type,
                          size_t value_bytes, void *keys, void *values,
                          size_t n, int descending,
                          void *temp, size_t *temp_bytes);
/* compute::sort_by_key on host iterators: copies keys/values from host
 * memory, sorts them on the device, copies them back and synchronizes
 * (the host-iterator sort path, sort.hpp:125-148). */
bcx_status bcx_sort_pairs_host(bcx_stream stream, bcx_dtype key_type,
                               size_t value_bytes, void *host_keys,
                               void *host_values, size_t n, int descending);

/* ---- scan ---------------------------------------------------------------
 * exclusive_scan / inclusive_scan (exclusive_scan.hpp:55-104,
 * inclusive_scan.hpp:53-87, detail/scan_on_gpu.hpp:187-324).
 * out[i] = init op in[0] op ... op in[i-1] (exclusive; out[0] = init) or
 * in[0] op ... op in[i] (inclusive; init ignored).  `init` points at one
 * host value of `type` (NULL = 0).  in == out is allowed.  compensated = 1
 * with BCX_FLOAT/BCX_DOUBLE plus selects Neumaier-compensated tile sums with
 * an FP64 carry between tiles. */
bcx_status bcx_scan(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive,
                    const void *init, const void *in, void *out, size_t n,
                    int compensated, void *temp, size_t *temp_bytes);

/* Scan that allocates nothing (no counterpart in the reference: Boost.Compute
 * always allocates its temporaries per call).  For callers that cannot call
 * cudaMalloc when they scan -- a host application whose own pool owns every
 * device allocation, or a latency-critical path where an allocation that may
 * synchronize the device is not acceptable.  Same types, functors, init and
 * in-place rules as bcx_scan; the look-back scratch is one fixed 4 MiB array
 * inside libbcx that every GPU loading the library keeps until exit.  Limit:
 * at most 2^30 elements per call for 1-4 byte types, about 2^27-2^28 for
 * 8-byte types (the exact bound depends on the carry type); larger n is
 * rejected with BCX_INVALID_BUFFER_SIZE and a message giving the bound.  The
 * first call on each device looks up the array's device address; make that
 * first call before any stream capture.  Every call reuses the array (each
 * clears what it needs on its own stream first), so calls whose work
 * overlaps on the GPU race and must be serialized by the caller. */
bcx_status bcx_scan_noalloc(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive,
                            const void *init, const void *in, void *out, size_t n,
                            int compensated);

/* ---- reduce / accumulate -------------------------------------------------
 * reduce(first, last, result, op) into ONE device value at out_dev
 * (reduce.hpp:205-305, detail/reduce_on_gpu.hpp:169-280).  n == 0 writes
 * nothing (reduce.hpp:291-296).  Integer results are exact (mod 2^bits);
 * compensated = 1 with float plus uses Neumaier sums in warps and blocks and
 * an FP64 combine of the block partials. */
bcx_status bcx_reduce(bcx_stream stream, bcx_dtype type, bcx_op op,
                      const void *in, size_t n, void *out_dev, int compensated,
                      void *temp, size_t *temp_bytes);
/* accumulate(first, last, init, op) (accumulate.hpp:102-188): the value
 * init op reduce(in) written to out_dev; `init` is one host value; n == 0
 * writes init. */
bcx_status bcx_accumulate(bcx_stream stream, bcx_dtype type, bcx_op op,
                          const void *in, size_t n, const void *init,
                          void *out_dev, int compensated,
                          void *temp, size_t *temp_bytes);

/* ---- transform -----------------------------------------------------------
 * transform(first, last, result, f) = copy(transform_iterator) on the device
 * (transform.hpp:38-82, detail/copy_on_device.hpp:60-92). */
bcx_status bcx_transform_unary(bcx_stream stream, bcx_dtype type, bcx_unary_op op,
                               const void *in, void *out, size_t n);
/* transform(first1, last1, first2, result, op) with a built-in functor. */
bcx_status bcx_transform_binary(bcx_stream stream, bcx_dtype type, bcx_op op,
                                const void *in0, const void *in1, void *out,
                                size_t n);
/* transform(x, x+n, y, r, alpha*_1 + _2) (perf/perf_saxpy.cpp:50-56) for
 * float/double: r[i] = fma(alpha, x[i], y[i]) (single rounding). `alpha`
 * points at one host value of `type`. */
bcx_status bcx_transform_saxpy(bcx_stream stream, bcx_dtype type, const void *alpha,
                               const void *x, const void *y, void *out, size_t n);

/* ---- reduce_by_key -------------------------------------------------------
 * reduce_by_key(keys, keys+n, values, keys_out, values_out, op, equal_to)
 * (reduce_by_key.hpp, detail/reduce_by_key_with_scan.hpp:432-486): one output
 * per run of equal consecutive keys; the run count goes to *num_runs_dev
 * (a device uint64).  Key types int/uint/long/ulong/float (typed ==);
 * value types int/uint/long/ulong/float/double; functors plus, multiplies,
 * min, max.  compensated = 1 with float plus keeps Neumaier pairs.
 * keys_out may be NULL (the run keys are discarded, as with a
 * discard_iterator output). */
bcx_status bcx_reduce_by_key(bcx_stream stream, bcx_dtype key_type,
                             bcx_dtype value_type, bcx_op op,
                             const void *keys_in, const void *values_in, size_t n,
                             void *keys_out, void *values_out,
                             uint64_t *num_runs_dev, int compensated,
                             void *temp, size_t *temp_bytes);

/* ---- segmented algorithms ------------------------------------------------
 * No reference counterpart as one call: the reference's callers loop over
 * segments with one exclusive_scan / reduce each (scan_on_gpu.hpp:187-267,
 * reduce_on_gpu.hpp:169-280) or use reduce_by_key with segment ids
 * (reduce_by_key_with_scan.hpp:432-486).  Segments are CSR offsets in device
 * memory: nseg + 1 uint64 values, offsets[0] == 0, offsets[nseg] == n,
 * non-decreasing (empty segments allowed).  Types int/uint/long/ulong/float/
 * double; functors plus, multiplies, min, max.  One kernel launch each. */
/* Scan restarted at every segment start (exclusive: each segment starts at
 * *init). */
bcx_status bcx_segmented_scan(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive,
                              const void *init, const void *in, void *out, size_t n,
                              const uint64_t *offsets, size_t nseg, int compensated,
                              void *temp, size_t *temp_bytes);
/* out[s] = *init op fold(in[offsets[s] .. offsets[s+1])) for each segment
 * (*init for an empty segment). */
bcx_status bcx_segmented_reduce(bcx_stream stream, bcx_dtype type, bcx_op op, const void *in,
                                const uint64_t *offsets, size_t nseg, const void *init, void *out,
                                int compensated, void *temp, size_t *temp_bytes);

/* Segmented sort / sort_by_key: every segment [offsets[s], offsets[s+1]) is
 * sorted independently and stably in the order of bcx_radix_sort_pairs
 * (value_bytes = 0 sorts keys only).  Replaces one sort_by_key call per
 * segment (sort_by_key.hpp:33-163).  Small segments are sorted in shared
 * memory by one block each, large ones by segment-confined onesweep passes;
 * all work is asynchronous on `stream` and reads nothing back, so the call
 * can be captured in a CUDA graph.  n < 2^31. */
bcx_status bcx_segmented_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes,
                                    void *keys, void *values, size_t n, const uint64_t *offsets,
                                    size_t nseg, int descending, void *temp, size_t *temp_bytes);

/* ---- request server (continuous batching) --------------------------------
 * No reference counterpart: the reference serves one blocking call at a time
 * on a queue.  A server owns `slots` CUDA streams and a device-memory budget
 * (0 = half of the free memory).  Requests are admitted in arrival order as
 * slots and memory free up; small waiting requests of the same kind, dtype and
 * value size are packed into one segmented launch; large ones run alone.
 * Buffers are host memory (use page-locked memory for copy overlap) or, with
 * BCX_REQ_DEVICE_RESIDENT, device memory; either way they must stay valid
 * until bcx_server_wait returns.  Sort requests read keys (and values) and
 * write the stably sorted pairs to out (and out_values), which may alias the
 * inputs; scan requests write the exclusive plus-scan of keys to out; reduce
 * requests write the plus-sum of keys to out[0].  Float scans and sums use the
 * compensated kernels. */
typedef struct bcx_server bcx_server;
typedef enum { BCX_REQ_SORT_PAIRS = 0, BCX_REQ_EXCLUSIVE_SCAN = 1, BCX_REQ_REDUCE = 2 } bcx_req_kind;
#define BCX_REQ_DEVICE_RESIDENT 1
typedef struct {
    int kind;            /* bcx_req_kind */
    bcx_dtype dtype;     /* key / element type */
    size_t value_bytes;  /* sort: bytes per value (0 = keys only) */
    size_t n;            /* elements */
    int flags;           /* BCX_REQ_DEVICE_RESIDENT: all buffers are device memory */
    const void *keys;    /* sort keys, scan / reduce input */
    const void *values;  /* sort values */
    void *out;           /* sorted keys, scan output (n elements), reduce output (1 element) */
    void *out_values;    /* sorted values */
} bcx_request;
typedef struct {
    uint64_t completed, batches, batched_requests, pending;
    size_t used_bytes;
    double p50_ms, p99_ms, max_ms; /* submit -> results in host memory */
} bcx_server_stats_t;
bcx_status bcx_server_create(bcx_server **server, int slots, size_t memory_budget_bytes);
/* Requests of at most small_limit elements may be batched, up to batch_elems
 * elements and batch_count requests per batch (0 keeps a value). */
bcx_status bcx_server_configure(bcx_server *server, size_t small_limit, size_t batch_elems,
                                size_t batch_count);
/* Test hook (no counterpart in the reference): admission sees
 * `fake_free_bytes` of free device memory instead of the measured figure (0 =
 * measure), and the next `fail_allocations` batches fail as if their device
 * allocation had failed (their requests end with BCX_MEM_ALLOCATION_FAILURE;
 * later requests are served normally). */
bcx_status bcx_server_inject_faults(bcx_server *server, size_t fake_free_bytes, int fail_allocations);
bcx_status bcx_server_submit(bcx_server *server, const bcx_request *request, uint64_t *ticket);
/* Blocks until the request's results are in place (host or device buffers). */
bcx_status bcx_server_wait(bcx_server *server, uint64_t ticket, double *latency_ms);
/* As bcx_server_wait, for at most timeout_ms milliseconds (negative: no
 * limit); returns BCX_DEVICE_TIMEOUT when the request is still running, and
 * the ticket stays valid. */
bcx_status bcx_server_wait_for(bcx_server *server, uint64_t ticket, double timeout_ms, double *latency_ms);
bcx_status bcx_server_drain(bcx_server *server);
bcx_status bcx_server_stats(bcx_server *server, bcx_server_stats_t *stats);
bcx_status bcx_server_reset_stats(bcx_server *server);
/* Waits up to 60 s for queued and running requests, then stops the scheduler
 * and frees the server; if requests are still running it returns
 * BCX_DEVICE_TIMEOUT and leaves the server alive. */
bcx_status bcx_server_destroy(bcx_server *server);

/* ---- run-time compiled kernels ------------------------------------------
 * Replaces clBuildProgram + program_cache (utility/program_cache.hpp:52-168,
 * program.hpp:638-692) and the offline binary cache (program.hpp:656-690):
 * `source` is CUDA C++ generated by the drop-in headers for user functions,
 * lambda expressions and iterator expressions (detail/meta_kernel.hpp).  It
 * is compiled once with NVRTC for the current device's architecture and
 * cached (LRU, 256 modules by default; cubins also kept in $BCX_CACHE_DIR when
 * set).  A failed build returns BCX_BUILD_PROGRAM_FAILURE; the NVRTC log is
 * then available from bcx_jit_build_log.  Kernel handles stay valid until
 * their module is evicted: fetch the handle right before each launch. */
typedef void *bcx_jit_kernel;
bcx_status bcx_jit_get_kernel(const char *source, const char *kernel_name, const char *options,
                              bcx_jit_kernel *kernel);
/* Launch `kernel` (args as for cudaLaunchKernel) on `stream`. */
bcx_status bcx_jit_launch(bcx_jit_kernel kernel, unsigned grid, unsigned block, size_t shared_bytes,
                          bcx_stream stream, void **args);
bcx_status bcx_jit_build_log(char *buf, size_t len, size_t *needed);
bcx_status bcx_jit_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *compiles,
                               uint64_t *disk_hits, uint64_t *entries);
/* capacity 0 keeps the current capacity; clear != 0 unloads every module. */
bcx_status bcx_jit_cache_configure(size_t capacity, int clear);
/* Streaming multiprocessors of the current device (grid sizing of generated
 * kernels). */
bcx_status bcx_device_sm_count(int *sm_count);
/* Device address of the current device's error word: generated kernels with
 * bounded waits record an expired wait there (atomicOr of 1), and
 * bcx_device_error_check reports it.  (The reference reports errors through
 * exceptions only, exception/opencl_error.hpp:30.) */
bcx_status bcx_device_error_word(void **word);

/* ---- tuning parameters and autotuner (detail::parameter_cache,
 *      detail/parameter_cache.hpp:38-110; the perf/ tuning programs that fill
 *      it) ---------------------------------------------------------------
 * A per-device table (object, parameter) -> unsigned, kept in memory and, when
 * BCX_CACHE_DIR is set, in $BCX_CACHE_DIR/tune/<device name>.json (read on
 * first use, written by bcx_param_save and by every tuner).  Tunables read at
 * dispatch time:
 *   "segmented_sort_k<key bits>_v<value bytes>": "small_tile" (1024, 2048 or
 *       4096: segments up to this many pairs sort in shared memory),
 *       "small_blocks_per_sm" (0 = as many as fit);
 *   "segmented_scan_<type>": "items_per_thread" (32/64 for 4-byte types, 8/16
 *       for 8-byte types);
 *   "segmented_reduce_<type>": "blocks_per_sm".
 * Temporary-storage sizes never depend on these values. */
bcx_status bcx_param_get(const char *object, const char *parameter, unsigned default_value, unsigned *value);
bcx_status bcx_param_set(const char *object, const char *parameter, unsigned value);
bcx_status bcx_param_save(void);
/* Forgets the in-memory tables (the next lookup re-reads the file). */
bcx_status bcx_param_clear(void);
/* Autotuners: time every candidate value of the operation's tunables on the
 * caller's workload (CUDA events, median of 3 runs after a warm-up; inputs are
 * left unchanged -- trial runs sort copies and write scratch outputs), store
 * the fastest and save the table.  `report` (optional) receives one line per
 * trial: "<object>.<parameter>=<value> <ms> ms".  They synchronize the
 * stream and allocate scratch memory: not for use inside stream capture. */
bcx_status bcx_tune_segmented_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes,
                                         const void *keys, const void *values, size_t n, const uint64_t *offsets,
                                         size_t nseg, char *report, size_t report_len);
bcx_status bcx_tune_segmented_scan(bcx_stream stream, bcx_dtype type, const void *in, size_t n,
                                   const uint64_t *offsets, size_t nseg, char *report, size_t report_len);
bcx_status bcx_tune_segmented_reduce(bcx_stream stream, bcx_dtype type, const void *in, const uint64_t *offsets,
                                     size_t nseg, char *report, size_t report_len);

/* ---- profiling (command_queue::enable_profiling / event::duration,
 *      command_queue.hpp:82, event.hpp:269) --------------------------------
 * When enabled, every kernel this library launches is bracketed by CUDA
 * events on its stream; bcx_profile_read sums the durations per kernel name
 * (synchronizing first).  Names are "<family>" strings such as
 * "radix_onesweep", "scan_lookback", "reduce_partials". */
bcx_status bcx_profile_enable(int enable);
bcx_status bcx_profile_reset(void);
/* Fills up to `cap` entries; *count receives the number of kernel names. */
bcx_status bcx_profile_read(char *names, size_t name_stride, uint64_t *launches,
                            double *total_ms, size_t cap, size_t *count);

#ifdef __cplusplus
}
#endif

#endif /* BCX_H */
