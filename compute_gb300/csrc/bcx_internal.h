// bcx_internal.h -- host-side plumbing shared by the libbcx translation units:
// per-thread error text, CUDA error mapping, per-device state, the temporary
// storage protocol and the optional per-kernel event profiler.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <atomic>
#include <string>

#include "bcx.h"

namespace bcx {

// Per-thread "last error" text returned by bcx_last_error_string().
void set_error(const char *fmt, ...);
void clear_error();

// Maps a CUDA runtime error to a bcx_status and records its text.
bcx_status cuda_status(cudaError_t e, const char *what);

#define BCX_CUDA(call)                                             \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return ::bcx::cuda_status(e_, #call);   \
  } while (0)

#define BCX_CHECK(cond, status, ...)                               \
  do {                                                             \
    if (!(cond)) {                                                 \
      ::bcx::set_error(__VA_ARGS__);                               \
      return (status);                                             \
    }                                                              \
  } while (0)

// Per-device state: SM count and the device-resident error word that bounded
// spin-waits report into.
struct DeviceState {
  int device = -1;
  int sm_count = 0;
  uint32_t *err_word = nullptr;  // device memory, 4 bytes
  cudaStream_t aux_stream = nullptr;  // second stream for copies split in two
};
// State of the current device (created on first use).
bcx_status current_device_state(DeviceState **out);

// Opts `kernel` into `bytes` of dynamic shared memory (needed above 48 KB)
// on the current device, once per device: `done` keeps one bit per device
// already opted in, one mask per kernel.
cudaError_t smem_optin(const void *kernel, int bytes, std::atomic<uint64_t> *done);

size_t dtype_size(bcx_dtype t);
bool dtype_valid(int t);
const char *dtype_name(bcx_dtype t);  // OpenCL C spelling: "int", "ulong", ...

// Bytes rounded up to a 256-byte boundary (alignment of every sub-buffer
// carved out of a temporary allocation).
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Temporary storage protocol shared by every algorithm entry point:
//   temp == NULL && temp_bytes != NULL -> size query (returns 1 = "query done")
//   temp == NULL && temp_bytes == NULL -> stream-ordered pool allocation
//   temp != NULL                        -> caller-provided, *temp_bytes checked
class TempStorage {
 public:
  TempStorage() = default;
  ~TempStorage();
  // Returns BCX_SUCCESS and sets *query_only when the call only asked for the
  // size.
  bcx_status acquire(void *temp, size_t *temp_bytes, size_t need, cudaStream_t s,
                     bool *query_only);
  void *ptr() const { return ptr_; }

 private:
  void *ptr_ = nullptr;
  bool owned_ = false;
  cudaStream_t stream_ = nullptr;
};

// Kernel profiler (command_queue::enable_profiling analogue).  Scope objects
// bracket one launch with CUDA events on the launching stream when profiling
// is on; otherwise they cost one relaxed flag load.
class KernelScope {
 public:
  KernelScope(const char *name, cudaStream_t s);
  ~KernelScope();

 private:
  const char *name_;
  cudaStream_t stream_;
  cudaEvent_t start_ = nullptr;
};
bool profiling_enabled();

// Reads and clears the error word of the no-alloc scan on the current device
// (0 if that entry point never ran there).  Sets up no device state.
bcx_status noalloc_take_error(uint32_t *word);
// The library's state of the current device if an entry point has created it,
// else nullptr (never creates it).
DeviceState *existing_device_state();

// Checks the launch that just happened.
bcx_status launch_status(const char *kernel);

// Tuning parameters of the current device (bcx_tune.cpp): the stored value of
// (object, parameter), or default_value when none is stored.
uint32_t param_get(const std::string &object, const char *parameter, uint32_t default_value);
void param_set(const std::string &object, const char *parameter, uint32_t value);
bcx_status param_save();
// Largest small-segment tile the segmented sort is compiled for with these
// key and value sizes (bcx_segmented_sort.cu).
uint32_t segsort_small_tile_limit(size_t key_bytes, size_t value_bytes);
// Items per thread the segmented scan is compiled for (bcx_segmented.cu).
void segscan_shapes(size_t elem_bytes, uint32_t *small, uint32_t *large);

// One piece of a batched gather/scatter: `bytes` bytes from src to dst, both
// device-accessible.  The request server splits every buffer it moves into
// pieces of at most kCopyChunkBytes so that one launch of copy_chunks (one
// block per piece) moves the buffers of a whole batch.
struct CopyChunk {
  const void *src;
  void *dst;
  uint64_t bytes;
  uint64_t reserved;
};
constexpr size_t kCopyChunkBytes = size_t(64) << 10;
// chunks: device array of `count` pieces.
bcx_status copy_chunks(const CopyChunk *chunks, size_t count, cudaStream_t s);

}  // namespace bcx
