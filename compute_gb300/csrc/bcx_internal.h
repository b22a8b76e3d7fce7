// bcx_internal.h -- host-side plumbing shared by the libbcx translation units:
// per-thread error text, CUDA error mapping, per-device state, the temporary
// storage protocol and the optional per-kernel event profiler.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
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
};
// State of the current device (created on first use).
bcx_status current_device_state(DeviceState **out);

size_t dtype_size(bcx_dtype t);
bool dtype_valid(int t);

// Bytes rounded up to a 256-byte boundary (alignment of every sub-buffer
// carved out of a temporary allocation).
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

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

// Checks the launch that just happened.
bcx_status launch_status(const char *kernel);

}  // namespace bcx
