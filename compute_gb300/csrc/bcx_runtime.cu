// bcx_runtime.cu -- runtime half of the C ABI: devices, streams, memory,
// error text, the temporary-storage protocol and the kernel profiler.
//
// Replaces, for the hot path only, the reference's OpenCL wrapper layer:
// system::default_queue (system.hpp:181-298), command_queue
// (command_queue.hpp:78-1570), buffer (buffer.hpp) and event profiling
// (event.hpp:204-269).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "bcx.h"
#include "bcx_internal.h"

namespace bcx {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

bcx_status cuda_status(cudaError_t e, const char *what) {
  set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  if (e == cudaErrorMemoryAllocation) return BCX_MEM_ALLOCATION_FAILURE;
  if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) return BCX_DEVICE_NOT_FOUND;
  if (e == cudaErrorInvalidValue) return BCX_INVALID_VALUE;
  return BCX_OUT_OF_RESOURCES;
}

static std::mutex g_dev_mu;
static std::map<int, DeviceState *> g_devices;

cudaError_t smem_optin(const void *kernel, int bytes, std::atomic<uint64_t> *done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev < 64 ? (uint64_t(1) << dev) : 0;
  if (bit && (done->load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done->fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

bcx_status current_device_state(DeviceState **out) {
  int dev = 0;
  BCX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_dev_mu);
  auto it = g_devices.find(dev);
  if (it != g_devices.end()) {
    *out = it->second;
    return BCX_SUCCESS;
  }
  DeviceState *st = new DeviceState();
  st->device = dev;
  BCX_CUDA(cudaDeviceGetAttribute(&st->sm_count, cudaDevAttrMultiProcessorCount, dev));
  BCX_CUDA(cudaMalloc(&st->err_word, sizeof(uint32_t)));
  BCX_CUDA(cudaMemset(st->err_word, 0, sizeof(uint32_t)));
  // Temporaries come from the device's default stream-ordered pool.  Its
  // default release threshold (0) hands freed memory back to the driver at
  // every synchronization, so a sequence of blocking calls would map and unmap
  // its temporaries each time; keep freed memory cached in the pool instead
  // (BCX_POOL_RELEASE_THRESHOLD, in bytes, overrides).
  {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t threshold = UINT64_MAX;
      if (const char *env = std::getenv("BCX_POOL_RELEASE_THRESHOLD")) threshold = std::strtoull(env, nullptr, 10);
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
  }
  BCX_CUDA(cudaStreamCreateWithFlags(&st->aux_stream, cudaStreamNonBlocking));
  BCX_CUDA(cudaDeviceSynchronize());
  g_devices[dev] = st;
  *out = st;
  return BCX_SUCCESS;
}

DeviceState *existing_device_state() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  auto it = g_devices.find(dev);
  return it == g_devices.end() ? nullptr : it->second;
}

size_t dtype_size(bcx_dtype t) {
  switch (t) {
    case BCX_CHAR: case BCX_UCHAR: return 1;
    case BCX_SHORT: case BCX_USHORT: return 2;
    case BCX_INT: case BCX_UINT: case BCX_FLOAT: return 4;
    case BCX_LONG: case BCX_ULONG: case BCX_DOUBLE: return 8;
  }
  return 0;
}

bool dtype_valid(int t) { return t >= BCX_CHAR && t <= BCX_DOUBLE; }

const char *dtype_name(bcx_dtype t) {
  static const char *names[] = {"char", "uchar", "short", "ushort", "int", "uint", "long", "ulong", "float", "double"};
  return dtype_valid(int(t)) ? names[int(t)] : "invalid";
}

TempStorage::~TempStorage() {
  if (owned_ && ptr_) cudaFreeAsync(ptr_, stream_);
}

bcx_status TempStorage::acquire(void *temp, size_t *temp_bytes, size_t need,
                                cudaStream_t s, bool *query_only) {
  *query_only = false;
  if (temp == nullptr && temp_bytes != nullptr) {
    *temp_bytes = need;
    *query_only = true;
    return BCX_SUCCESS;
  }
  if (temp != nullptr) {
    BCX_CHECK(temp_bytes != nullptr && *temp_bytes >= need, BCX_INVALID_BUFFER_SIZE,
              "temporary storage too small: %zu bytes given, %zu needed",
              temp_bytes ? *temp_bytes : size_t(0), need);
    ptr_ = temp;
    owned_ = false;
    return BCX_SUCCESS;
  }
  if (need == 0) return BCX_SUCCESS;
  stream_ = s;
  cudaError_t e = cudaMallocAsync(&ptr_, need, s);
  if (e != cudaSuccess) {
    ptr_ = nullptr;
    return cuda_status(e, "cudaMallocAsync(temporary storage)");
  }
  owned_ = true;
  return BCX_SUCCESS;
}

// ---------------------------------------------------------------------------
// Profiler.
struct ProfRecord {
  const char *name;
  cudaEvent_t start, stop;
};
struct ProfTotal {
  uint64_t launches = 0;
  double ms = 0.0;
};
static std::mutex g_prof_mu;
static volatile int g_prof_on = 0;
static std::vector<ProfRecord> g_prof_pending;
static std::map<std::string, ProfTotal> g_prof_totals;

bool profiling_enabled() { return g_prof_on != 0; }

KernelScope::KernelScope(const char *name, cudaStream_t s) : name_(name), stream_(s) {
  if (!g_prof_on) return;
  if (cudaEventCreate(&start_) == cudaSuccess) cudaEventRecord(start_, s);
}

KernelScope::~KernelScope() {
  if (!start_) return;
  cudaEvent_t stop = nullptr;
  if (cudaEventCreate(&stop) != cudaSuccess) {
    cudaEventDestroy(start_);
    return;
  }
  cudaEventRecord(stop, stream_);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_pending.push_back(ProfRecord{name_, start_, stop});
}

static void prof_drain_locked() {
  for (auto &r : g_prof_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.stop) == cudaSuccess &&
        cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
      ProfTotal &t = g_prof_totals[r.name];
      t.launches += 1;
      t.ms += ms;
    }
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  g_prof_pending.clear();
}

bcx_status launch_status(const char *kernel) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, kernel);
  return BCX_SUCCESS;
}

}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_get_version(int *version) {
  if (!version) return BCX_INVALID_VALUE;
  *version = 1 * 10000 + 0 * 100 + 0;
  return BCX_SUCCESS;
}

const char *bcx_last_error_string(void) { return g_last_error.c_str(); }

bcx_status bcx_device_count(int *count) {
  BCX_CHECK(count != nullptr, BCX_INVALID_VALUE, "count is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
    cudaGetLastError();
    *count = 0;
    return BCX_SUCCESS;
  }
  BCX_CUDA(e);
  *count = n;
  return BCX_SUCCESS;
}

bcx_status bcx_set_device(int device) {
  BCX_CUDA(cudaSetDevice(device));
  return BCX_SUCCESS;
}

bcx_status bcx_device_info(int device, char *name, size_t name_len, int *compute_units,
                           size_t *global_mem_bytes) {
  cudaDeviceProp p;
  BCX_CUDA(cudaGetDeviceProperties(&p, device));
  if (name && name_len) {
    strncpy(name, p.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (compute_units) *compute_units = p.multiProcessorCount;
  if (global_mem_bytes) *global_mem_bytes = p.totalGlobalMem;
  return BCX_SUCCESS;
}

bcx_status bcx_stream_create(bcx_stream *stream) {
  BCX_CHECK(stream != nullptr, BCX_INVALID_VALUE, "stream is NULL");
  cudaStream_t s;
  BCX_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = (bcx_stream)s;
  return BCX_SUCCESS;
}

bcx_status bcx_stream_destroy(bcx_stream stream) {
  BCX_CUDA(cudaStreamDestroy((cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_stream_synchronize(bcx_stream stream) {
  BCX_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_event_create(bcx_event *event) {
  BCX_CHECK(event != nullptr, BCX_INVALID_VALUE, "event is NULL");
  cudaEvent_t e;
  BCX_CUDA(cudaEventCreate(&e));
  *event = (bcx_event)e;
  return BCX_SUCCESS;
}

bcx_status bcx_event_destroy(bcx_event event) {
  BCX_CHECK(event != nullptr, BCX_INVALID_VALUE, "event is NULL");
  BCX_CUDA(cudaEventDestroy((cudaEvent_t)event));
  return BCX_SUCCESS;
}

bcx_status bcx_event_record(bcx_event event, bcx_stream stream) {
  BCX_CHECK(event != nullptr, BCX_INVALID_VALUE, "event is NULL");
  BCX_CUDA(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_event_synchronize(bcx_event event) {
  BCX_CHECK(event != nullptr, BCX_INVALID_VALUE, "event is NULL");
  BCX_CUDA(cudaEventSynchronize((cudaEvent_t)event));
  return BCX_SUCCESS;
}

bcx_status bcx_event_query(bcx_event event, int *complete) {
  BCX_CHECK(event != nullptr && complete != nullptr, BCX_INVALID_VALUE, "event or complete is NULL");
  const cudaError_t e = cudaEventQuery((cudaEvent_t)event);
  if (e == cudaErrorNotReady) {
    // Not an error: the work before the event is still running.  Clear it from
    // the runtime's last-error slot so a later launch check does not report it.
    if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
    *complete = 0;
    return BCX_SUCCESS;
  }
  BCX_CUDA(e);
  *complete = 1;
  return BCX_SUCCESS;
}

bcx_status bcx_event_elapsed_ms(bcx_event start, bcx_event end, float *ms) {
  BCX_CHECK(start != nullptr && end != nullptr && ms != nullptr, BCX_INVALID_VALUE, "NULL argument");
  BCX_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end));
  return BCX_SUCCESS;
}

bcx_status bcx_stream_wait_event(bcx_stream stream, bcx_event event) {
  BCX_CHECK(event != nullptr, BCX_INVALID_VALUE, "event is NULL");
  BCX_CUDA(cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)event, 0));
  return BCX_SUCCESS;
}

bcx_status bcx_malloc(void **ptr, size_t bytes) {
  BCX_CHECK(ptr != nullptr, BCX_INVALID_VALUE, "ptr is NULL");
  *ptr = nullptr;
  if (bytes == 0) return BCX_SUCCESS;
  BCX_CUDA(cudaMalloc(ptr, bytes));
  return BCX_SUCCESS;
}

bcx_status bcx_free(void *ptr) {
  if (ptr) BCX_CUDA(cudaFree(ptr));
  return BCX_SUCCESS;
}

static std::mutex g_reg_mu;
static std::map<void *, int> g_registered;  // host address -> registrations

bcx_status bcx_host_register(void *host, size_t bytes, int read_only, void **device_ptr) {
  BCX_CHECK(host != nullptr && device_ptr != nullptr && bytes > 0, BCX_INVALID_VALUE, "bad host registration");
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_registered.find(host);
  if (it == g_registered.end()) {
    unsigned flags = cudaHostRegisterMapped | cudaHostRegisterPortable;
    if (read_only) flags |= cudaHostRegisterReadOnly;
    BCX_CUDA(cudaHostRegister(host, bytes, flags));
    it = g_registered.emplace(host, 0).first;
  }
  cudaError_t e = cudaHostGetDevicePointer(device_ptr, host, 0);
  if (e != cudaSuccess) {
    if (it->second == 0) {
      cudaHostUnregister(host);
      g_registered.erase(it);
    }
    return cuda_status(e, "cudaHostGetDevicePointer");
  }
  it->second += 1;
  return BCX_SUCCESS;
}

bcx_status bcx_host_unregister(void *host) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_registered.find(host);
  BCX_CHECK(it != g_registered.end(), BCX_INVALID_VALUE, "host memory %p is not registered", host);
  if (--it->second == 0) {
    g_registered.erase(it);
    BCX_CUDA(cudaHostUnregister(host));
  }
  return BCX_SUCCESS;
}

bcx_status bcx_malloc_async(void **ptr, size_t bytes, bcx_stream stream) {
  BCX_CHECK(ptr != nullptr, BCX_INVALID_VALUE, "ptr is NULL");
  *ptr = nullptr;
  if (bytes == 0) return BCX_SUCCESS;
  DeviceState *st = nullptr;
  bcx_status rc = current_device_state(&st);  // keeps freed memory cached in the pool
  if (rc) return rc;
  BCX_CUDA(cudaMallocAsync(ptr, bytes, (cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_free_async(void *ptr, bcx_stream stream) {
  if (ptr) BCX_CUDA(cudaFreeAsync(ptr, (cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_device_error_word(void **word) {
  BCX_CHECK(word != nullptr, BCX_INVALID_VALUE, "NULL argument");
  DeviceState *st = nullptr;
  bcx_status rc = current_device_state(&st);
  if (rc) return rc;
  *word = st->err_word;
  return BCX_SUCCESS;
}

bcx_status bcx_malloc_host(void **ptr, size_t bytes) {
  BCX_CHECK(ptr != nullptr, BCX_INVALID_VALUE, "ptr is NULL");
  *ptr = nullptr;
  if (bytes == 0) return BCX_SUCCESS;
  BCX_CUDA(cudaMallocHost(ptr, bytes));
  return BCX_SUCCESS;
}

bcx_status bcx_free_host(void *ptr) {
  if (ptr) BCX_CUDA(cudaFreeHost(ptr));
  return BCX_SUCCESS;
}

bcx_status bcx_memcpy_async(void *dst, const void *src, size_t bytes, bcx_stream stream) {
  if (bytes == 0) return BCX_SUCCESS;
  BCX_CHECK(dst && src, BCX_INVALID_VALUE, "memcpy with NULL pointer");
  BCX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_memset_async(void *dst, int byte_value, size_t bytes, bcx_stream stream) {
  if (bytes == 0) return BCX_SUCCESS;
  BCX_CHECK(dst != nullptr, BCX_INVALID_VALUE, "memset with NULL pointer");
  BCX_CUDA(cudaMemsetAsync(dst, byte_value, bytes, (cudaStream_t)stream));
  return BCX_SUCCESS;
}

bcx_status bcx_device_error_check(bcx_stream stream) {
  BCX_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  // Both error words of the current device: the library's (if any entry point
  // set up the device) and the no-alloc scan's (if it ran here).  Checking
  // sets up nothing, so a caller of the no-alloc scan stays allocation-free.
  uint32_t word = 0;
  if (DeviceState *st = existing_device_state()) {
    BCX_CUDA(cudaMemcpy(&word, st->err_word, sizeof(word), cudaMemcpyDeviceToHost));
    if (word) BCX_CUDA(cudaMemset(st->err_word, 0, sizeof(uint32_t)));
  }
  uint32_t na = 0;
  bcx_status rc = noalloc_take_error(&na);
  if (rc) return rc;
  word |= na;
  if (word) {
    BCX_CUDA(cudaDeviceSynchronize());
    set_error("a bounded device-side wait expired (error word 0x%x)", word);
    return BCX_DEVICE_TIMEOUT;
  }
  return BCX_SUCCESS;
}

bcx_status bcx_profile_enable(int enable) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = enable ? 1 : 0;
  return BCX_SUCCESS;
}

bcx_status bcx_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  prof_drain_locked();
  g_prof_totals.clear();
  return BCX_SUCCESS;
}

bcx_status bcx_profile_read(char *names, size_t name_stride, uint64_t *launches,
                            double *total_ms, size_t cap, size_t *count) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  prof_drain_locked();
  size_t i = 0;
  for (auto &kv : g_prof_totals) {
    if (i < cap) {
      if (names && name_stride) {
        strncpy(names + i * name_stride, kv.first.c_str(), name_stride - 1);
        names[i * name_stride + name_stride - 1] = 0;
      }
      if (launches) launches[i] = kv.second.launches;
      if (total_ms) total_ms[i] = kv.second.ms;
    }
    ++i;
  }
  if (count) *count = g_prof_totals.size();
  return BCX_SUCCESS;
}

}  // extern "C"
