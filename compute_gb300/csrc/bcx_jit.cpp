// bcx_jit.cpp -- run-time compilation of generated kernels (NVRTC) and the
// program cache.
//
// Reference: user functors and iterator expressions become OpenCL C source
// (detail/meta_kernel.hpp:270-401, function.hpp:116-463) that is built with
// clBuildProgram and kept in program_cache, an LRU of built programs keyed by
// (key, options) (utility/program_cache.hpp:52-168), with an optional on-disk
// binary cache under $HOME/.boost_compute (program.hpp:656-690).
//
// Here: the drop-in headers emit CUDA C++ source; bcx_jit_get_kernel compiles
// it with NVRTC straight to a cubin for the current device's architecture
// (sm_103a on GB300), loads it with the runtime library API and returns a
// kernel handle.  Modules are cached in memory, least recently used first out,
// keyed by a 128-bit hash of (source, kernel name, options, architecture) with
// the full key text compared on every hit.  When BCX_CACHE_DIR is set, cubins
// are also written there and reused by later processes.  A compile failure
// returns BCX_BUILD_PROGRAM_FAILURE and keeps the NVRTC log for
// bcx_jit_build_log (the reference throws program_build_failure with the
// build log, program.hpp:266-281).
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <list>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "bcx.h"
#include "bcx_internal.h"

namespace bcx {
namespace {

struct JitEntry {
  std::string key;  // full key text (source + name + options + arch)
  cudaLibrary_t library = nullptr;
  cudaKernel_t kernel = nullptr;
};

struct JitCache {
  std::mutex mu;
  std::list<JitEntry> lru;  // front = most recent
  std::map<std::string, std::list<JitEntry>::iterator> index;  // hash hex -> entry
  size_t capacity = 256;
  uint64_t hits = 0, misses = 0, compiles = 0, disk_hits = 0;
  std::string last_log;
};

JitCache &cache() {
  static JitCache *c = new JitCache();
  return *c;
}

uint64_t fnv1a(const std::string &s, uint64_t seed) {
  uint64_t h = 1469598103934665603ull ^ seed;
  for (unsigned char ch : s) {
    h ^= ch;
    h *= 1099511628211ull;
  }
  return h;
}

std::string hex_key(const std::string &text) {
  char buf[40];
  snprintf(buf, sizeof(buf), "%016llx%016llx", (unsigned long long)fnv1a(text, 0),
           (unsigned long long)fnv1a(text, 0x9e3779b97f4a7c15ull));
  return buf;
}

bcx_status device_arch(std::string *arch) {
  int dev = 0, major = 0, minor = 0;
  BCX_CUDA(cudaGetDevice(&dev));
  BCX_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  BCX_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  char buf[32];
  // Architecture-specific features (the "a" targets) exist from 9.0 on.
  snprintf(buf, sizeof(buf), "sm_%d%d%s", major, minor, major >= 9 ? "a" : "");
  *arch = buf;
  return BCX_SUCCESS;
}

std::string disk_path(const std::string &hex) {
  const char *dir = std::getenv("BCX_CACHE_DIR");
  if (!dir || !*dir) return std::string();
  return std::string(dir) + "/" + hex + ".cubin";
}

// Disk entry: [8-byte key length][key text][cubin].  The key text is compared
// on load, so a hash collision can never load the wrong module.
bool disk_load(const std::string &path, const std::string &key, std::vector<char> *cubin) {
  if (path.empty()) return false;
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  uint64_t klen = 0;
  f.read(reinterpret_cast<char *>(&klen), sizeof(klen));
  if (!f || klen != key.size()) return false;
  std::string k(klen, '\0');
  f.read(&k[0], std::streamsize(klen));
  if (!f || k != key) return false;
  std::vector<char> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (data.empty()) return false;
  cubin->swap(data);
  return true;
}

void disk_store(const std::string &path, const std::string &key, const std::vector<char> &cubin) {
  if (path.empty()) return;
  const std::string tmp = path + ".tmp";
  std::ofstream f(tmp, std::ios::binary);
  if (!f) return;
  uint64_t klen = key.size();
  f.write(reinterpret_cast<const char *>(&klen), sizeof(klen));
  f.write(key.data(), std::streamsize(key.size()));
  f.write(cubin.data(), std::streamsize(cubin.size()));
  f.close();
  std::rename(tmp.c_str(), path.c_str());
}

std::vector<std::string> split_options(const char *options) {
  std::vector<std::string> out;
  if (!options) return out;
  std::istringstream is(options);
  std::string tok;
  while (is >> tok) out.push_back(tok);
  return out;
}

bcx_status compile(const std::string &source, const char *name, const char *options, const std::string &arch,
                   std::vector<char> *cubin, std::string *log) {
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "bcx_jit.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) {
    *log = nvrtcGetErrorString(r);
    return BCX_BUILD_PROGRAM_FAILURE;
  }
  std::vector<std::string> opts = {"--gpu-architecture=" + arch, "-std=c++17", "-default-device"};
  for (auto &o : split_options(options)) opts.push_back(o);
  std::vector<const char *> copts;
  for (auto &o : opts) copts.push_back(o.c_str());
  nvrtcAddNameExpression(prog, name);
  r = nvrtcCompileProgram(prog, int(copts.size()), copts.data());
  size_t log_size = 0;
  nvrtcGetProgramLogSize(prog, &log_size);
  log->assign(log_size, '\0');
  if (log_size) nvrtcGetProgramLog(prog, &(*log)[0]);
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return BCX_BUILD_PROGRAM_FAILURE;
  }
  size_t size = 0;
  nvrtcGetCUBINSize(prog, &size);
  cubin->resize(size);
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  return BCX_SUCCESS;
}

}  // namespace
}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_jit_get_kernel(const char *source, const char *kernel_name, const char *options,
                              bcx_jit_kernel *kernel) {
  clear_error();
  BCX_CHECK(source && kernel_name && kernel, BCX_INVALID_VALUE, "NULL argument");
  std::string arch;
  bcx_status rc = device_arch(&arch);
  if (rc) return rc;
  const std::string key = std::string(source) + "\n//name=" + kernel_name + "\n//options=" +
                          (options ? options : "") + "\n//arch=" + arch;
  const std::string hex = hex_key(key);
  JitCache &c = cache();
  {
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.index.find(hex);
    if (it != c.index.end() && it->second->key == key) {
      c.lru.splice(c.lru.begin(), c.lru, it->second);
      ++c.hits;
      *kernel = reinterpret_cast<bcx_jit_kernel>(c.lru.front().kernel);
      return BCX_SUCCESS;
    }
    ++c.misses;
  }
  std::vector<char> cubin;
  const std::string path = disk_path(hex);
  bool from_disk = disk_load(path, key, &cubin);
  if (!from_disk) {
    std::string log;
    rc = compile(source, kernel_name, options, arch, &cubin, &log);
    {
      std::lock_guard<std::mutex> lk(c.mu);
      c.last_log = log;
      ++c.compiles;
    }
    if (rc) {
      set_error("NVRTC failed to build kernel %s: %s", kernel_name, log.c_str());
      return rc;
    }
    disk_store(path, key, cubin);
  }
  JitEntry e;
  e.key = key;
  cudaError_t err = cudaLibraryLoadData(&e.library, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (err != cudaSuccess) return cuda_status(err, "cudaLibraryLoadData");
  err = cudaLibraryGetKernel(&e.kernel, e.library, kernel_name);
  if (err != cudaSuccess) {
    cudaLibraryUnload(e.library);
    set_error("kernel %s not found in the generated module", kernel_name);
    return BCX_INVALID_KERNEL_NAME;
  }
  std::lock_guard<std::mutex> lk(c.mu);
  if (from_disk) ++c.disk_hits;
  auto it = c.index.find(hex);
  if (it != c.index.end()) {  // another thread built it meanwhile, or a collision: replace
    cudaLibraryUnload(it->second->library);
    c.lru.erase(it->second);
    c.index.erase(it);
  }
  c.lru.push_front(e);
  c.index[hex] = c.lru.begin();
  *kernel = reinterpret_cast<bcx_jit_kernel>(e.kernel);
  while (c.lru.size() > c.capacity) {
    JitEntry &old = c.lru.back();
    // Evicting unloads the module; kernels already enqueued keep running
    // (the driver defers the unload), but an evicted handle must not be
    // launched again -- callers fetch handles right before each launch.
    c.index.erase(hex_key(old.key));
    cudaLibraryUnload(old.library);
    c.lru.pop_back();
  }
  return BCX_SUCCESS;
}

bcx_status bcx_jit_launch(bcx_jit_kernel kernel, unsigned grid, unsigned block, size_t shared_bytes,
                          bcx_stream stream, void **args) {
  BCX_CHECK(kernel != nullptr, BCX_INVALID_VALUE, "NULL kernel");
  KernelScope ks("jit", (cudaStream_t)stream);
  cudaError_t e = cudaSuccess;
  // Dynamic shared memory above the default 48 KB needs the kernel's opt-in
  // on the current device (cheap, and idempotent).
  if (shared_bytes > 48 * 1024)
    e = cudaFuncSetAttribute(reinterpret_cast<const void *>(kernel), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(shared_bytes));
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(jit shared memory)");
  e = cudaLaunchKernel(reinterpret_cast<const void *>(kernel), dim3(grid), dim3(block), args, shared_bytes,
                       (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "cudaLaunchKernel(jit)");
  return BCX_SUCCESS;
}

bcx_status bcx_jit_build_log(char *buf, size_t len, size_t *needed) {
  JitCache &c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  if (needed) *needed = c.last_log.size() + 1;
  if (buf && len) {
    strncpy(buf, c.last_log.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return BCX_SUCCESS;
}

bcx_status bcx_jit_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *compiles, uint64_t *disk_hits,
                               uint64_t *entries) {
  JitCache &c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  if (hits) *hits = c.hits;
  if (misses) *misses = c.misses;
  if (compiles) *compiles = c.compiles;
  if (disk_hits) *disk_hits = c.disk_hits;
  if (entries) *entries = c.lru.size();
  return BCX_SUCCESS;
}

bcx_status bcx_jit_cache_configure(size_t capacity, int clear) {
  JitCache &c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  if (capacity) c.capacity = capacity;
  if (clear) {
    for (auto &e : c.lru) cudaLibraryUnload(e.library);
    c.lru.clear();
    c.index.clear();
  }
  return BCX_SUCCESS;
}

bcx_status bcx_device_sm_count(int *sm_count) {
  BCX_CHECK(sm_count != nullptr, BCX_INVALID_VALUE, "NULL argument");
  DeviceState *st = nullptr;
  bcx_status rc = current_device_state(&st);
  if (rc) return rc;
  *sm_count = st->sm_count;
  return BCX_SUCCESS;
}

}  // extern "C"
