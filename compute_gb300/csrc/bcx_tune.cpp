// bcx_tune.cpp -- per-device table of tuning parameters and its disk file.
//
// Counterpart of the reference's detail::parameter_cache
// (detail/parameter_cache.hpp:38-110): (object, parameter) -> unsigned value,
// one table per device name, read from and written to a JSON file.  The
// reference keeps the file in ~/.boost_compute/tune/<device>.json; here the
// file is $BCX_CACHE_DIR/tune/<device>.json and is only touched when
// BCX_CACHE_DIR is set.  The kernels that have tunables (segmented sort small
// tile and grid, segmented scan tile, segmented and plain reduce grid) look
// their values up at dispatch time; the autotuner entry points
// (bcx_tune_segmented_*) fill the table by timing every candidate on the
// caller's workload.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "bcx.h"
#include "bcx_internal.h"

namespace bcx {
namespace {

struct Table {
  bool loaded = false;
  std::map<std::pair<std::string, std::string>, uint32_t> values;
};

std::mutex g_mu;
std::map<std::string, Table> g_tables;  // device name -> table

// Device name with spaces and parentheses replaced, as a file name; looked
// up once per device so that dispatch inside stream capture makes no
// property queries.
std::string canonical_device_name() {
  static std::mutex mu;
  static std::map<int, std::string> names;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return "unknown";
  std::lock_guard<std::mutex> lk(mu);
  auto it = names.find(dev);
  if (it != names.end()) return it->second;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string n(prop.name);
  while (!n.empty() && std::isspace(static_cast<unsigned char>(n.back()))) n.pop_back();
  for (char &c : n)
    if (c == ' ' || c == '(' || c == ')' || c == '/') c = '_';
  names[dev] = n;
  return n;
}

std::string table_path(const std::string &dev) {
  const char *dir = std::getenv("BCX_CACHE_DIR");
  if (!dir || !*dir) return std::string();
  return std::string(dir) + "/tune/" + dev + ".json";
}

// Reads {"object": {"parameter": value, ...}, ...}.  Anything unexpected ends
// the read; what was read so far is kept.
void read_table(const std::string &path, Table &t) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  size_t i = 0;
  auto skip = [&] {
    while (i < text.size() && (std::isspace(static_cast<unsigned char>(text[i])) || text[i] == ',' ||
                               text[i] == ':'))
      ++i;
  };
  auto str = [&](std::string &out) -> bool {
    skip();
    if (i >= text.size() || text[i] != '"') return false;
    size_t j = text.find('"', i + 1);
    if (j == std::string::npos) return false;
    out = text.substr(i + 1, j - i - 1);
    i = j + 1;
    return true;
  };
  skip();
  if (i >= text.size() || text[i] != '{') return;
  ++i;
  while (true) {
    std::string object;
    if (!str(object)) return;
    skip();
    if (i >= text.size() || text[i] != '{') return;
    ++i;
    while (true) {
      skip();
      if (i < text.size() && text[i] == '}') {
        ++i;
        break;
      }
      std::string param;
      if (!str(param)) return;
      skip();
      char *end = nullptr;
      const unsigned long v = std::strtoul(text.c_str() + i, &end, 10);
      if (end == text.c_str() + i) return;
      i = size_t(end - text.c_str());
      t.values[{object, param}] = uint32_t(v);
    }
  }
}

Table &table_locked(const std::string &dev) {
  Table &t = g_tables[dev];
  if (!t.loaded) {
    t.loaded = true;
    const std::string p = table_path(dev);
    if (!p.empty()) read_table(p, t);
  }
  return t;
}

}  // namespace

uint32_t param_get(const std::string &object, const char *parameter, uint32_t default_value) {
  const std::string dev = canonical_device_name();
  std::lock_guard<std::mutex> lk(g_mu);
  Table &t = table_locked(dev);
  auto it = t.values.find({object, parameter});
  return it == t.values.end() ? default_value : it->second;
}

void param_set(const std::string &object, const char *parameter, uint32_t value) {
  const std::string dev = canonical_device_name();
  std::lock_guard<std::mutex> lk(g_mu);
  table_locked(dev).values[{object, parameter}] = value;
}

bcx_status param_save() {
  const std::string dev = canonical_device_name();
  const std::string path = table_path(dev);
  if (path.empty()) return BCX_SUCCESS;
  std::lock_guard<std::mutex> lk(g_mu);
  Table &t = table_locked(dev);
  const char *dir = std::getenv("BCX_CACHE_DIR");
  ::mkdir(dir, 0755);
  ::mkdir((std::string(dir) + "/tune").c_str(), 0755);
  const std::string tmp = path + ".tmp";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  BCX_CHECK(f, BCX_OUT_OF_RESOURCES, "cannot write %s", tmp.c_str());
  std::fprintf(f, "{\n");
  std::string cur;
  bool first_obj = true, first_param = true;
  for (auto &kv : t.values) {
    if (kv.first.first != cur || first_obj) {
      if (!first_obj) std::fprintf(f, "},\n");
      std::fprintf(f, "  \"%s\": {", kv.first.first.c_str());
      cur = kv.first.first;
      first_obj = false;
      first_param = true;
    }
    std::fprintf(f, "%s\"%s\": %u", first_param ? "" : ", ", kv.first.second.c_str(), kv.second);
    first_param = false;
  }
  if (!first_obj) std::fprintf(f, "}\n");
  std::fprintf(f, "}\n");
  std::fclose(f);
  BCX_CHECK(std::rename(tmp.c_str(), path.c_str()) == 0, BCX_OUT_OF_RESOURCES, "cannot rename %s", tmp.c_str());
  return BCX_SUCCESS;
}

namespace {

// Scratch device memory of one tuning run, freed on every exit path.
struct Scratch {
  std::vector<void *> ptrs;
  ~Scratch() {
    for (void *p : ptrs) cudaFree(p);
  }
  bcx_status alloc(void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return BCX_SUCCESS;
    BCX_CUDA(cudaMalloc(p, bytes));
    ptrs.push_back(*p);
    return BCX_SUCCESS;
  }
};

struct Report {
  char *buf;
  size_t len, used = 0;
  void add(const char *fmt, ...) {
    if (!buf || len == 0 || used + 1 >= len) return;
    va_list ap;
    va_start(ap, fmt);
    const int w = std::vsnprintf(buf + used, len - used, fmt, ap);
    va_end(ap);
    if (w > 0) used = std::min(len - 1, used + size_t(w));
  }
};

// Median of `reps` timed runs of `run` (each preceded by the untimed `reset`).
template <class Reset, class Run>
bcx_status time_trial(cudaStream_t s, int reps, Reset &&reset, Run &&run, float *ms_out) {
  cudaEvent_t a = nullptr, b = nullptr;
  BCX_CUDA(cudaEventCreate(&a));
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return cuda_status(cudaErrorMemoryAllocation, "cudaEventCreate");
  }
  std::vector<float> t;
  bcx_status rc = BCX_SUCCESS;
  for (int r = 0; r <= reps && !rc; ++r) {  // run 0 warms up
    rc = reset();
    if (rc) break;
    cudaEventRecord(a, s);
    rc = run();
    cudaEventRecord(b, s);
    if (!rc && cudaEventSynchronize(b) != cudaSuccess) rc = cuda_status(cudaGetLastError(), "tuning run");
    float ms = 0.f;
    if (!rc && r > 0 && cudaEventElapsedTime(&ms, a, b) == cudaSuccess) t.push_back(ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  std::sort(t.begin(), t.end());
  *ms_out = t.empty() ? 0.f : t[t.size() / 2];
  return BCX_SUCCESS;
}

constexpr int kTuneReps = 3;

// Tries every value of `param` in `cands` (others fixed), keeps the fastest.
template <class Run>
bcx_status tune_param(cudaStream_t s, const std::string &obj, const char *param, const std::vector<uint32_t> &cands,
                      Report &rep, const std::function<bcx_status()> &reset, Run &&run) {
  uint32_t best = cands.front();
  float best_ms = -1.f;
  for (uint32_t c : cands) {
    param_set(obj, param, c);
    float ms = 0.f;
    bcx_status rc = time_trial(s, kTuneReps, reset, run, &ms);
    if (rc) return rc;
    rep.add("%s.%s=%u %.4f ms\n", obj.c_str(), param, c, ms);
    if (best_ms < 0.f || ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  param_set(obj, param, best);
  rep.add("%s.%s -> %u\n", obj.c_str(), param, best);
  return BCX_SUCCESS;
}

}  // namespace
}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_param_get(const char *object, const char *parameter, unsigned default_value, unsigned *value) {
  clear_error();
  BCX_CHECK(object && parameter && value, BCX_INVALID_VALUE, "NULL argument");
  *value = param_get(object, parameter, default_value);
  return BCX_SUCCESS;
}

bcx_status bcx_param_set(const char *object, const char *parameter, unsigned value) {
  clear_error();
  BCX_CHECK(object && parameter, BCX_INVALID_VALUE, "NULL argument");
  BCX_CHECK(std::strchr(object, '"') == nullptr && std::strchr(parameter, '"') == nullptr, BCX_INVALID_VALUE,
            "names may not contain quotes");
  param_set(object, parameter, value);
  return BCX_SUCCESS;
}

bcx_status bcx_param_save(void) {
  clear_error();
  return param_save();
}

bcx_status bcx_param_clear(void) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  g_tables.clear();  // the next lookup re-reads the file, if any
  return BCX_SUCCESS;
}

bcx_status bcx_tune_segmented_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes,
                                         const void *keys, const void *values, size_t n, const uint64_t *offsets,
                                         size_t nseg, char *report, size_t report_len) {
  clear_error();
  BCX_CHECK(dtype_valid(key_type), BCX_INVALID_VALUE, "invalid key type");
  BCX_CHECK(keys && offsets && nseg > 0 && n > 0, BCX_INVALID_VALUE, "NULL argument or empty workload");
  BCX_CHECK(value_bytes == 0 || values, BCX_INVALID_VALUE, "NULL values");
  cudaStream_t s = (cudaStream_t)stream;
  Report rep{report, report_len};
  if (report && report_len) report[0] = 0;
  const size_t kb = dtype_size(key_type);
  Scratch sc;
  void *k2 = nullptr, *v2 = nullptr, *tmp = nullptr;
  size_t tb = 0;
  bcx_status rc = bcx_segmented_sort_pairs(stream, key_type, value_bytes, const_cast<void *>(keys),
                                           const_cast<void *>(values), n, offsets, nseg, 0, nullptr, &tb);
  if (rc) return rc;
  if ((rc = sc.alloc(&k2, n * kb)) || (rc = sc.alloc(&v2, n * value_bytes)) || (rc = sc.alloc(&tmp, tb))) return rc;
  const std::function<bcx_status()> reset = [&]() -> bcx_status {
    BCX_CUDA(cudaMemcpyAsync(k2, keys, n * kb, cudaMemcpyDeviceToDevice, s));
    if (value_bytes) BCX_CUDA(cudaMemcpyAsync(v2, values, n * value_bytes, cudaMemcpyDeviceToDevice, s));
    return BCX_SUCCESS;
  };
  auto run = [&]() -> bcx_status {
    size_t t = tb;
    return bcx_segmented_sort_pairs(stream, key_type, value_bytes, k2, v2, n, offsets, nseg, 0, tmp, &t);
  };
  const std::string obj = "segmented_sort_k" + std::to_string(8 * kb) + "_v" + std::to_string(value_bytes);
  const uint32_t limit = segsort_small_tile_limit(kb, value_bytes);
  std::vector<uint32_t> tiles;
  for (uint32_t t : {1024u, 2048u, 4096u})
    if (t <= limit) tiles.push_back(t);
  param_set(obj, "small_blocks_per_sm", 0);
  if ((rc = tune_param(s, obj, "small_tile", tiles, rep, reset, run))) return rc;
  if ((rc = tune_param(s, obj, "small_blocks_per_sm", {0u, 1u, 2u, 4u, 8u}, rep, reset, run))) return rc;
  return param_save();
}

bcx_status bcx_tune_segmented_scan(bcx_stream stream, bcx_dtype type, const void *in, size_t n,
                                   const uint64_t *offsets, size_t nseg, char *report, size_t report_len) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype");
  BCX_CHECK(in && offsets && nseg > 0 && n > 0, BCX_INVALID_VALUE, "NULL argument or empty workload");
  cudaStream_t s = (cudaStream_t)stream;
  Report rep{report, report_len};
  if (report && report_len) report[0] = 0;
  const size_t es = dtype_size(type);
  const int comp = type == BCX_FLOAT ? 1 : 0;
  unsigned char zero[8] = {0};
  Scratch sc;
  void *out = nullptr, *tmp = nullptr;
  size_t tb = 0;
  bcx_status rc = bcx_segmented_scan(stream, type, BCX_PLUS, 1, zero, in, const_cast<void *>(in), n, offsets, nseg, comp, nullptr, &tb);
  if (rc) return rc;
  if ((rc = sc.alloc(&out, n * es)) || (rc = sc.alloc(&tmp, tb))) return rc;
  const std::function<bcx_status()> reset = [] { return BCX_SUCCESS; };
  auto run = [&]() -> bcx_status {
    size_t t = tb;
    return bcx_segmented_scan(stream, type, BCX_PLUS, 1, zero, in, out, n, offsets, nseg, comp, tmp, &t);
  };
  const std::string obj = std::string("segmented_scan_") + dtype_name(type);
  uint32_t small = 0, large = 0;
  segscan_shapes(es, &small, &large);
  const std::vector<uint32_t> items{small, large};
  if ((rc = tune_param(s, obj, "items_per_thread", items, rep, reset, run))) return rc;
  return param_save();
}

bcx_status bcx_tune_segmented_reduce(bcx_stream stream, bcx_dtype type, const void *in, const uint64_t *offsets,
                                     size_t nseg, char *report, size_t report_len) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype");
  BCX_CHECK(in && offsets && nseg > 0, BCX_INVALID_VALUE, "NULL argument or no segments");
  cudaStream_t s = (cudaStream_t)stream;
  Report rep{report, report_len};
  if (report && report_len) report[0] = 0;
  const size_t es = dtype_size(type);
  const int comp = type == BCX_FLOAT ? 1 : 0;
  unsigned char zero[8] = {0};
  Scratch sc;
  void *out = nullptr, *tmp = nullptr;
  size_t tb = 0;
  bcx_status rc = sc.alloc(&out, nseg * es);
  if (rc) return rc;
  rc = bcx_segmented_reduce(stream, type, BCX_PLUS, in, offsets, nseg, zero, out, comp, nullptr, &tb);
  if (rc) return rc;
  if ((rc = sc.alloc(&tmp, tb))) return rc;
  const std::function<bcx_status()> reset = [] { return BCX_SUCCESS; };
  auto run = [&]() -> bcx_status {
    size_t t = tb;
    return bcx_segmented_reduce(stream, type, BCX_PLUS, in, offsets, nseg, zero, out, comp, tmp, &t);
  };
  const std::string obj = std::string("segmented_reduce_") + dtype_name(type);
  if ((rc = tune_param(s, obj, "blocks_per_sm", {2u, 4u, 8u, 16u, 32u}, rep, reset, run))) return rc;
  return param_save();
}

}  // extern "C"
