// oracle.cpp -- CPU restatement of the reference's algorithms for the hot path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker: only the test suite,
// the package smoke check and the benchmark's CPU-baseline leg load it.  The
// product path (libbcx.so) never links, loads or calls it.
//
// Parity is pinned: every function here is checked against the golden vectors
// of the reference's own test suite (tests/golden/reference_vectors.json,
// extracted from test/test_*.cpp by tests/golden/extract_reference_vectors.py).
//
// Contents
//   * GPU-path semantics (what the reference computes on a GPU device, which is
//     what libbcx reproduces):
//       radix key transform        algorithm/detail/radix_sort.hpp:100-127
//       stable LSD radix order     algorithm/detail/radix_sort.hpp:186-250,347
//       serial insertion sort      algorithm/detail/insertion_sort.hpp:26-159
//       sort / sort_by_key dispatch algorithm/sort.hpp:34-80,
//                                  algorithm/sort_by_key.hpp:33-83
//       scan (left fold, init)     algorithm/exclusive_scan.hpp:89-104,
//                                  algorithm/detail/scan_on_gpu.hpp:59-66
//       reduce / accumulate        algorithm/reduce.hpp:205-305,
//                                  algorithm/accumulate.hpp:102-188,
//                                  algorithm/detail/serial_accumulate.hpp:33-49
//       transform / saxpy          algorithm/transform.hpp:38-82, perf/perf_saxpy.cpp:50-56
//       reduce_by_key              algorithm/detail/reduce_by_key_with_scan.hpp:432-486
//   * FP64 reference sums (Neumaier in double) to measure float error.
//   * CPU-device algorithms (what the reference runs on an OpenCL CPU device
//     such as pocl), threaded over host cores for the timed CPU baseline:
//       merge_sort_on_cpu          algorithm/detail/merge_sort_on_cpu.hpp:27-366
//       scan_on_cpu                algorithm/detail/scan_on_cpu.hpp:70-195
//       reduce_on_cpu              algorithm/detail/reduce_on_cpu.hpp
//       copy_on_device_cpu         algorithm/detail/copy_on_device.hpp:32-57
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

enum Dtype { CHAR = 0, UCHAR, SHORT, USHORT, INT, UINT, LONG, ULONG, FLOAT, DOUBLE };
enum Op { PLUS = 0, MULTIPLIES, MIN, MAX, BIT_AND, BIT_OR, BIT_XOR, MINUS, DIVIDES, MODULUS };

size_t dsize(int t) {
  static const size_t s[] = {1, 1, 2, 2, 4, 4, 8, 8, 4, 8};
  return s[t];
}
bool is_float(int t) { return t == FLOAT || t == DOUBLE; }
bool is_signed(int t) { return t == CHAR || t == SHORT || t == INT || t == LONG || is_float(t); }

// radix() of algorithm/detail/radix_sort.hpp:100-127 on the unsigned bit
// pattern of width `bits`; returns the transformed key.
uint64_t radix_key(uint64_t x, int bits, bool flt, bool sgn, bool desc) {
  const uint64_t mask_all = bits == 64 ? ~0ull : ((1ull << bits) - 1);
  const uint64_t sign = 1ull << (bits - 1);
  x &= mask_all;
  const uint64_t negx = (0 - x) & mask_all;
  if (flt) {
    const uint64_t m = ((0 - (x >> (bits - 1))) | sign) & mask_all;
    return ((desc ? negx : x) ^ m) & mask_all;
  }
  if (sgn) return ((desc ? negx : x) ^ sign) & mask_all;
  return desc ? (mask_all - x) : x;
}

uint64_t load_bits(const void *p, size_t i, size_t w) {
  uint64_t v = 0;
  memcpy(&v, static_cast<const char *>(p) + i * w, w);
  return v;
}

template <class T> T at(const void *p, size_t i) {
  T v;
  memcpy(&v, static_cast<const char *>(p) + i * sizeof(T), sizeof(T));
  return v;
}

// Applies a permutation (out[i] = in[perm[i]]) to an array of w-byte items.
void permute(void *data, size_t w, const std::vector<size_t> &perm) {
  const size_t n = perm.size();
  std::vector<char> tmp(n * w);
  for (size_t i = 0; i < n; ++i) memcpy(&tmp[i * w], static_cast<char *>(data) + perm[i] * w, w);
  memcpy(data, tmp.data(), n * w);
}

template <class T> bool typed_less(const void *keys, size_t a, size_t b, bool desc) {
  const T x = at<T>(keys, a), y = at<T>(keys, b);
  return desc ? (x > y) : (x < y);
}

bool cmp_dispatch(int t, const void *keys, size_t a, size_t b, bool desc) {
  switch (t) {
    case CHAR: return typed_less<int8_t>(keys, a, b, desc);
    case UCHAR: return typed_less<uint8_t>(keys, a, b, desc);
    case SHORT: return typed_less<int16_t>(keys, a, b, desc);
    case USHORT: return typed_less<uint16_t>(keys, a, b, desc);
    case INT: return typed_less<int32_t>(keys, a, b, desc);
    case UINT: return typed_less<uint32_t>(keys, a, b, desc);
    case LONG: return typed_less<int64_t>(keys, a, b, desc);
    case ULONG: return typed_less<uint64_t>(keys, a, b, desc);
    case FLOAT: return typed_less<float>(keys, a, b, desc);
    case DOUBLE: return typed_less<double>(keys, a, b, desc);
  }
  return false;
}

// ---- integer arithmetic with wrap-around ----------------------------------
template <class T> struct UnsignedOf { typedef T type; };
template <> struct UnsignedOf<int8_t> { typedef uint8_t type; };
template <> struct UnsignedOf<int16_t> { typedef uint16_t type; };
template <> struct UnsignedOf<int32_t> { typedef uint32_t type; };
template <> struct UnsignedOf<int64_t> { typedef uint64_t type; };

template <class T> T apply(int op, T a, T b) {
  typedef typename UnsignedOf<T>::type U;
  if constexpr (std::is_floating_point<T>::value) {
    switch (op) {
      case PLUS: return a + b;
      case MULTIPLIES: return a * b;
      case MIN: return (b < a || a != a) ? b : a;
      case MAX: return (b > a || a != a) ? b : a;
      case MINUS: return a - b;
      case DIVIDES: return a / b;
    }
    return a;
  } else {
    switch (op) {
      case PLUS: return T(U(U(a) + U(b)));
      case MULTIPLIES: return T(U(uint64_t(U(a)) * uint64_t(U(b))));
      case MIN: return b < a ? b : a;
      case MAX: return b > a ? b : a;
      case BIT_AND: return T(a & b);
      case BIT_OR: return T(a | b);
      case BIT_XOR: return T(a ^ b);
      case MINUS: return T(U(U(a) - U(b)));
      case DIVIDES: return b == 0 ? T(0) : T(a / b);
      case MODULUS: return b == 0 ? T(0) : T(a % b);
    }
    return a;
  }
}

template <class T> T identity(int op) {
  switch (op) {
    case MULTIPLIES: return T(1);
    case MIN: return std::is_floating_point<T>::value ? T(INFINITY) : std::numeric_limits<T>::max();
    case MAX: return std::is_floating_point<T>::value ? T(-INFINITY) : std::numeric_limits<T>::lowest();
    case BIT_AND: return T(~uint64_t(0));
  }
  return T(0);
}

template <class T>
void scan_t(int op, int exclusive, const void *init, const void *in, void *out, size_t n) {
  T acc = exclusive ? (init ? at<T>(init, 0) : T(0)) : identity<T>(op);
  for (size_t i = 0; i < n; ++i) {
    const T x = at<T>(in, i);
    if (exclusive) {
      memcpy(static_cast<char *>(out) + i * sizeof(T), &acc, sizeof(T));
      acc = apply<T>(op, acc, x);
    } else {
      acc = (i == 0) ? x : apply<T>(op, acc, x);
      memcpy(static_cast<char *>(out) + i * sizeof(T), &acc, sizeof(T));
    }
  }
}

template <class T>
void fold_t(int op, const void *in, size_t n, const void *init, void *out) {
  T acc = init ? at<T>(init, 0) : (n ? at<T>(in, 0) : T(0));
  for (size_t i = init ? 0 : 1; i < n; ++i) acc = apply<T>(op, acc, at<T>(in, i));
  memcpy(out, &acc, sizeof(T));
}

#define DISPATCH(t, FN, ...)                              \
  switch (t) {                                            \
    case CHAR: FN<int8_t>(__VA_ARGS__); break;            \
    case UCHAR: FN<uint8_t>(__VA_ARGS__); break;          \
    case SHORT: FN<int16_t>(__VA_ARGS__); break;          \
    case USHORT: FN<uint16_t>(__VA_ARGS__); break;        \
    case INT: FN<int32_t>(__VA_ARGS__); break;            \
    case UINT: FN<uint32_t>(__VA_ARGS__); break;          \
    case LONG: FN<int64_t>(__VA_ARGS__); break;           \
    case ULONG: FN<uint64_t>(__VA_ARGS__); break;         \
    case FLOAT: FN<float>(__VA_ARGS__); break;            \
    case DOUBLE: FN<double>(__VA_ARGS__); break;          \
  }

template <class T> double as_double(const void *p, size_t i) { return double(at<T>(p, i)); }

double value_as_double(int t, const void *p, size_t i) {
  switch (t) {
    case CHAR: return as_double<int8_t>(p, i);
    case UCHAR: return as_double<uint8_t>(p, i);
    case SHORT: return as_double<int16_t>(p, i);
    case USHORT: return as_double<uint16_t>(p, i);
    case INT: return as_double<int32_t>(p, i);
    case UINT: return as_double<uint32_t>(p, i);
    case LONG: return as_double<int64_t>(p, i);
    case ULONG: return as_double<uint64_t>(p, i);
    case FLOAT: return as_double<float>(p, i);
    case DOUBLE: return as_double<double>(p, i);
  }
  return 0;
}

int threads_for(int threads) {
  if (threads > 0) return threads;
  unsigned h = std::thread::hardware_concurrency();
  return h ? int(h) : 1;
}

template <class F> void parallel_for(int threads, size_t n, F f) {
  threads = threads_for(threads);
  if (threads <= 1 || n < 2) {
    f(size_t(0), n, 0);
    return;
  }
  std::vector<std::thread> pool;
  const size_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const size_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back(f, b, e, t);
  }
  for (auto &th : pool) th.join();
}

}  // namespace

extern "C" {

// Transformed radix keys (as uint64) of n elements of dtype t.
void oracle_radix_keys(int t, int desc, const void *in, uint64_t *out, size_t n) {
  const size_t w = dsize(t);
  for (size_t i = 0; i < n; ++i)
    out[i] = radix_key(load_bits(in, i, w), int(w * 8), is_float(t), is_signed(t), desc != 0);
}

// detail::radix_sort / radix_sort_by_key: LSD with stable passes is a stable
// sort by the transformed key.  vb = value bytes (0 = keys only).
void oracle_radix_sort(int t, size_t vb, void *keys, void *vals, size_t n, int desc) {
  const size_t w = dsize(t);
  std::vector<uint64_t> k(n);
  oracle_radix_keys(t, desc, keys, k.data(), n);
  std::vector<size_t> perm(n);
  std::iota(perm.begin(), perm.end(), size_t(0));
  std::stable_sort(perm.begin(), perm.end(), [&](size_t a, size_t b) { return k[a] < k[b]; });
  permute(keys, w, perm);
  if (vb) permute(vals, vb, perm);
}

// detail::serial_insertion_sort(_by_key) with less<T> (desc = 0) or
// greater<T> (desc = 1) on typed keys.
void oracle_insertion_sort(int t, size_t vb, void *keys, void *vals, size_t n, int desc) {
  const size_t w = dsize(t);
  std::vector<char> kk(w), vv(vb ? vb : 1);
  char *K = static_cast<char *>(keys);
  char *V = static_cast<char *>(vals);
  for (size_t i = 1; i < n; ++i) {
    memcpy(kk.data(), K + i * w, w);
    if (vb) memcpy(vv.data(), V + i * vb, vb);
    size_t pos = i;
    while (pos > 0) {
      // compare(key, keys[pos-1]) on a two-element view
      char pair[16];
      memcpy(pair, kk.data(), w);
      memcpy(pair + w, K + (pos - 1) * w, w);
      if (!cmp_dispatch(t, pair, 0, 1, desc != 0)) break;
      memcpy(K + pos * w, K + (pos - 1) * w, w);
      if (vb) memcpy(V + pos * vb, V + (pos - 1) * vb, vb);
      --pos;
    }
    memcpy(K + pos * w, kk.data(), w);
    if (vb) memcpy(V + pos * vb, vv.data(), vb);
  }
}

// compute::sort dispatch on a GPU device (sort.hpp:34-80).
void oracle_sort(int t, void *keys, size_t n, int desc) {
  if (n < 2) return;
  if (n <= 32) oracle_insertion_sort(t, 0, keys, nullptr, n, desc);
  else oracle_radix_sort(t, 0, keys, nullptr, n, desc);
}

// compute::sort_by_key dispatch on a GPU device (sort_by_key.hpp:33-83).
void oracle_sort_by_key(int t, size_t vb, void *keys, void *vals, size_t n, int desc) {
  if (n < 32) oracle_insertion_sort(t, vb, keys, vals, n, desc);
  else oracle_radix_sort(t, vb, keys, vals, n, desc);
}

// exclusive_scan / inclusive_scan as the left fold std::partial_sum computes
// (the reference tests compare against it, test/test_scan.cpp:392-436).
void oracle_scan(int t, int op, int exclusive, const void *init, const void *in, void *out, size_t n) {
  DISPATCH(t, scan_t, op, exclusive, init, in, out, n);
}

// Left fold: accumulate(first, last, init, op) when init != NULL (the serial
// single-work-item loop of serial_accumulate.hpp:33-49, i.e. what the
// reference computes for float accumulate), reduce(first, last, op) when
// init == NULL.  Integer results are exact modulo 2^bits.
void oracle_fold(int t, int op, const void *in, size_t n, const void *init, void *out) {
  DISPATCH(t, fold_t, op, in, n, init, out);
}

// FP64 reference sum (Neumaier in double) of n values of dtype t, plus init.
double oracle_sum_f64(int t, const void *in, size_t n, double init) {
  double s = init, c = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double x = value_as_double(t, in, i);
    const double u = s + x;
    c += (std::fabs(s) >= std::fabs(x)) ? ((s - u) + x) : ((x - u) + s);
    s = u;
  }
  return s + c;
}

// FP64 reference inclusive (exclusive = 0) or exclusive prefix sums.
void oracle_prefix_f64(int t, int exclusive, const void *in, size_t n, double init, double *out) {
  double s = exclusive ? init : 0.0, c = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double x = value_as_double(t, in, i);
    if (exclusive) out[i] = s + c;
    const double u = s + x;
    c += (std::fabs(s) >= std::fabs(x)) ? ((s - u) + x) : ((x - u) + s);
    s = u;
    if (!exclusive) out[i] = s + c;
  }
}

// transform(x, y, r, alpha*_1 + _2): fused = 1 -> fma (one rounding),
// fused = 0 -> alpha*x rounded, then + y rounded.
void oracle_saxpy(int t, const void *alpha, const void *x, const void *y, void *out, size_t n, int fused) {
  if (t == FLOAT) {
    const float a = at<float>(alpha, 0);
    for (size_t i = 0; i < n; ++i) {
      const float xi = at<float>(x, i), yi = at<float>(y, i);
      float r;
      if (fused) r = std::fmaf(a, xi, yi);
      else {
        volatile float p = a * xi;
        r = p + yi;
      }
      memcpy(static_cast<char *>(out) + i * 4, &r, 4);
    }
  } else {
    const double a = at<double>(alpha, 0);
    for (size_t i = 0; i < n; ++i) {
      const double xi = at<double>(x, i), yi = at<double>(y, i);
      double r;
      if (fused) r = std::fma(a, xi, yi);
      else {
        volatile double p = a * xi;
        r = p + yi;
      }
      memcpy(static_cast<char *>(out) + i * 8, &r, 8);
    }
  }
}

// transform with a built-in binary functor.
void oracle_transform_binary(int t, int op, const void *a, const void *b, void *out, size_t n) {
  const size_t w = dsize(t);
  for (size_t i = 0; i < n; ++i) {
    char r[8];
    switch (t) {
#define CASE(D, T) case D: { T v = apply<T>(op, at<T>(a, i), at<T>(b, i)); memcpy(r, &v, sizeof(T)); } break;
      CASE(CHAR, int8_t) CASE(UCHAR, uint8_t) CASE(SHORT, int16_t) CASE(USHORT, uint16_t)
      CASE(INT, int32_t) CASE(UINT, uint32_t) CASE(LONG, int64_t) CASE(ULONG, uint64_t)
      CASE(FLOAT, float) CASE(DOUBLE, double)
#undef CASE
    }
    memcpy(static_cast<char *>(out) + i * w, r, w);
  }
}

// reduce_by_key with equal_to: one output per run of equal consecutive keys.
// Integer values fold exactly in their type; float values are summed in FP64
// and rounded once.  Returns the number of runs.
size_t oracle_reduce_by_key(int kt, int vt, int op, const void *keys, const void *vals, size_t n,
                            void *keys_out, void *vals_out) {
  const size_t kw = dsize(kt), vw = dsize(vt);
  size_t runs = 0;
  size_t i = 0;
  while (i < n) {
    size_t j = i + 1;
    while (j < n && memcmp(static_cast<const char *>(keys) + j * kw,
                           static_cast<const char *>(keys) + i * kw, kw) == 0)
      ++j;
    memcpy(static_cast<char *>(keys_out) + runs * kw, static_cast<const char *>(keys) + i * kw, kw);
    char r[8];
    if (is_float(vt) && op == PLUS) {
      double s = oracle_sum_f64(vt, static_cast<const char *>(vals) + i * vw, j - i, 0.0);
      if (vt == FLOAT) { float f = float(s); memcpy(r, &f, 4); }
      else memcpy(r, &s, 8);
    } else {
      oracle_fold(vt, op, static_cast<const char *>(vals) + i * vw, j - i, nullptr, r);
    }
    memcpy(static_cast<char *>(vals_out) + runs * vw, r, vw);
    ++runs;
    i = j;
  }
  return runs;
}

// ---- CPU-device algorithms, threaded (timed CPU baseline) -----------------

// merge_sort_on_cpu / merge_sort_by_key_on_cpu for uint32 keys with uint32
// values and less<uint>: insertion sort of 64-element blocks, then bottom-up
// stable pairwise merges (merge_sort_on_cpu.hpp:238-366).  Block sorts and
// merges are spread over `threads` host threads; when fewer merges than
// threads remain, each merge is split at merge-path diagonals
// (merge_with_merge_path.hpp) so all threads stay busy.
void oracle_cpu_merge_sort_by_key_u32(uint32_t *keys, uint32_t *vals, size_t n, int threads) {
  if (n < 2) return;
  threads = threads_for(threads);
  const size_t block = 64;
  const size_t nblocks = (n + block - 1) / block;
  parallel_for(threads, nblocks, [&](size_t b0, size_t b1, int) {
    for (size_t b = b0; b < b1; ++b) {
      const size_t s = b * block, e = std::min(n, s + block);
      for (size_t i = s + 1; i < e; ++i) {
        const uint32_t k = keys[i], v = vals[i];
        size_t pos = i;
        while (pos > s && k < keys[pos - 1]) {
          keys[pos] = keys[pos - 1];
          vals[pos] = vals[pos - 1];
          --pos;
        }
        keys[pos] = k;
        vals[pos] = v;
      }
    }
  });
  std::vector<uint32_t> tk(n), tv(n);
  uint32_t *sk = keys, *sv = vals, *dk = tk.data(), *dv = tv.data();
  for (size_t width = block; width < n; width *= 2) {
    const size_t pairs = (n + 2 * width - 1) / (2 * width);
    // split every merge into `parts` merge-path segments
    const size_t parts = std::max<size_t>(1, (size_t(threads) + pairs - 1) / pairs);
    parallel_for(threads, pairs * parts, [&](size_t j0, size_t j1, int) {
      for (size_t j = j0; j < j1; ++j) {
        const size_t pr = j / parts, part = j % parts;
        const size_t a0 = pr * 2 * width, a1 = std::min(n, a0 + width);
        const size_t b0 = a1, b1 = std::min(n, b0 + width);
        const size_t total = (a1 - a0) + (b1 - b0);
        const size_t d0 = total * part / parts, d1 = total * (part + 1) / parts;
        auto corank = [&](size_t d) {  // elements taken from A for the first d outputs
          size_t lo = d > (b1 - b0) ? d - (b1 - b0) : 0, hi = std::min(d, a1 - a0);
          while (lo < hi) {
            size_t i = (lo + hi) / 2;
            // stable: A[i] goes before B[d-i-1] unless B[d-i-1] < A[i]
            if (sk[b0 + (d - i - 1)] < sk[a0 + i]) hi = i;
            else lo = i + 1;
          }
          return lo;
        };
        size_t i = a0 + corank(d0), k = b0 + (d0 - (i - a0));
        const size_t iend = a0 + corank(d1), kend = b0 + (d1 - (iend - a0));
        size_t o = a0 + d0;
        while (i < iend && k < kend) {
          if (sk[k] < sk[i]) { dk[o] = sk[k]; dv[o] = sv[k]; ++k; }
          else { dk[o] = sk[i]; dv[o] = sv[i]; ++i; }
          ++o;
        }
        while (i < iend) { dk[o] = sk[i]; dv[o] = sv[i]; ++i; ++o; }
        while (k < kend) { dk[o] = sk[k]; dv[o] = sv[k]; ++k; ++o; }
      }
    });
    std::swap(sk, dk);
    std::swap(sv, dv);
  }
  if (sk != keys) {
    memcpy(keys, sk, n * 4);
    memcpy(vals, sv, n * 4);
  }
}

// scan_on_cpu for int32 plus: one chunk per thread, chunk sums, serial scan of
// the chunk sums, then each chunk scanned from its offset
// (scan_on_cpu.hpp:70-195).
void oracle_cpu_exclusive_scan_i32(const int32_t *in, int32_t *out, size_t n, int32_t init, int threads) {
  threads = threads_for(threads);
  std::vector<uint32_t> sums(threads + 1, 0);
  parallel_for(threads, n, [&](size_t b, size_t e, int t) {
    uint32_t s = 0;
    for (size_t i = b; i < e; ++i) s += uint32_t(in[i]);
    sums[t + 1] = s;
  });
  sums[0] = uint32_t(init);
  for (int t = 1; t <= threads; ++t) sums[t] += sums[t - 1];
  parallel_for(threads, n, [&](size_t b, size_t e, int t) {
    uint32_t s = sums[t];
    for (size_t i = b; i < e; ++i) {
      const uint32_t x = uint32_t(in[i]);
      out[i] = int32_t(s);
      s += x;
    }
  });
}

// reduce_on_cpu for int32 plus: per-thread partial sums, then a serial fold.
int32_t oracle_cpu_reduce_i32(const int32_t *in, size_t n, int threads) {
  threads = threads_for(threads);
  std::vector<uint32_t> sums(threads, 0);
  parallel_for(threads, n, [&](size_t b, size_t e, int t) {
    uint32_t s = 0;
    for (size_t i = b; i < e; ++i) s += uint32_t(in[i]);
    sums[t] = s;
  });
  uint32_t r = 0;
  for (uint32_t s : sums) r += s;
  return int32_t(r);
}

// copy_on_device_cpu for saxpy: one chunk per thread.
void oracle_cpu_saxpy_f32(float a, const float *x, const float *y, float *out, size_t n, int threads) {
  parallel_for(threads, n, [&](size_t b, size_t e, int) {
    for (size_t i = b; i < e; ++i) out[i] = std::fmaf(a, x[i], y[i]);
  });
}

int oracle_hardware_threads(void) { return threads_for(0); }

}  // extern "C"
