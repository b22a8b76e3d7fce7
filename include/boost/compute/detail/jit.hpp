// boost/compute/detail/jit.hpp -- generated kernels for user functors.
//
// The reference turns every iterator expression and user function into
// OpenCL C text through meta_kernel (detail/meta_kernel.hpp:270-401) and
// builds it once per context (utility/program_cache.hpp).  This layer emits
// CUDA C++ instead and hands it to bcx_jit_get_kernel (NVRTC + LRU/disk cache
// inside libbcx).  Three kernel shapes cover the algorithms:
//   transform: out[i] = EXPR(_1 = a[i], _2 = b[i])   (16-byte vector path)
//   reduce:    per-block folds of OP, then one block folds the partials
//   scan:      tile totals, one block scans them, tiles rescanned with carry
// OP and EXPR are the user's source; they must be associative where the
// reference requires it (reduce.hpp:263-281 documents the same).
#ifndef BOOST_COMPUTE_DETAIL_JIT_HPP
#define BOOST_COMPUTE_DETAIL_JIT_HPP

#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include <bcx.h>
#include <boost/compute/command_queue.hpp>
#include <boost/compute/exception.hpp>
#include <boost/compute/types.hpp>

namespace boost {
namespace compute {
namespace detail {

// OpenCL-C spellings used by BOOST_COMPUTE_FUNCTION bodies, made valid CUDA.
inline const char *jit_prelude() {
  return "typedef unsigned int uint; typedef unsigned long long ulong;\n"
         "typedef unsigned char uchar; typedef unsigned short ushort;\n"
         "typedef signed char char_; typedef unsigned char uchar_; typedef short short_;\n"
         "typedef unsigned short ushort_; typedef int int_; typedef unsigned int uint_;\n"
         "typedef long long long_; typedef unsigned long long ulong_; typedef float float_;\n"
         "typedef double double_; typedef int2 int2_; typedef int4 int4_; typedef uint2 uint2_;\n"
         "typedef float2 float2_; typedef float4 float4_;\n"
         "template <class T> __device__ __forceinline__ T clamp(T x, T lo, T hi)"
         " { return x < lo ? lo : (x > hi ? hi : x); }\n"
         "template <class T> __device__ __forceinline__ T mad(T a, T b, T c) { return a * b + c; }\n"
         "template <class T> __device__ __forceinline__ T pown(T x, int n) {\n"
         "  T r = T(1); bool neg = n < 0; unsigned m = neg ? unsigned(-n) : unsigned(n);\n"
         "  while (m) { if (m & 1u) r *= x; x *= x; m >>= 1; } return neg ? T(1) / r : r; }\n"
         "__device__ __forceinline__ int popcount(unsigned x) { return __popc(x); }\n";
}

// Exact source literal of a host value.
inline std::string literal(float v) {
  unsigned u;
  std::memcpy(&u, &v, 4);
  char b[48];
  std::snprintf(b, sizeof(b), "__int_as_float(0x%08xu)", u);
  return b;
}
inline std::string literal(double v) {
  unsigned long long u;
  std::memcpy(&u, &v, 8);
  char b[64];
  std::snprintf(b, sizeof(b), "__longlong_as_double(0x%016llxull)", u);
  return b;
}
inline std::string literal(int v) { return "(" + std::to_string(v) + ")"; }
inline std::string literal(unsigned v) { return std::to_string(v) + "u"; }
inline std::string literal(long long v) { return "(" + std::to_string(v) + "ll)"; }
inline std::string literal(unsigned long long v) { return std::to_string(v) + "ull"; }
inline std::string literal(long v) { return literal((long long)v); }
inline std::string literal(unsigned long v) { return literal((unsigned long long)v); }
inline std::string literal(short v) { return "short(" + std::to_string(v) + ")"; }
inline std::string literal(char v) { return "char(" + std::to_string(int(v)) + ")"; }
inline std::string literal(signed char v) { return "(signed char)(" + std::to_string(int(v)) + ")"; }
inline std::string literal(unsigned char v) { return "(unsigned char)(" + std::to_string(unsigned(v)) + ")"; }
inline std::string literal(unsigned short v) { return "(unsigned short)(" + std::to_string(unsigned(v)) + ")"; }
inline std::string literal(bool v) { return v ? "true" : "false"; }

inline int sm_count() {
  int n = 0;
  check(bcx_device_sm_count(&n));
  return n;
}

// Compile (or fetch from the program cache) and launch.
inline void jit_launch(const std::string &source, const char *name, unsigned grid, unsigned block,
                       command_queue &queue, void **args) {
  bcx_jit_kernel k = nullptr;
  int rc = bcx_jit_get_kernel(source.c_str(), name, "", &k);
  if (rc == BCX_BUILD_PROGRAM_FAILURE) {
    size_t need = 0;
    bcx_jit_build_log(nullptr, 0, &need);
    std::string log(need, '\0');
    if (need) bcx_jit_build_log(&log[0], need, nullptr);
    throw program_build_failure(rc, log);
  }
  check(rc);
  check(bcx_jit_launch(k, grid, block, 0, queue.get(), args));
}

inline unsigned grid_for(size_t work, unsigned block) {
  size_t g = (work + block - 1) / block;
  size_t cap = size_t(sm_count()) * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return unsigned(g);
}

// out[i] = EXPR, with _1 = a[i] and (binary) _2 = b[i].
inline void jit_transform(const std::string &defs, const std::string &expr, const char *t0, const char *t1,
                          const char *tout, size_t s0, size_t s1, size_t sout, const void *a, const void *b,
                          void *out, size_t n, command_queue &queue) {
  if (n == 0) return;
  const bool binary = b != nullptr;
  std::ostringstream src;
  src << jit_prelude() << defs << "\n"
      << "extern \"C\" __global__ void bcx_jit_transform(const " << t0 << " *__restrict__ a, const "
      << (binary ? t1 : t0) << " *__restrict__ b, " << tout
      << " *__restrict__ r, unsigned long long n, unsigned long long nvec) {\n"
      << "  const unsigned long long s = (unsigned long long)gridDim.x * blockDim.x;\n"
      << "  unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;\n";
  const bool same = s0 == sout && (!binary || s1 == sout) && 16 % sout == 0;
  if (same) {
    const size_t N = 16 / sout;
    src << "  struct alignas(16) VA { " << t0 << " v[" << N << "]; };\n"
        << "  struct alignas(16) VB { " << (binary ? t1 : t0) << " v[" << N << "]; };\n"
        << "  struct alignas(16) VR { " << tout << " v[" << N << "]; };\n"
        << "  for (unsigned long long j = i; j < nvec; j += s) {\n"
        << "    const VA x = reinterpret_cast<const VA *>(a)[j];\n"
        << (binary ? "    const VB y = reinterpret_cast<const VB *>(b)[j];\n" : "")
        << "    VR z;\n"
        << "#pragma unroll\n    for (int k = 0; k < " << N << "; ++k) {\n"
        << "      const auto _1 = x.v[k];\n"
        << (binary ? "      const auto _2 = y.v[k];\n" : "")
        << "      z.v[k] = (" << tout << ")(" << expr << ");\n    }\n"
        << "    reinterpret_cast<VR *>(r)[j] = z;\n  }\n"
        << "  i += nvec * " << N << ";\n";
  }
  src << "  for (; i < n; i += s) {\n"
      << "    const auto _1 = a[i];\n"
      << (binary ? "    const auto _2 = b[i];\n" : "")
      << "    r[i] = (" << tout << ")(" << expr << ");\n  }\n}\n";
  unsigned long long nn = n, nvec = 0;
  if (same) {
    const size_t N = 16 / sout;
    bool aligned = reinterpret_cast<uintptr_t>(a) % 16 == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0 &&
                   (!binary || reinterpret_cast<uintptr_t>(b) % 16 == 0);
    nvec = aligned ? n / N : 0;
  }
  const void *bb = binary ? b : a;
  void *args[] = {(void *)&a, (void *)&bb, (void *)&out, (void *)&nn, (void *)&nvec};
  jit_launch(src.str(), "bcx_jit_transform", grid_for(n / 4 + 1, 256), 256, queue, args);
}

// result = init OP fold(load(i)) (has_init) or fold(load(i)); one value of
// type T at `out` (device).  OP is an expression of (_1, _2); LOAD the body of
// the element read, a function of a[i] (and b[i]) -- "return a[i];" for a
// plain reduce, the transform function applied to a[i] (and b[i]) for a fused
// transform_reduce, so the transformed values are never written out.
inline void jit_fold(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                     const std::string &load, const char *ta, const char *tb, const void *a, const void *b,
                     size_t n, const void *init, void *out, command_queue &queue) {
  std::ostringstream src;
  src << jit_prelude() << defs << "\n"
      << "typedef " << t << " T;\n"
      << "typedef " << ta << " TA;\n"
      << "typedef " << (tb ? tb : ta) << " TB;\n"
      << "__device__ __forceinline__ T bcx_op(const T &_1, const T &_2) { return (T)(" << op << "); }\n"
      << "__device__ __forceinline__ T bcx_load(const TA *__restrict__ a, const TB *__restrict__ b,"
      << " unsigned long long i) { " << load << " }\n"
      << "struct Acc { T v; int has; };\n"
      << "__device__ __forceinline__ Acc comb(Acc a, Acc b) {\n"
      << "  if (!a.has) return b; if (!b.has) return a; Acc r; r.v = bcx_op(a.v, b.v); r.has = 1; return r; }\n"
      << "__device__ Acc block_fold(Acc a) {\n"
      << "  __shared__ T sv[256]; __shared__ int sh[256];\n"
      << "  sv[threadIdx.x] = a.v; sh[threadIdx.x] = a.has; __syncthreads();\n"
      << "  for (unsigned w = 1; w < blockDim.x; w <<= 1) {\n"
      << "    if ((threadIdx.x & (2 * w - 1)) == 0 && threadIdx.x + w < blockDim.x) {\n"
      << "      Acc x{sv[threadIdx.x], sh[threadIdx.x]}, y{sv[threadIdx.x + w], sh[threadIdx.x + w]};\n"
      << "      Acc z = comb(x, y); sv[threadIdx.x] = z.v; sh[threadIdx.x] = z.has; }\n"
      << "    __syncthreads(); }\n"
      << "  Acc r{sv[0], sh[0]}; return r; }\n"
      << "extern \"C\" __global__ void bcx_jit_reduce_partials(const TA *__restrict__ a, const TB *__restrict__ b,"
      << " unsigned long long n, T *__restrict__ pv, int *__restrict__ ph) {\n"
      << "  const unsigned long long per = (n + gridDim.x - 1) / gridDim.x;\n"
      << "  const unsigned long long b0 = blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;\n"
      << "  Acc acc; acc.has = 0; acc.v = T();\n"
      << "  const unsigned long long chunk = (b1 > b0 ? b1 - b0 : 0) / blockDim.x + 1;\n"
      << "  const unsigned long long t0 = b0 + threadIdx.x * chunk;\n"
      << "  for (unsigned long long i = t0; i < t0 + chunk && i < b1; ++i) {"
      << " Acc x; x.v = bcx_load(a, b, i); x.has = 1; acc = comb(acc, x); }\n"
      << "  acc = block_fold(acc);\n"
      << "  if (threadIdx.x == 0) { pv[blockIdx.x] = acc.v; ph[blockIdx.x] = acc.has; } }\n"
      << "extern \"C\" __global__ void bcx_jit_reduce_final(const T *__restrict__ pv, const int *__restrict__ ph,"
      << " int count, const T *__restrict__ init, T *__restrict__ out) {\n"
      << "  if (threadIdx.x != 0) return;\n"
      << "  Acc acc; acc.has = init != 0; acc.v = init ? *init : T();\n"
      << "  for (int i = 0; i < count; ++i) { Acc x{pv[i], ph[i]}; acc = comb(acc, x); }\n"
      << "  if (acc.has) *out = acc.v; }\n";
  const std::string s = src.str();
  // Each thread folds a contiguous run in index order and the block folds
  // threads in order, so non-commutative (but associative) functors work.
  const unsigned blocks = n < 4096 ? 1u : unsigned(std::min<size_t>(size_t(sm_count()) * 4, (n + 4095) / 4096));
  void *partials = nullptr, *flags = nullptr, *dinit = nullptr;
  check(bcx_malloc(&partials, blocks * 16 + 16));
  check(bcx_malloc(&flags, blocks * sizeof(int)));
  if (init) {
    check(bcx_malloc(&dinit, 16));
    check(bcx_memcpy_async(dinit, init, tsize, queue.get()));
  }
  unsigned long long nn = n;
  const void *bb = b ? b : a;
  void *a1[] = {(void *)&a, (void *)&bb, (void *)&nn, (void *)&partials, (void *)&flags};
  jit_launch(s, "bcx_jit_reduce_partials", blocks, 256, queue, a1);
  int count = int(blocks);
  void *a2[] = {(void *)&partials, (void *)&flags, (void *)&count, (void *)&dinit, (void *)&out};
  jit_launch(s, "bcx_jit_reduce_final", 1, 32, queue, a2);
  queue.finish();
  bcx_free(partials);
  bcx_free(flags);
  if (dinit) bcx_free(dinit);
}

inline void jit_reduce(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                       const void *in, size_t n, const void *init, void *out, command_queue &queue) {
  jit_fold(defs, op, t, tsize, "return a[i];", t, nullptr, in, nullptr, n, init, out, queue);
}

// Scan with a user functor: tile totals -> one block scans them -> tiles
// rescanned from their carry.  Exclusive scans start from init.
inline void jit_scan(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                     const void *in, void *out, size_t n, bool exclusive, const void *init,
                     command_queue &queue) {
  if (n == 0) return;
  const unsigned kTile = 1024;
  std::ostringstream src;
  src << jit_prelude() << defs << "\n"
      << "typedef " << t << " T;\n"
      << "__device__ __forceinline__ T bcx_op(const T &_1, const T &_2) { return (T)(" << op << "); }\n"
      << "extern \"C\" __global__ void bcx_jit_scan_tiles(const T *__restrict__ in, unsigned long long n, T *__restrict__ sums) {\n"
      << "  const unsigned long long b0 = (unsigned long long)blockIdx.x * " << kTile << ";\n"
      << "  if (threadIdx.x == 0) { T acc = in[b0]; for (unsigned long long i = b0 + 1; i < b0 + " << kTile
      << " && i < n; ++i) acc = bcx_op(acc, in[i]); sums[blockIdx.x] = acc; } }\n"
      << "extern \"C\" __global__ void bcx_jit_scan_sums(T *__restrict__ sums, unsigned tiles, const T *__restrict__ init, int has_init) {\n"
      << "  if (threadIdx.x != 0) return;\n"
      << "  T run = has_init ? *init : sums[0]; int started = has_init;\n"
      << "  for (unsigned i = 0; i < tiles; ++i) { T s = sums[i];\n"
      << "    if (!started) { sums[i] = T(); run = s; started = 1; continue; }\n"
      << "    sums[i] = run; run = bcx_op(run, s); } }\n"
      << "extern \"C\" __global__ void bcx_jit_scan_apply(const T *__restrict__ in, T *__restrict__ out, unsigned long long n,"
      << " const T *__restrict__ sums, int exclusive, int has_carry) {\n"
      << "  __shared__ T buf[" << kTile << "];\n"
      << "  const unsigned long long b0 = (unsigned long long)blockIdx.x * " << kTile << ";\n"
      << "  const unsigned cnt = (unsigned)((n - b0) < " << kTile << " ? (n - b0) : " << kTile << ");\n"
      << "  for (unsigned i = threadIdx.x; i < cnt; i += blockDim.x) buf[i] = in[b0 + i];\n"
      << "  __syncthreads();\n"
      << "  if (threadIdx.x == 0) {\n"
      << "    const bool carry = has_carry || blockIdx.x > 0;\n"
      << "    T run = carry ? sums[blockIdx.x] : T();\n"
      << "    for (unsigned i = 0; i < cnt; ++i) { T x = buf[i];\n"
      << "      if (exclusive) { buf[i] = run; run = (carry || i > 0) ? bcx_op(run, x) : x; }\n"
      << "      else { run = (carry || i > 0) ? bcx_op(run, x) : x; buf[i] = run; } } }\n"
      << "  __syncthreads();\n"
      << "  for (unsigned i = threadIdx.x; i < cnt; i += blockDim.x) out[b0 + i] = buf[i]; }\n";
  const std::string s = src.str();
  const unsigned tiles = unsigned((n + kTile - 1) / kTile);
  void *sums = nullptr, *dinit = nullptr, *tmp = nullptr;
  check(bcx_malloc(&sums, size_t(tiles) * tsize + 16));
  if (exclusive && init) {
    check(bcx_malloc(&dinit, 16));
    check(bcx_memcpy_async(dinit, init, tsize, queue.get()));
  }
  const void *src_in = in;
  if (in == out) {  // in place: scan from a copy
    check(bcx_malloc(&tmp, n * tsize));
    check(bcx_memcpy_async(tmp, in, n * tsize, queue.get()));
    src_in = tmp;
  }
  unsigned long long nn = n;
  void *a1[] = {(void *)&src_in, (void *)&nn, (void *)&sums};
  jit_launch(s, "bcx_jit_scan_tiles", tiles, 32, queue, a1);
  int has_init = dinit != nullptr;
  void *a2[] = {(void *)&sums, (void *)&tiles, (void *)&dinit, (void *)&has_init};
  jit_launch(s, "bcx_jit_scan_sums", 1, 32, queue, a2);
  int ex = exclusive ? 1 : 0;
  void *a3[] = {(void *)&src_in, (void *)&out, (void *)&nn, (void *)&sums, (void *)&ex, (void *)&has_init};
  jit_launch(s, "bcx_jit_scan_apply", tiles, 128, queue, a3);
  queue.finish();
  bcx_free(sums);
  if (dinit) bcx_free(dinit);
  if (tmp) bcx_free(tmp);
}

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
