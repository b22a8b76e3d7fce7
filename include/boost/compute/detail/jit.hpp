// boost/compute/detail/jit.hpp -- generated kernels for user functors.
//
// The reference turns every iterator expression and user function into
// OpenCL C text through meta_kernel (detail/meta_kernel.hpp:270-401) and
// builds it once per context (utility/program_cache.hpp).  This layer emits
// CUDA C++ instead and hands it to bcx_jit_get_kernel (NVRTC + LRU/disk cache
// inside libbcx).  Three kernel shapes cover the algorithms, each one launch,
// asynchronous on the caller's queue:
//   transform: out[i] = EXPR(_1 = a[i], _2 = b[i])   (16-byte vector path)
//   fold:      per-block in-order folds of OP, the last block folds the partials
//   scan:      single-pass decoupled look-back over ticketed tiles
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
         "__device__ __forceinline__ int popcount(unsigned x) { return __popc(x); }\n"
         // qualified spellings of the same types in user function signatures
         "namespace boost { namespace compute { typedef signed char char_; typedef unsigned char uchar_;\n"
         "typedef short short_; typedef unsigned short ushort_; typedef int int_; typedef unsigned int uint_;\n"
         "typedef long long long_; typedef unsigned long long ulong_; typedef float float_; typedef double double_;\n"
         "typedef ::int2 int2_; typedef ::int4 int4_; typedef ::uint2 uint2_; typedef ::float2 float2_;\n"
         "typedef ::float4 float4_; } }\nnamespace compute = ::boost::compute;\n"
         // element N of a tuple struct or component N of a vector type
         "template <int N, class T> __device__ __forceinline__ auto bcx_get(const T &t) {"
         " return t.template bcx_at<N>(); }\n"
         "#define BCX_VEC_GET(V, S) template <int N> __device__ __forceinline__ S bcx_get(const V &v) {"
         " return N == 0 ? v.x : (N == 1 ? v.y : (N == 2 ? v.z : v.w)); }\n"
         "#define BCX_VEC2_GET(V, S) template <int N> __device__ __forceinline__ S bcx_get(const V &v) {"
         " return N == 0 ? v.x : v.y; }\n"
         "BCX_VEC_GET(int4, int) BCX_VEC_GET(float4, float) BCX_VEC2_GET(int2, int) BCX_VEC2_GET(uint2, unsigned)\n"
         "BCX_VEC2_GET(float2, float)\n"
         "#define boost_tuple_get(x, n) bcx_get<n>(x)\n";
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
                       command_queue &queue, void **args, size_t shared_bytes = 0) {
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
  check(bcx_jit_launch(k, grid, block, shared_bytes, queue.get(), args));
}

inline unsigned grid_for(size_t work, unsigned block) {
  size_t g = (work + block - 1) / block;
  size_t cap = size_t(sm_count()) * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return unsigned(g);
}

// out[i] = EXPR, with _1 = a[i] and (binary) _2 = b[i].
inline std::string jit_transform_source(const std::string &defs, const std::string &expr, const char *t0,
                                        const char *t1, const char *tout, size_t s0, size_t s1, size_t sout,
                                        bool binary) {
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
  return src.str();
}

inline void jit_transform(const std::string &defs, const std::string &expr, const char *t0, const char *t1,
                          const char *tout, size_t s0, size_t s1, size_t sout, const void *a, const void *b,
                          void *out, size_t n, command_queue &queue) {
  if (n == 0) return;
  const bool binary = b != nullptr;
  const bool same = s0 == sout && (!binary || s1 == sout) && 16 % sout == 0;
  const std::string source = jit_transform_source(defs, expr, t0, t1, tout, s0, s1, sout, binary);
  unsigned long long nn = n, nvec = 0;
  if (same) {
    const size_t N = 16 / sout;
    bool aligned = reinterpret_cast<uintptr_t>(a) % 16 == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0 &&
                   (!binary || reinterpret_cast<uintptr_t>(b) % 16 == 0);
    nvec = aligned ? n / N : 0;
  }
  const void *bb = binary ? b : a;
  void *args[] = {(void *)&a, (void *)&bb, (void *)&out, (void *)&nn, (void *)&nvec};
  jit_launch(source, "bcx_jit_transform", grid_for(n / 4 + 1, 256), 256, queue, args);
}

// ---- shared pieces of the generated fold and scan kernels -----------------
// Both are written for any element type T the user's functor works on
// (built-in scalars, CUDA vector types, structs): values move between lanes
// as 32-bit words, partial results carry a "has a value" flag instead of an
// identity element (a user functor has none), and every combination keeps
// the input order, so a functor need only be associative, as the reference
// requires (reduce.hpp:263-281).
inline std::string jit_common(const std::string &defs, const std::string &op, const char *t) {
  std::ostringstream src;
  src << jit_prelude() << defs << "\n"
      << "typedef " << t << " T;\n"
      << "__device__ __forceinline__ T bcx_op(const T &_1, const T &_2) { return (T)(" << op << "); }\n"
      << R"BCX(
#define BCX_WORDS ((sizeof(T) + 3) / 4)
// Byte copy of a compile-time size (registers after unrolling).
template <unsigned long long BYTES>
__device__ __forceinline__ void bcx_copy(void *d, const void *s) {
#pragma unroll
  for (unsigned long long i = 0; i < BYTES; ++i)
    static_cast<unsigned char *>(d)[i] = static_cast<const unsigned char *>(s)[i];
}
__device__ __forceinline__ void bcx_to_words(const T &v, unsigned (&w)[BCX_WORDS]) {
#pragma unroll
  for (int k = 0; k < (int)BCX_WORDS; ++k) w[k] = 0u;
  bcx_copy<sizeof(T)>(w, &v);
}
__device__ __forceinline__ T bcx_from_words(const unsigned (&w)[BCX_WORDS]) {
  T r;
  bcx_copy<sizeof(T)>(&r, w);
  return r;
}
// Read of a value another block wrote, from L2 (never a stale L1 line).
__device__ __forceinline__ T bcx_ldcg(const T *p) {
  T r;
  if (sizeof(T) % 4 == 0) {
    unsigned w[BCX_WORDS];
#pragma unroll
    for (int k = 0; k < (int)BCX_WORDS; ++k) w[k] = __ldcg(reinterpret_cast<const unsigned *>(p) + k);
    bcx_copy<sizeof(T)>(&r, w);
  } else {
    unsigned char c[sizeof(T)];
#pragma unroll
    for (int k = 0; k < (int)sizeof(T); ++k) c[k] = __ldcg(reinterpret_cast<const unsigned char *>(p) + k);
    bcx_copy<sizeof(T)>(&r, c);
  }
  return r;
}
__device__ __forceinline__ T bcx_shfl_up(const T &v, unsigned d) {
  unsigned w[BCX_WORDS];
  bcx_to_words(v, w);
#pragma unroll
  for (int k = 0; k < (int)BCX_WORDS; ++k) w[k] = __shfl_up_sync(0xffffffffu, w[k], d);
  return bcx_from_words(w);
}
__device__ __forceinline__ T bcx_shfl_down(const T &v, unsigned d) {
  unsigned w[BCX_WORDS];
  bcx_to_words(v, w);
#pragma unroll
  for (int k = 0; k < (int)BCX_WORDS; ++k) w[k] = __shfl_down_sync(0xffffffffu, w[k], d);
  return bcx_from_words(w);
}
__device__ __forceinline__ T bcx_shfl_idx(const T &v, int src) {
  unsigned w[BCX_WORDS];
  bcx_to_words(v, w);
#pragma unroll
  for (int k = 0; k < (int)BCX_WORDS; ++k) w[k] = __shfl_sync(0xffffffffu, w[k], src);
  return bcx_from_words(w);
}
// (a, ha) followed by (b, hb) in input order.
__device__ __forceinline__ void bcx_comb(T &a, int &ha, const T &b, int hb) {
  if (hb) { a = ha ? bcx_op(a, b) : b; ha = 1; }
}
// In-order fold of one value per lane (lane order = input order, lanes with
// h == 0 hold nothing); the result is returned in every lane.
__device__ __forceinline__ T bcx_warp_fold(T v, int &h) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (unsigned d = 1; d < 32; d <<= 1) {
    const T o = bcx_shfl_down(v, d);
    const int oh = __shfl_down_sync(0xffffffffu, h, d);
    if ((lane & (2 * d - 1)) == 0 && lane + d < 32) bcx_comb(v, h, o, oh);
  }
  h = __shfl_sync(0xffffffffu, h, 0);
  return bcx_shfl_idx(v, 0);
}
)BCX";
  return src.str();
}

// Elements per thread of the generated scan: 128 bytes per thread, at most 32
// elements.  2^30 int32 on GB300 with the shared-memory transpose and the L2
// prefetch: 16 per thread 2.94 ms, 24 2.61 ms, 32 2.13 ms (4035 GB/s); the
// transpose took 32 per thread from 2.64 ms, the prefetch from 2.52 ms.
inline int jit_scan_items(size_t tsize) {
  const size_t k = 128 / (tsize ? tsize : 1);
  return int(k < 1 ? 1 : (k > 32 ? 32 : k));
}
// Tiles ahead whose input the generated scan asks L2 to prefetch (16 MB for
// 32 KB tiles).
inline int jit_scan_prefetch_tiles() { return 512; }
// 1: the generated scan reads its tile twice (the second time from L2) and
// keeps only per-thread totals across the look-back.
inline int jit_scan_two_read() { return 0; }
// 1: full aligned tiles move through shared memory (coalesced global access).
inline int jit_scan_transpose() { return 1; }
// Tile bytes of the staged generated scan (whole tiles moved into and out of
// shared memory by bulk copies), or 0 where it does not apply: the element
// size must divide 16 (the tile is handled as 16-byte vectors).  64 KB tiles
// hold three blocks per SM; 8- and 16-byte elements take 96 KB tiles (two per
// SM): fewer tiles, so fewer of their dearer fenced look-back steps.
inline int jit_scan_staged_tile_bytes(size_t tsize) {
  if (tsize == 0 || tsize > 16 || 16 % tsize != 0) return 0;
  return tsize >= 8 ? 96 * 1024 : 64 * 1024;
}
// Bytes ahead of a staged tile whose input is prefetched into L2.
inline size_t jit_scan_staged_prefetch_bytes() { return size_t(16) << 20; }

// Elements per thread of the generated fold: 64 bytes per thread, at most 16
// elements.
inline int jit_items(size_t tsize) {
  const size_t k = 64 / (tsize ? tsize : 1);
  return int(k < 1 ? 1 : (k > 16 ? 16 : k));
}

// result = init OP fold(load(i)) (init given) or fold(load(i)); one value of
// type T at `out` (device).  OP is an expression of (_1, _2); LOAD the body of
// the element read, a function of a[i] (and b[i]) -- "return a[i];" for a
// plain reduce, the transform function applied to a[i] (and b[i]) for a fused
// transform_reduce, so the transformed values are never written out.
//
// One launch, no block-wide barrier in the main loop: every warp folds its
// own contiguous range in order, 32 x ITEMS elements at a time (lane l folds
// its ITEMS consecutive elements -- 16-byte vector loads for a plain read of
// an aligned array -- then the warp folds its lanes in order); a block folds
// its eight warps in order and writes its partial, and the last block to
// finish (a ticket taken after a fence) folds the partials in block order with
// init.  Asynchronous on the queue: its temporaries are stream-ordered and
// nothing waits for the device.
inline bool jit_plain_load(const std::string &load) { return load == "return a[i];"; }

inline std::string jit_fold_source(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                                   const std::string &load, const char *ta, const char *tb) {
  const int items = jit_items(tsize);
  std::ostringstream src;
  src << jit_common(defs, op, t)
      << "typedef " << ta << " TA;\n"
      << "typedef " << (tb ? tb : ta) << " TB;\n"
      << "#define BCX_ITEMS " << items << "\n"
      << "#define BCX_PLAIN_LOAD " << (jit_plain_load(load) ? 1 : 0) << "\n"
      << "__device__ __forceinline__ T bcx_load(const TA *__restrict__ a, const TB *__restrict__ b,"
      << " unsigned long long i) { " << load << " }\n"
      << R"BCX(
constexpr unsigned long long BCX_CHUNK = 32ull * BCX_ITEMS;
constexpr bool BCX_VEC_OK = BCX_PLAIN_LOAD && (BCX_ITEMS * sizeof(TA)) % 16 == 0;
// This lane's ITEMS elements from t0 (all in range when FULL), folded in order.
template <bool FULL, class TAx = TA>
__device__ __forceinline__ void bcx_lane_fold(const TAx *__restrict__ a, const TB *__restrict__ b,
                                              unsigned long long t0, unsigned long long hi, int vec, T &v, int &h) {
  v = T();
  h = 0;
  if constexpr (BCX_VEC_OK && FULL) {
    if (vec) {
      constexpr int V = (int)(BCX_ITEMS * sizeof(TA) / 16);
      uint4 u[V > 0 ? V : 1];
#pragma unroll
      for (int j = 0; j < V; ++j) u[j] = __ldcs(reinterpret_cast<const uint4 *>(a + t0) + j);
      TAx x[BCX_ITEMS];
      bcx_copy<(sizeof(x) < sizeof(u) ? sizeof(x) : sizeof(u))>(x, u);
#pragma unroll
      for (int k = 0; k < BCX_ITEMS; ++k) bcx_comb(v, h, (T)x[k], 1);
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < BCX_ITEMS; ++k)
    if (FULL || t0 + k < hi) bcx_comb(v, h, bcx_load(a, b, t0 + k), 1);
}

extern "C" __global__ void __launch_bounds__(256)
bcx_jit_fold(const TA *__restrict__ a, const TB *__restrict__ b, unsigned long long n, unsigned long long per_warp,
             T *__restrict__ part, int *__restrict__ part_has, unsigned *__restrict__ done, T init, int has_init,
             T *__restrict__ out, int vec) {
  __shared__ __align__(16) unsigned char s_raw[8 * sizeof(T)];
  __shared__ int s_has[8];
  __shared__ bool s_last;
  T *s_val = reinterpret_cast<T *>(s_raw);
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned long long gw = (unsigned long long)blockIdx.x * 8 + warp;
  const unsigned long long lo = gw * per_warp < n ? gw * per_warp : n;
  const unsigned long long hi = lo + per_warp < n ? lo + per_warp : n;
  T acc = T();
  int acc_h = 0;
  unsigned long long base = lo;
  // two chunks per step, so two chunks of loads are in flight
  for (; base + 2 * BCX_CHUNK <= hi; base += 2 * BCX_CHUNK) {
    T v0, v1;
    int h0, h1;
    bcx_lane_fold<true>(a, b, base + lane * BCX_ITEMS, hi, vec, v0, h0);
    bcx_lane_fold<true>(a, b, base + BCX_CHUNK + lane * BCX_ITEMS, hi, vec, v1, h1);
    v0 = bcx_warp_fold(v0, h0);
    v1 = bcx_warp_fold(v1, h1);
    bcx_comb(acc, acc_h, v0, h0);
    bcx_comb(acc, acc_h, v1, h1);
  }
  for (; base < hi; base += BCX_CHUNK) {
    T v;
    int h;
    bcx_lane_fold<false>(a, b, base + lane * BCX_ITEMS, hi, vec, v, h);
    v = bcx_warp_fold(v, h);
    bcx_comb(acc, acc_h, v, h);
  }
  if (lane == 0) { s_val[warp] = acc; s_has[warp] = acc_h; }
  __syncthreads();
  if (warp == 0) {
    T w = lane < 8 ? s_val[lane] : T();
    int wh = lane < 8 ? s_has[lane] : 0;
    w = bcx_warp_fold(w, wh);
    if (lane == 0) {
      part[blockIdx.x] = w;
      part_has[blockIdx.x] = wh;
      __threadfence();
      s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!s_last || warp != 0) return;
  __threadfence();
  T r = T();
  int rh = 0;
  if (has_init) { r = init; rh = 1; }
  for (unsigned base2 = 0; base2 < gridDim.x; base2 += 32) {
    const unsigned i = base2 + lane;
    T w = T();
    int wh = 0;
    if (i < gridDim.x) { w = bcx_ldcg(part + i); wh = __ldcg(part_has + i); }
    w = bcx_warp_fold(w, wh);
    bcx_comb(r, rh, w, wh);
  }
  if (lane == 0 && rh) *out = r;
}
)BCX";
  return src.str();
}

inline void jit_fold(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                     const std::string &load, const char *ta, const char *tb, const void *a, const void *b,
                     size_t n, const void *init, void *out, command_queue &queue, size_t ta_size = 0) {
  const std::string s = jit_fold_source(defs, op, t, tsize, load, ta, tb);
  const size_t items = size_t(jit_items(tsize));
  const size_t chunk = 32 * items;
  const size_t chunks = (n + chunk - 1) / chunk;
  // about 8 blocks of 8 warps per SM, each warp a contiguous range of whole
  // chunks (at least 4)
  size_t warps = size_t(sm_count()) * 64;
  const size_t max_warps = (chunks + 3) / 4;
  if (warps > max_warps) warps = max_warps;
  if (warps < 1) warps = 1;
  const size_t per_warp_chunks = (chunks + warps - 1) / warps;
  unsigned long long per_warp = (unsigned long long)(per_warp_chunks * chunk);
  const size_t blocks = ((chunks + per_warp_chunks - 1) / per_warp_chunks + 7) / 8;
  const size_t tas = ta_size ? ta_size : tsize;
  int vec = jit_plain_load(load) && (items * tas) % 16 == 0 && reinterpret_cast<uintptr_t>(a) % 16 == 0;
  // partials, their flags and the ticket of the last block, in one temporary
  const size_t part_bytes = (blocks * tsize + 255) & ~size_t(255);
  const size_t has_bytes = (blocks * sizeof(int) + 255) & ~size_t(255);
  void *tmp = nullptr;
  check(bcx_malloc_async(&tmp, part_bytes + has_bytes + 256, queue.get()));
  char *base = static_cast<char *>(tmp);
  void *part = base, *part_has = base + part_bytes, *done = base + part_bytes + has_bytes;
  check(bcx_memset_async(done, 0, 4, queue.get()));
  std::vector<unsigned char> init_bytes(tsize + 16, 0);
  if (init) std::memcpy(init_bytes.data(), init, tsize);
  int has_init = init != nullptr;
  unsigned long long nn = n;
  const void *bb = b ? b : a;
  void *args[] = {(void *)&a, (void *)&bb, (void *)&nn, (void *)&per_warp, (void *)&part, (void *)&part_has,
                  (void *)&done, (void *)init_bytes.data(), (void *)&has_init, (void *)&out, (void *)&vec};
  jit_launch(s, "bcx_jit_fold", unsigned(blocks), 256, queue, args);
  check(bcx_free_async(tmp, queue.get()));
}

// accumulate(first, last, init, f) where the result type T (init's type)
// differs from the element type IT: the reference folds serially on one
// work-item, converting every intermediate result to T (detail/
// serial_accumulate.hpp:33-49, accumulate.hpp:31-55), so the result depends
// on the order and cannot be reassociated.  One warp reads 32 elements at a
// time (coalesced) and folds them in order: acc = (T)(OP) with _1 = acc,
// _2 = the element.  Writes the result to `out` (device).
inline std::string jit_serial_fold_source(const std::string &defs, const std::string &op, const char *t,
                                          const char *it) {
  std::ostringstream src;
  src << jit_prelude() << defs << "\n"
      << "typedef " << t << " T;\ntypedef " << it << " IT;\n"
      << R"BCX(
extern "C" __global__ void __launch_bounds__(32)
bcx_jit_serial_fold(const IT *__restrict__ in, unsigned long long n, T init, T *__restrict__ out) {
  const unsigned lane = threadIdx.x;
  constexpr int W = (int)((sizeof(IT) + 3) / 4);
  T acc = init;
  for (unsigned long long b = 0; b < n; b += 32) {
    IT v = IT();
    if (b + lane < n) v = in[b + lane];
    unsigned w[W];
#pragma unroll
    for (int k = 0; k < W; ++k) w[k] = 0u;
    {
      const unsigned char *src = reinterpret_cast<const unsigned char *>(&v);
      unsigned char *dst = reinterpret_cast<unsigned char *>(w);
      for (int k = 0; k < (int)sizeof(IT); ++k) dst[k] = src[k];
    }
    const unsigned cnt = (n - b) < 32ull ? (unsigned)(n - b) : 32u;
    for (unsigned j = 0; j < cnt; ++j) {
      unsigned x[W];
#pragma unroll
      for (int k = 0; k < W; ++k) x[k] = __shfl_sync(0xffffffffu, w[k], (int)j);
      IT _2;
      {
        const unsigned char *src = reinterpret_cast<const unsigned char *>(x);
        unsigned char *dst = reinterpret_cast<unsigned char *>(&_2);
        for (int k = 0; k < (int)sizeof(IT); ++k) dst[k] = src[k];
      }
      const T _1 = acc;
      acc = (T)()BCX" << op << R"BCX();
    }
  }
  if (lane == 0) *out = acc;
}
)BCX";
  return src.str();
}

inline void jit_serial_fold(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                            const char *it, const void *in, size_t n, const void *init, void *out,
                            command_queue &queue) {
  std::vector<unsigned char> init_bytes(tsize + 16, 0);
  std::memcpy(init_bytes.data(), init, tsize);
  unsigned long long nn = n;
  void *args[] = {(void *)&in, (void *)&nn, (void *)init_bytes.data(), (void *)&out};
  jit_launch(jit_serial_fold_source(defs, op, t, it), "bcx_jit_serial_fold", 1, 32, queue, args);
}

inline void jit_reduce(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                       const void *in, size_t n, const void *init, void *out, command_queue &queue) {
  jit_fold(defs, op, t, tsize, "return a[i];", t, nullptr, in, nullptr, n, init, out, queue);
}

// Scan with a user functor: one launch of a single-pass decoupled look-back
// scan (the design of the library's built-in scan, detail/scan_on_gpu.hpp
// replaced): each block takes the next tile from a ticket and asks L2 for the
// tile prefetch_tiles tickets ahead.  With 16-byte aligned input and output
// and an element size that divides 16, the staged kernel moves each whole
// tile into shared memory by bulk copies and back out the same way (the
// built-in scan's design); otherwise register tiles are used, full aligned
// ones arriving through a shared-memory transpose (coalesced 16-byte loads,
// then each thread reads its contiguous run).  Either way the tile is scanned
// a thread's run, then the warp, then the block at a time, its aggregate
// published, and warp 0 looks back over 32 predecessor tiles per step
// (lookback_depth windows polled at once) -- bounded waits, reported through
// the library's error word -- for the exclusive prefix, which every thread
// folds into its outputs.  Exclusive scans start from init (tile 0 publishes
// init OP its aggregate).  In place is allowed: a tile is read whole before
// any of it is written, and no other tile touches it.  Asynchronous on the
// queue: no host waits, and the status array is a stream-ordered temporary.
// Tuning knobs of the register-tile kernel (-1 or 0 = default): items per
// thread, evict-first hints, prefetch distance, two_read (re-read the tile
// from L2 instead of keeping it in registers across the look-back), look-back
// depth, transpose.  staged_tile_bytes > 0 generates the staged kernel
// bcx_jit_scan_staged (tiles of that many bytes), else bcx_jit_scan.
inline std::string jit_scan_source(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                                   int items_override = 0, bool streaming = true, int prefetch_tiles = -1,
                                   int two_read = -1, int lookback_depth = 1, int transpose = -1,
                                   int staged_tile_bytes = 0) {
  if (two_read < 0) two_read = jit_scan_two_read();
  if (transpose < 0) transpose = jit_scan_transpose();
  const int items = items_override > 0 ? items_override : jit_scan_items(tsize);
  if (prefetch_tiles < 0)
    prefetch_tiles = staged_tile_bytes > 0 ? int(jit_scan_staged_prefetch_bytes() / size_t(staged_tile_bytes))
                                           : jit_scan_prefetch_tiles();
  const bool packed = tsize <= 4;
  const int staged_blocks = staged_tile_bytes > 0 ? (227 * 1024) / (staged_tile_bytes + 1024) : 1;
  std::ostringstream src;
  src << jit_common(defs, op, t) << "#define BCX_STAGED " << (staged_tile_bytes > 0 ? 1 : 0)
      << "\n#define BCX_STAGED_TILE_BYTES " << (staged_tile_bytes > 0 ? staged_tile_bytes : 16)
      << "\n#define BCX_STAGED_BLOCKS " << (staged_blocks < 8 ? staged_blocks : 8)
      << "\n#define BCX_ITEMS " << items << "\n#define BCX_PACKED " << (packed ? 1 : 0)
      << "\n#define BCX_PREFETCH_TILES " << prefetch_tiles << "\n#define BCX_TWO_READ " << two_read
      << "\n#define BCX_LOOKBACK_DEPTH " << (lookback_depth > 0 ? lookback_depth : 1)
      << "\n#define BCX_TRANSPOSE " << ((transpose && (items * tsize) % 16 == 0) ? 1 : 0)
      << "\n#define BCX_LD(p) " << (streaming ? "__ldcs(p)" : "(*(p))") << "\n#define BCX_ST(p, v) "
      << (streaming ? "__stcs(p, v)" : "(*(p) = (v))")
      << R"BCX(
#define BCX_SPIN_LIMIT (1u << 22)
// Tile status: flag 0 = nothing yet, 1 = aggregate, 2 = inclusive prefix.
#if BCX_PACKED
// flag and value (<= 4 bytes) in one 64-bit word: one relaxed access each way
__device__ __forceinline__ void bcx_publish(unsigned long long *words, unsigned *, T *, T *, unsigned long long t,
                                            unsigned flag, const T &v) {
  unsigned bits = 0u;
  bcx_copy<sizeof(T)>(&bits, &v);
  const unsigned long long x = ((unsigned long long)bits << 32) | flag;
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(words + t), "l"(x) : "memory");
}
__device__ __forceinline__ unsigned bcx_poll(unsigned long long *words, unsigned *, T *, T *, unsigned long long t,
                                             T *v) {
  unsigned long long x;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(x) : "l"(words + t) : "memory");
  const unsigned bits = unsigned(x >> 32);
  bcx_copy<sizeof(T)>(v, &bits);
  return unsigned(x & 0xffffffffu);
}
#else
// flag word ordered after the value by release/acquire; values read from L2
__device__ __forceinline__ void bcx_publish(unsigned long long *, unsigned *flags, T *agg, T *inc,
                                            unsigned long long t, unsigned flag, const T &v) {
  (flag == 1u ? agg : inc)[t] = v;
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(flags + t), "r"(flag) : "memory");
}
__device__ __forceinline__ unsigned bcx_poll(unsigned long long *, unsigned *flags, T *agg, T *inc,
                                             unsigned long long t, T *v) {
  unsigned f;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(f) : "l"(flags + t) : "memory");
  if (f) *v = bcx_ldcg((f == 1u ? agg : inc) + t);
  return f;
}
#endif

// Warp 0: exclusive prefix of tile `tile` (>= 1) over its predecessors.
__device__ T bcx_lookback(unsigned long long *words, unsigned *flags, T *agg, T *inc, unsigned long long tile,
                          unsigned *err) {
  // Each step polls BCX_LOOKBACK_DEPTH windows of 32 predecessors at once (one
  // L2 round trip), then folds them nearest first up to the nearest prefix.
  const unsigned lane = threadIdx.x & 31u;
  T ex = T();
  int eh = 0;
  long long pred = (long long)tile - 1;
  bool gave_up = false;
  while (true) {
    T v[BCX_LOOKBACK_DEPTH];
    unsigned f[BCX_LOOKBACK_DEPTH];
    int vh[BCX_LOOKBACK_DEPTH];
#pragma unroll
    for (int j = 0; j < BCX_LOOKBACK_DEPTH; ++j) {
      const long long t = pred - (long long)lane - 32ll * j;
      v[j] = T();
      f[j] = 2u;  // before tile 0: never reached (tile 0 publishes a prefix)
      vh[j] = 0;
      if (t >= 0) { f[j] = bcx_poll(words, flags, agg, inc, (unsigned long long)t, &v[j]); vh[j] = 1; }
    }
    bool done = false;
#pragma unroll
    for (int j = 0; j < BCX_LOOKBACK_DEPTH; ++j) {
      if (done) break;
      const long long t = pred - (long long)lane - 32ll * j;
      unsigned spins = 0;
      while (true) {
        const unsigned pmask = __ballot_sync(0xffffffffu, f[j] == 2u);
        const int first = pmask ? __ffs(pmask) - 1 : 31;
        const unsigned need = first == 31 ? 0xffffffffu : ((2u << first) - 1u);
        if (!(__ballot_sync(0xffffffffu, f[j] == 0u) & need)) break;
        if (++spins > BCX_SPIN_LIMIT) {
          gave_up = true;
          if (f[j] == 0u) { f[j] = 2u; vh[j] = 0; }
          break;
        }
        __nanosleep(spins < 32 ? 32 : 256);
        if (f[j] == 0u && t >= 0) f[j] = bcx_poll(words, flags, agg, inc, (unsigned long long)t, &v[j]);
      }
      const unsigned pmask = __ballot_sync(0xffffffffu, f[j] == 2u);
      const int first = pmask ? __ffs(pmask) - 1 : 31;
      int wh = ((int)lane <= first) ? vh[j] : 0;
      // lane order is newest-first: fold from the oldest (highest lane) down
      const T rv = bcx_shfl_idx(v[j], 31 - (int)lane);
      int fh = __shfl_sync(0xffffffffu, wh, 31 - (int)lane);
      const T w = bcx_warp_fold(rv, fh);
      if (fh) {
        ex = eh ? bcx_op(w, ex) : w;
        eh = 1;
      }
      done = pmask != 0;
    }
    if (done) break;
    pred -= 32ll * BCX_LOOKBACK_DEPTH;
  }
  if (__any_sync(0xffffffffu, gave_up) && lane == 0 && err) atomicOr(err, 1u);
  return ex;
}

// This thread's elements t0 .. t0+ITEMS-1 (vector loads for full aligned
// tiles; `keep` caches the read in L2 for a second read).
template <bool FULL>
__device__ __forceinline__ void bcx_scan_load(const T *in, unsigned long long t0, int cnt, int vec,
                                              T (&x)[BCX_ITEMS], bool keep) {
  if (FULL && vec) {
    constexpr int V = (int)(BCX_ITEMS * sizeof(T) / 16);
    uint4 u[V > 0 ? V : 1];
#pragma unroll
    for (int j = 0; j < V; ++j)
      u[j] = keep ? __ldcg(reinterpret_cast<const uint4 *>(in + t0) + j)
                  : BCX_LD(reinterpret_cast<const uint4 *>(in + t0) + j);
    bcx_copy<(sizeof(x) < sizeof(u) ? sizeof(x) : sizeof(u))>(x, u);
  } else {
#pragma unroll
    for (int k = 0; k < BCX_ITEMS; ++k) x[k] = (FULL || k < cnt) ? in[t0 + k] : T();
  }
}

// Full aligned tiles moved through shared memory: the warp reads and writes
// global memory in coalesced 16-byte vectors (lane-consecutive), each thread
// works on its contiguous run.  One 16-byte pad slot every 8 vectors keeps a
// thread's run reads free of bank conflicts.
constexpr int BCX_TVECS = (int)(256ull * BCX_ITEMS * sizeof(T) / 16);
constexpr int BCX_TV = (int)(BCX_ITEMS * sizeof(T) / 16);  // vectors per thread
__device__ __forceinline__ int bcx_pad(int i) { return i + (i >> 3); }
__device__ __forceinline__ uint4 *bcx_tile_smem() {
  __shared__ uint4 s_tile[BCX_TRANSPOSE ? BCX_TVECS + BCX_TVECS / 8 : 1];
  return s_tile;
}
__device__ __forceinline__ void bcx_transpose_load(const T *in, unsigned long long tile_base, T (&x)[BCX_ITEMS]) {
  uint4 *sm = bcx_tile_smem();
  const uint4 *src = reinterpret_cast<const uint4 *>(in + tile_base);
#pragma unroll
  for (int j = 0; j < BCX_TV; ++j) {
    const int i = j * 256 + (int)threadIdx.x;
    sm[bcx_pad(i)] = BCX_LD(src + i);
  }
  __syncthreads();
  uint4 u[BCX_TV > 0 ? BCX_TV : 1];
#pragma unroll
  for (int j = 0; j < BCX_TV; ++j) u[j] = sm[bcx_pad((int)threadIdx.x * BCX_TV + j)];
  bcx_copy<(sizeof(x) < sizeof(u) ? sizeof(x) : sizeof(u))>(x, u);
}
__device__ __forceinline__ void bcx_transpose_store(T *out, unsigned long long tile_base, const T (&y)[BCX_ITEMS]) {
  uint4 *sm = bcx_tile_smem();
  uint4 u[BCX_TV > 0 ? BCX_TV : 1];
  bcx_copy<(sizeof(y) < sizeof(u) ? sizeof(y) : sizeof(u))>(u, y);
  // every thread has read its own run before the look-back barrier, so the
  // runs can be overwritten in place
#pragma unroll
  for (int j = 0; j < BCX_TV; ++j) sm[bcx_pad((int)threadIdx.x * BCX_TV + j)] = u[j];
  __syncthreads();
  uint4 *dst = reinterpret_cast<uint4 *>(out + tile_base);
#pragma unroll
  for (int j = 0; j < BCX_TV; ++j) {
    const int i = j * 256 + (int)threadIdx.x;
    BCX_ST(dst + i, sm[bcx_pad(i)]);
  }
}

template <bool FULL>
__device__ __forceinline__ void bcx_scan_tile(const T *in, T *out, unsigned long long n, unsigned long long tile,
                                              unsigned long long *words, unsigned *flags, T *agg, T *inc,
                                              const T &init, int has_init, int exclusive, int vec, unsigned *err) {
  constexpr unsigned long long TILE = 256ull * BCX_ITEMS;
  __shared__ __align__(16) unsigned char s_raw[9 * sizeof(T)];
  __shared__ int s_has[9];
  T *s_val = reinterpret_cast<T *>(s_raw);  // [0, 8): warp totals; [8]: tile prefix
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned long long t0 = tile * TILE + (unsigned long long)threadIdx.x * BCX_ITEMS;
  int cnt = BCX_ITEMS;
  if (!FULL) {
    const long long r = (long long)n - (long long)t0;
    cnt = r <= 0 ? 0 : (r < BCX_ITEMS ? (int)r : BCX_ITEMS);
  }
  T x[BCX_ITEMS];
  const unsigned long long tile_base = tile * TILE;
  if (BCX_TRANSPOSE && FULL && vec) bcx_transpose_load(in, tile_base, x);
  else bcx_scan_load<FULL>(in, t0, cnt, vec, x, BCX_TWO_READ != 0);
  // this thread's run, inclusive (kept in x unless the tile is read twice)
  T run = x[0];
#pragma unroll
  for (int k = 1; k < BCX_ITEMS; ++k)
    if (FULL || k < cnt) {
      run = bcx_op(run, x[k]);
      if (!BCX_TWO_READ) x[k] = run;
    }
  int h = FULL ? 1 : (cnt > 0);
  // lanes of the warp, inclusive
  T a = run;
#pragma unroll
  for (unsigned d = 1; d < 32; d <<= 1) {
    const T o = bcx_shfl_up(a, d);
    const int oh = __shfl_up_sync(0xffffffffu, h, d);
    if (lane >= d && oh) { a = h ? bcx_op(o, a) : o; h = 1; }
  }
  const T lane_ex = bcx_shfl_up(a, 1);
  int lane_eh = __shfl_up_sync(0xffffffffu, h, 1);
  if (lane == 0) lane_eh = 0;
  if (lane == 31) { s_val[warp] = a; s_has[warp] = h; }
  __syncthreads();
  if (warp == 0) {
    T w = lane < 8 ? s_val[lane] : T();
    int wh = lane < 8 ? s_has[lane] : 0;
    const T agg_t = bcx_warp_fold(w, wh);
    T ex = T();
    int eh = 0;
    if (tile == 0) {
      if (has_init) { ex = init; eh = 1; }
      const T inc_t = eh ? bcx_op(ex, agg_t) : agg_t;
      if (lane == 0) bcx_publish(words, flags, agg, inc, 0, 2u, inc_t);
    } else {
      if (lane == 0) bcx_publish(words, flags, agg, inc, tile, 1u, agg_t);
      ex = bcx_lookback(words, flags, agg, inc, tile, err);
      eh = 1;
      if (lane == 0) bcx_publish(words, flags, agg, inc, tile, 2u, bcx_op(ex, agg_t));
    }
    if (lane == 0) { s_val[8] = ex; s_has[8] = eh; }
  }
  __syncthreads();
  // prefix of this thread's run: tile prefix, earlier warps, earlier lanes
  T p = s_val[8];
  int ph = s_has[8];
  for (unsigned j = 0; j < warp; ++j) bcx_comb(p, ph, s_val[j], s_has[j]);
  bcx_comb(p, ph, lane_ex, lane_eh);
  T y[BCX_ITEMS];
  if (BCX_TWO_READ) {
    // second read of the tile (from L2): fold the prefix through the run
    bcx_scan_load<FULL>(in, t0, cnt, vec, x, false);
    T r = p;
    int rh = ph;
#pragma unroll
    for (int k = 0; k < BCX_ITEMS; ++k) {
      if (exclusive) y[k] = rh ? r : T();
      bcx_comb(r, rh, x[k], 1);
      if (!exclusive) y[k] = r;
    }
  } else if (exclusive) {
    y[0] = ph ? p : T();
#pragma unroll
    for (int k = 1; k < BCX_ITEMS; ++k) y[k] = ph ? bcx_op(p, x[k - 1]) : x[k - 1];
  } else {
#pragma unroll
    for (int k = 0; k < BCX_ITEMS; ++k) y[k] = ph ? bcx_op(p, x[k]) : x[k];
  }
  if (BCX_TRANSPOSE && FULL && vec) {
    bcx_transpose_store(out, tile_base, y);
  } else if (FULL && vec) {
    constexpr int V = (int)(BCX_ITEMS * sizeof(T) / 16);
    uint4 u[V > 0 ? V : 1];
    bcx_copy<(sizeof(y) < sizeof(u) ? sizeof(y) : sizeof(u))>(u, y);
#pragma unroll
    for (int j = 0; j < V; ++j) BCX_ST(reinterpret_cast<uint4 *>(out + t0) + j, u[j]);
  } else {
#pragma unroll
    for (int k = 0; k < BCX_ITEMS; ++k)
      if (FULL || k < cnt) out[t0 + k] = y[k];
  }
}

#if !BCX_STAGED
extern "C" __global__ void __launch_bounds__(256)
bcx_jit_scan(const T *in, T *out, unsigned long long n, unsigned *ticket, unsigned long long *words,
             unsigned *flags, T *agg, T *inc, T init, int has_init, int exclusive, int vec, unsigned *err) {
  __shared__ unsigned s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const unsigned long long tile = s_tile;
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  // ask L2 for the tile BCX_PREFETCH_TILES tickets ahead (16-byte aligned
  // input only, clipped to the array)
  if (BCX_PREFETCH_TILES > 0 && vec && threadIdx.x == 0) {
    const unsigned long long f0 = (tile + BCX_PREFETCH_TILES) * (256ull * BCX_ITEMS);
    if (f0 < n) {
      const unsigned long long m = n - f0 < 256ull * BCX_ITEMS ? n - f0 : 256ull * BCX_ITEMS;
      const unsigned bytes = (unsigned)(m * sizeof(T)) & ~15u;
      if (bytes)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(in + f0), "r"(bytes) : "memory");
    }
  }
#endif
  if (n - tile * (256ull * BCX_ITEMS) >= 256ull * BCX_ITEMS)
    bcx_scan_tile<true>(in, out, n, tile, words, flags, agg, inc, init, has_init, exclusive, vec, err);
  else
    bcx_scan_tile<false>(in, out, n, tile, words, flags, agg, inc, init, has_init, exclusive, vec, err);
}
#endif  // !BCX_STAGED

#if BCX_STAGED
// ---- staged tiles ----------------------------------------------------------
// One block = one tile of BCX_STAGED_TILE_BYTES, moved into shared memory by
// bulk copies on an mbarrier (the whole tile in flight at once, no registers
// held for it) and out again by bulk copies after the scan.  Thread t owns the
// contiguous run of BCX_SVPT 16-byte vectors from vector t*BCX_SVPT and visits
// them from vector (t mod BCX_SVPT) on, wrapping around, so the eight threads
// of each shared-memory phase touch eight different bank groups; the run is
// still combined in element order (vectors [r, VPT) fold into pa, [0, r) into
// pb, and the run is pb then pa).  The second pass rewrites the run in place
// with its outputs.  Every wait is bounded.
#define BCX_SVPT ((int)(BCX_STAGED_TILE_BYTES / (256 * 16)))
#define BCX_SN ((int)(16 / sizeof(T)))
#define BCX_SITEMS (BCX_SVPT * BCX_SN)
#define BCX_SPIECE 16384u
__device__ __forceinline__ unsigned bcx_smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool bcx_mbar_wait(unsigned long long *bar) {
  for (unsigned i = 0; i < BCX_SPIN_LIMIT; ++i) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(bcx_smem_addr(bar))
                 : "memory");
    if (ok) return true;
  }
  return false;
}

extern "C" __global__ void __launch_bounds__(256, BCX_STAGED_BLOCKS)
bcx_jit_scan_staged(const T *in, T *out, unsigned long long n, unsigned *ticket, unsigned long long *words,
                    unsigned *flags, T *agg, T *inc, T init, int has_init, int exclusive, unsigned *err) {
  extern __shared__ __align__(128) unsigned char bcx_stage[];
  uint4 *tv = reinterpret_cast<uint4 *>(bcx_stage);
  T *te = reinterpret_cast<T *>(bcx_stage);
  __shared__ unsigned long long s_bar;
  __shared__ unsigned s_tile;
  __shared__ __align__(16) unsigned char s_raw[9 * sizeof(T)];
  __shared__ int s_has[9];
  T *s_val = reinterpret_cast<T *>(s_raw);  // [0, 8): warp totals; [8]: tile prefix
  constexpr unsigned long long TILE = 256ull * BCX_SITEMS;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(ticket, 1u);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bcx_smem_addr(&s_bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const unsigned long long tile = s_tile;
  const unsigned long long base = tile * TILE;
  const unsigned cnt = (unsigned)(n - base < TILE ? n - base : TILE);
  const unsigned bulk = (cnt * (unsigned)sizeof(T)) & ~15u;
  const unsigned bulk_elems = bulk / (unsigned)sizeof(T);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bcx_smem_addr(&s_bar)), "r"(bulk)
                 : "memory");
    const char *src = reinterpret_cast<const char *>(in + base);
    for (unsigned off = 0; off < bulk; off += BCX_SPIECE) {
      const unsigned len = bulk - off < BCX_SPIECE ? bulk - off : BCX_SPIECE;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       bcx_smem_addr(bcx_stage + off)),
                   "l"(src + off), "r"(len), "r"(bcx_smem_addr(&s_bar))
                   : "memory");
    }
    // ask L2 for the tile BCX_PREFETCH_TILES tickets ahead
    const unsigned long long f0 = (tile + BCX_PREFETCH_TILES) * TILE;
    if (BCX_PREFETCH_TILES > 0 && f0 < n) {
      const unsigned long long m = n - f0 < TILE ? n - f0 : TILE;
      const unsigned pf = (unsigned)(m * sizeof(T)) & ~15u;
      const char *ps = reinterpret_cast<const char *>(in + f0);
      for (unsigned off = 0; off < pf; off += BCX_SPIECE)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ps + off),
                     "r"(pf - off < BCX_SPIECE ? pf - off : BCX_SPIECE)
                     : "memory");
    }
  }
  // the last tile's ragged end (under 16 bytes) comes in by plain loads
  for (unsigned i = bulk_elems + threadIdx.x; i < cnt; i += 256) te[i] = in[base + i];
  const bool arrived = bcx_mbar_wait(&s_bar);
  if (__syncthreads_or(!arrived)) {
    // leave only after the copies into this block's shared memory are done
    if (threadIdx.x == 0) {
      if (err) atomicOr(err, 2u);
      bcx_mbar_wait(&s_bar);
    }
    return;
  }
  const unsigned t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const bool full = cnt == TILE;
  const unsigned e_first = t * (unsigned)BCX_SITEMS;
  const int r = (int)(t % (unsigned)BCX_SVPT);
  // pass 1: the run's total, in element order (a full tile has every
  // element, so only each part's first element needs no combine)
  T a = T(), pa = T();
  int ah = 0, pah = 0;
  if (full) {
#pragma unroll
    for (int k = 0; k < BCX_SVPT; ++k) {
      int v = k + r;
      if (v >= BCX_SVPT) v -= BCX_SVPT;
      const uint4 u = tv[t * BCX_SVPT + v];
      T x[BCX_SN];
      bcx_copy<16>(x, &u);
      if (k == 0) {
        a = x[0];
      } else if (v == 0) {
        pa = a;
        a = x[0];
      } else {
        a = bcx_op(a, x[0]);
      }
#pragma unroll
      for (int m = 1; m < BCX_SN; ++m) a = bcx_op(a, x[m]);
    }
    ah = 1;
    if (r != 0) pah = 1;
  } else {
#pragma unroll
    for (int k = 0; k < BCX_SVPT; ++k) {
      int v = k + r;
      if (v >= BCX_SVPT) v -= BCX_SVPT;
      if (k > 0 && v == 0) {
        pa = a;
        pah = ah;
        a = T();
        ah = 0;
      }
      const uint4 u = tv[t * BCX_SVPT + v];
      T x[BCX_SN];
      bcx_copy<16>(x, &u);
#pragma unroll
      for (int m = 0; m < BCX_SN; ++m)
        if (e_first + (unsigned)(v * BCX_SN + m) < cnt) bcx_comb(a, ah, x[m], 1);
    }
  }
  T pb = T();
  int pbh = 0;
  if (r == 0) {
    pa = a;
    pah = ah;
  } else {
    pb = a;
    pbh = ah;
  }
  T run = pb;
  int h = pbh;
  bcx_comb(run, h, pa, pah);
  // lanes of the warp, inclusive
  T ia = run;
#pragma unroll
  for (unsigned d = 1; d < 32; d <<= 1) {
    const T o = bcx_shfl_up(ia, d);
    const int oh = __shfl_up_sync(0xffffffffu, h, d);
    if (lane >= d && oh) { ia = h ? bcx_op(o, ia) : o; h = 1; }
  }
  const T lane_ex = bcx_shfl_up(ia, 1);
  int lane_eh = __shfl_up_sync(0xffffffffu, h, 1);
  if (lane == 0) lane_eh = 0;
  if (lane == 31) { s_val[warp] = ia; s_has[warp] = h; }
  __syncthreads();
  if (warp == 0) {
    T w = lane < 8 ? s_val[lane] : T();
    int wh = lane < 8 ? s_has[lane] : 0;
    const T agg_t = bcx_warp_fold(w, wh);
    T ex = T();
    int eh = 0;
    if (tile == 0) {
      if (has_init) { ex = init; eh = 1; }
      const T inc_t = eh ? bcx_op(ex, agg_t) : agg_t;
      if (lane == 0) bcx_publish(words, flags, agg, inc, 0, 2u, inc_t);
    } else {
      if (lane == 0) bcx_publish(words, flags, agg, inc, tile, 1u, agg_t);
      ex = bcx_lookback(words, flags, agg, inc, tile, err);
      eh = 1;
      if (lane == 0) bcx_publish(words, flags, agg, inc, tile, 2u, bcx_op(ex, agg_t));
    }
    if (lane == 0) { s_val[8] = ex; s_has[8] = eh; }
  }
  __syncthreads();
  // prefix of this thread's run: tile prefix, earlier warps, earlier lanes
  T p = s_val[8];
  int ph = s_has[8];
  for (unsigned j = 0; j < warp; ++j) bcx_comb(p, ph, s_val[j], s_has[j]);
  bcx_comb(p, ph, lane_ex, lane_eh);
  // pass 2: outputs in place, vector r first (its prefix includes [0, r));
  // with a full tile and a prefix in hand (all but the array's first run
  // when there is no init) no element needs a flag
  T rr = p;
  int rh = ph;
  bcx_comb(rr, rh, pb, pbh);
  if (full && ph) {
#pragma unroll
    for (int k = 0; k < BCX_SVPT; ++k) {
      int v = k + r;
      if (v >= BCX_SVPT) v -= BCX_SVPT;
      if (k > 0 && v == 0) rr = p;
      uint4 u = tv[t * BCX_SVPT + v];
      T x[BCX_SN], y[BCX_SN];
      bcx_copy<16>(x, &u);
      if (exclusive) {
#pragma unroll
        for (int m = 0; m < BCX_SN; ++m) {
          y[m] = rr;
          rr = bcx_op(rr, x[m]);
        }
      } else {
#pragma unroll
        for (int m = 0; m < BCX_SN; ++m) {
          rr = bcx_op(rr, x[m]);
          y[m] = rr;
        }
      }
      bcx_copy<16>(&u, y);
      tv[t * BCX_SVPT + v] = u;
    }
  } else {
#pragma unroll
  for (int k = 0; k < BCX_SVPT; ++k) {
    int v = k + r;
    if (v >= BCX_SVPT) v -= BCX_SVPT;
    if (k > 0 && v == 0) {
      rr = p;
      rh = ph;
    }
    uint4 u = tv[t * BCX_SVPT + v];
    T x[BCX_SN], y[BCX_SN];
    bcx_copy<16>(x, &u);
#pragma unroll
    for (int m = 0; m < BCX_SN; ++m) {
      const bool ok = full || e_first + (unsigned)(v * BCX_SN + m) < cnt;
      if (exclusive) {
        y[m] = rh ? rr : T();
        if (ok) bcx_comb(rr, rh, x[m], 1);
      } else {
        if (ok) bcx_comb(rr, rh, x[m], 1);
        y[m] = rr;
      }
    }
    bcx_copy<16>(&u, y);
    tv[t * BCX_SVPT + v] = u;
  }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0) {
    char *dst = reinterpret_cast<char *>(out + base);
    for (unsigned off = 0; off < bulk; off += BCX_SPIECE) {
      const unsigned len = bulk - off < BCX_SPIECE ? bulk - off : BCX_SPIECE;
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst + off),
                   "r"(bcx_smem_addr(bcx_stage + off)), "r"(len)
                   : "memory");
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  }
  for (unsigned i = bulk_elems + threadIdx.x; i < cnt; i += 256) out[base + i] = te[i];
}
#endif  // BCX_STAGED
)BCX";
  return src.str();
}

inline void jit_scan(const std::string &defs, const std::string &op, const char *t, size_t tsize,
                     const void *in, void *out, size_t n, bool exclusive, const void *init,
                     command_queue &queue, int items_override = 0, bool streaming = true, int prefetch_tiles = -1,
                     int two_read = -1, int lookback_depth = 1, int transpose = -1, int staged = -1) {
  if (n == 0) return;
  // The staged kernel takes 16-byte aligned input and output whose element
  // size divides 16; anything else takes the register-tile kernel.
  const bool aligned = reinterpret_cast<uintptr_t>(in) % 16 == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0;
  const int stage_bytes = (staged != 0 && aligned) ? jit_scan_staged_tile_bytes(tsize) : 0;
  const std::string s = jit_scan_source(defs, op, t, tsize, items_override, streaming, prefetch_tiles, two_read,
                                        lookback_depth, transpose, stage_bytes);
  const int items = items_override > 0 ? items_override : jit_scan_items(tsize);
  const bool packed = tsize <= 4;
  const size_t tile = stage_bytes > 0 ? size_t(stage_bytes) / tsize : size_t(256) * size_t(items);
  const size_t tiles = (n + tile - 1) / tile;
  // ticket | status words (packed) or flags + aggregates + inclusive prefixes
  const size_t a256 = 255;
  const size_t flag_bytes = packed ? ((tiles * 8 + a256) & ~a256) : ((tiles * 4 + a256) & ~a256);
  const size_t val_bytes = packed ? 0 : ((tiles * tsize + a256) & ~a256);
  void *tmp = nullptr;
  check(bcx_malloc_async(&tmp, 256 + flag_bytes + 2 * val_bytes, queue.get()));
  char *base = static_cast<char *>(tmp);
  void *ticket = base;
  void *words = packed ? base + 256 : nullptr;
  void *flags = packed ? nullptr : base + 256;
  void *agg = packed ? nullptr : base + 256 + flag_bytes;
  void *inc = packed ? nullptr : base + 256 + flag_bytes + val_bytes;
  check(bcx_memset_async(tmp, 0, 256 + flag_bytes, queue.get()));
  void *err = nullptr;
  check(bcx_device_error_word(&err));
  std::vector<unsigned char> init_bytes(tsize + 16, 0);
  int has_init = exclusive && init != nullptr;
  if (has_init) std::memcpy(init_bytes.data(), init, tsize);
  int ex = exclusive ? 1 : 0;
  int vec = (items * tsize) % 16 == 0 && aligned;
  unsigned long long nn = n;
  if (stage_bytes > 0) {
    void *args[] = {(void *)&in, (void *)&out, (void *)&nn, (void *)&ticket, (void *)&words, (void *)&flags,
                    (void *)&agg, (void *)&inc, (void *)init_bytes.data(), (void *)&has_init, (void *)&ex,
                    (void *)&err};
    jit_launch(s, "bcx_jit_scan_staged", unsigned(tiles), 256, queue, args, size_t(stage_bytes));
  } else {
    void *args[] = {(void *)&in, (void *)&out, (void *)&nn, (void *)&ticket, (void *)&words, (void *)&flags,
                    (void *)&agg, (void *)&inc, (void *)init_bytes.data(), (void *)&has_init, (void *)&ex,
                    (void *)&vec, (void *)&err};
    jit_launch(s, "bcx_jit_scan", unsigned(tiles), 256, queue, args);
  }
  check(bcx_free_async(tmp, queue.get()));
}

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
