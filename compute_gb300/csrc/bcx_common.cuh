// bcx_common.cuh -- device-side building blocks shared by every libbcx kernel:
// element-type traits, the radix key transform, built-in functors with their
// identities, warp helpers and bounded spin-waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <limits.h>

#include "bcx.h"

namespace bcx {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Unsigned bit-pattern type of each radix-sortable element
// (algorithm/detail/radix_sort.hpp:49-72, radix_sort_value_type<sizeof(T)>).
template <int N> struct bits_of;
template <> struct bits_of<1> { typedef uint8_t type; };
template <> struct bits_of<2> { typedef uint16_t type; };
template <> struct bits_of<4> { typedef uint32_t type; };
template <> struct bits_of<8> { typedef unsigned long long type; };

template <class T> struct type_traits {
  static constexpr bool is_float = false;
  static constexpr bool is_signed = (T(-1) < T(0));
};
template <> struct type_traits<float> {
  static constexpr bool is_float = true;
  static constexpr bool is_signed = true;
};
template <> struct type_traits<double> {
  static constexpr bool is_float = true;
  static constexpr bool is_signed = true;
};

// ---------------------------------------------------------------------------
// Radix key transform.  The bit operations are the reference's radix()
// (algorithm/detail/radix_sort.hpp:100-127) so that the stable LSD order -- and
// therefore every output position, including -0.0/+0.0, NaNs and the signed
// minimum in descending order -- is identical:
//   ascending  float : x ^ (-(x >> sign) | signbit)
//   ascending  signed: x ^ signbit
//   descending float : (-x) ^ (-(x >> sign) | signbit)   (mask from x, not -x)
//   descending signed: (-x) ^ signbit                      (two's complement -x)
//   descending unsigned: ~0 - x
// U is the unsigned bit type; the result is an unsigned key ordered ascending.
template <class U, bool IS_FLOAT, bool IS_SIGNED, bool DESC>
__host__ __device__ __forceinline__ U radix_key(U x) {
  constexpr int kSign = int(sizeof(U) * 8 - 1);
  constexpr U kSignBit = U(U(1) << kSign);
  if (IS_FLOAT) {
    const U mask = U(U(-(x >> kSign)) | kSignBit);
    return DESC ? U(U(-x) ^ mask) : U(x ^ mask);
  } else if (IS_SIGNED) {
    return DESC ? U(U(-x) ^ kSignBit) : U(x ^ kSignBit);
  } else {
    return DESC ? U(U(~U(0)) - x) : x;
  }
}

// ---------------------------------------------------------------------------
// Built-in binary functors (functional/operator.hpp:57-92,
// functional/integer.hpp:24-25) with the identity each scan/reduce seeds.
template <class T> struct op_plus {
  __device__ __forceinline__ T operator()(T a, T b) const { return T(a + b); }
  __device__ __forceinline__ static T identity() { return T(0); }
};
template <class T> struct op_multiplies {
  __device__ __forceinline__ T operator()(T a, T b) const { return T(a * b); }
  __device__ __forceinline__ static T identity() { return T(1); }
};
template <class T> struct num_limits;
#define BCX_LIMITS(T, LO, HI) \
  template <> struct num_limits<T> { \
    __host__ __device__ static T lowest() { return LO; } \
    __host__ __device__ static T highest() { return HI; } };
BCX_LIMITS(int8_t, INT8_MIN, INT8_MAX)
BCX_LIMITS(uint8_t, 0, UINT8_MAX)
BCX_LIMITS(int16_t, INT16_MIN, INT16_MAX)
BCX_LIMITS(uint16_t, 0, UINT16_MAX)
BCX_LIMITS(int32_t, INT32_MIN, INT32_MAX)
BCX_LIMITS(uint32_t, 0u, UINT32_MAX)
BCX_LIMITS(long long, LLONG_MIN, LLONG_MAX)
BCX_LIMITS(unsigned long long, 0ull, ULLONG_MAX)
BCX_LIMITS(float, -INFINITY, INFINITY)
BCX_LIMITS(double, -(double)INFINITY, (double)INFINITY)
#undef BCX_LIMITS
template <class T> struct op_min {
  // OpenCL min(a, b) semantics for integers; fmin-style for floats (a NaN
  // operand yields the other operand).
  __device__ __forceinline__ T operator()(T a, T b) const {
    if (type_traits<T>::is_float) return (b < a || a != a) ? b : a;
    return b < a ? b : a;
  }
  __device__ __forceinline__ static T identity() { return num_limits<T>::highest(); }
};
template <class T> struct op_max {
  __device__ __forceinline__ T operator()(T a, T b) const {
    if (type_traits<T>::is_float) return (b > a || a != a) ? b : a;
    return b > a ? b : a;
  }
  __device__ __forceinline__ static T identity() { return num_limits<T>::lowest(); }
};
template <class T> struct op_bit_and {
  __device__ __forceinline__ T operator()(T a, T b) const { return T(a & b); }
  __device__ __forceinline__ static T identity() { return T(~T(0)); }
};
template <class T> struct op_bit_or {
  __device__ __forceinline__ T operator()(T a, T b) const { return T(a | b); }
  __device__ __forceinline__ static T identity() { return T(0); }
};
template <class T> struct op_bit_xor {
  __device__ __forceinline__ T operator()(T a, T b) const { return T(a ^ b); }
  __device__ __forceinline__ static T identity() { return T(0); }
};

// Integer arithmetic wraps modulo 2^bits exactly like the OpenCL kernels do;
// 8/16-bit values are combined in 32-bit registers and truncated on store,
// which gives the same residues for plus, multiplies and the bit operations.
template <class T> struct widen { typedef T type; };
template <> struct widen<int8_t> { typedef int32_t type; };
template <> struct widen<uint8_t> { typedef uint32_t type; };
template <> struct widen<int16_t> { typedef int32_t type; };
template <> struct widen<uint16_t> { typedef uint32_t type; };

// ---------------------------------------------------------------------------
// Neumaier-compensated FP32 pair: value = s + c with |c| << |s|.
struct comp_f32 {
  float s, c;
};
__device__ __forceinline__ comp_f32 comp_add(comp_f32 a, float x) {
  float t = a.s + x;
  float e = (fabsf(a.s) >= fabsf(x)) ? ((a.s - t) + x) : ((x - t) + a.s);
  return comp_f32{t, a.c + e};
}
__device__ __forceinline__ comp_f32 comp_merge(comp_f32 a, comp_f32 b) {
  float t = a.s + b.s;
  float e = (fabsf(a.s) >= fabsf(b.s)) ? ((a.s - t) + b.s) : ((b.s - t) + a.s);
  return comp_f32{t, (a.c + b.c) + e};
}
struct comp_f64 {
  double s, c;
};
__device__ __forceinline__ comp_f64 comp_add(comp_f64 a, double x) {
  double t = a.s + x;
  double e = (fabs(a.s) >= fabs(x)) ? ((a.s - t) + x) : ((x - t) + a.s);
  return comp_f64{t, a.c + e};
}
__device__ __forceinline__ comp_f64 comp_merge(comp_f64 a, comp_f64 b) {
  double t = a.s + b.s;
  double e = (fabs(a.s) >= fabs(b.s)) ? ((a.s - t) + b.s) : ((b.s - t) + a.s);
  return comp_f64{t, (a.c + b.c) + e};
}

// ---------------------------------------------------------------------------
// Warp helpers.
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <class T>
__device__ __forceinline__ T shfl_up(T v, int d) {
  if (sizeof(T) <= 4) {
    return __shfl_up_sync(0xffffffffu, v, d);
  } else {
    return __shfl_up_sync(0xffffffffu, v, d);
  }
}

// Acquire/release accessors for look-back status words (PTX memory model,
// gpu scope): a status word is published with st.release after its payload
// and read with ld.acquire before the payload.
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Every spin-wait on another block's status is bounded: after kSpinLimit polls
// (with nanosleep back-off, several seconds in total) the waiter records
// BCX_DEVICE_TIMEOUT in the library's error word and carries on with what it
// has, so a kernel always terminates and the host sees the failure through
// bcx_device_error_check().
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr uint32_t kErrLookbackTimeout = 1u;
// A bulk copy into shared memory did not complete within kSpinLimit polls.
constexpr uint32_t kErrCopyTimeout = 2u;

__device__ __forceinline__ void report_error(uint32_t *err, uint32_t code) {
  if (err) atomicOr(err, code);
}

// ---------------------------------------------------------------------------
// Vectorised (16-byte) access helpers.
template <class T> struct alignas(16) vec16 {
  static constexpr int N = 16 / sizeof(T);
  T v[N];
};

// 16-byte load with the evict-first (streaming) hint, for data read once.
template <class T>
__device__ __forceinline__ vec16<T> ld_stream16(const vec16<T> *p) {
  uint4 u = __ldcs(reinterpret_cast<const uint4 *>(p));
  vec16<T> r;
  static_assert(sizeof(r) == sizeof(u), "vec16 is 16 bytes");
  memcpy(&r, &u, 16);
  return r;
}
template <class T>
__device__ __forceinline__ void st_stream16(vec16<T> *p, const vec16<T> &v) {
  uint4 u;
  memcpy(&u, &v, 16);
  __stcs(reinterpret_cast<uint4 *>(p), u);
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, 1-D form) into shared memory, completed on an
// mbarrier.  A copy must start on a 16-byte boundary and move a multiple of 16
// bytes.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load_smem(void *dst, const void *src, uint32_t bytes,
                                               unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// Bulk prefetch of global memory into L2 (no completion to wait for).  Same
// rules: 16-byte aligned start, a multiple of 16 bytes.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
// Distance, in input bytes, at which the two-read tiled kernels (segmented
// scan, reduce_by_key) ask L2 to prefetch the tile they will reach later: far
// enough that the prefetch has landed when that tile's block starts, near
// enough that it is still in L2 then -- with tens of MB of input already in
// flight across the resident blocks, a short distance.  Measured on GB300
// over 9.5e8 elements in 10,000 segments: segmented scan 1.66 ms at 8 MB,
// 1.62 ms at 1 MB; reduce_by_key 2.16 ms at 8 MB, 2.11 ms at 1 MB, 2.22 ms at
// 16 MB, 2.15 ms without prefetch.
constexpr size_t kL2PrefetchBytes = size_t(1) << 20;
// Asks L2 to prefetch elements [first, first + count) of p, clipped to n.
// p + first must be 16-byte aligned.
template <class T>
__device__ __forceinline__ void prefetch_l2_range(const T *p, size_t first, size_t count, size_t n) {
  if (first >= n) return;
  const size_t m = (n - first) < count ? (n - first) : count;
  const uint32_t bytes = uint32_t(m * sizeof(T)) & ~15u;
  const char *src = reinterpret_cast<const char *>(p + first);
  for (uint32_t off = 0; off < bytes; off += 16384u)
    bulk_prefetch_l2(src + off, (bytes - off) < 16384u ? (bytes - off) : 16384u);
}
// Bulk copy from shared memory to global memory, tracked by bulk groups: the
// issuing thread commits the group and waits until the copy has finished
// reading shared memory before that memory may be released or rewritten.
__device__ __forceinline__ void bulk_store_global(void *dst, const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
// Per-thread asynchronous copy of BYTES (4, 8 or 16; both addresses aligned to
// BYTES) from global into shared memory, bypassing registers.  The thread
// waits for all of its copies with cp_async_wait_all(); a block barrier after
// that wait makes them visible to the other threads.
template <int BYTES>
__device__ __forceinline__ void cp_async_smem(void *dst, const void *src) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async moves 4, 8 or 16 bytes");
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src), "n"(BYTES)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void bulk_commit_group() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_group_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Bounded wait for phase `parity` of `bar`; false if the limit was reached.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity,
                                                  uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__host__ __device__ __forceinline__ size_t div_up(size_t a, size_t b) { return (a + b - 1) / b; }

}  // namespace bcx
