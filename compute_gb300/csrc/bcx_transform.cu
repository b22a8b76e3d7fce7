// bcx_transform.cu -- transform with built-in functors.
//
// Reference: transform(first, last, result, f) is copy(transform_iterator)
// (algorithm/transform.hpp:38-82); the binary form zips both inputs and
// unpacks the functor.  On a GPU, copy_on_device_gpu
// (algorithm/detail/copy_on_device.hpp:60-92) emits a kernel where each
// work-item handles VPT=4 elements at a stride of TPB=128, with scalar loads.
//
// GB300 design: a grid of (blocks per SM x SM count) threads striding over
// 16-byte vectors with two vectors per operand in flight; inputs are read with
// the evict-first hint and results stored the same way (data touched once).
// The functor is a template parameter, so the loop body is the functor's
// arithmetic and nothing else.  A pointer whose 16-byte phase differs from the
// output's falls back to the scalar loop (still coalesced).  saxpy computes
// fma(alpha, x, y) with a single rounding (what nvcc's default contraction of
// alpha * x + y produces).
#include <cuda_runtime.h>

#include <math.h>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"

namespace bcx {
namespace {

constexpr int kTfThreads = 256;

template <class T> struct u_identity { __device__ T operator()(T x) const { return x; } };
template <class T> struct u_negate { __device__ T operator()(T x) const { return T(-x); } };
template <class T> struct u_abs {
  __device__ T operator()(T x) const { return (type_traits<T>::is_signed && x < T(0)) ? T(-x) : x; }
};
template <> struct u_abs<float> { __device__ float operator()(float x) const { return fabsf(x); } };
template <> struct u_abs<double> { __device__ double operator()(double x) const { return fabs(x); } };
template <class T> struct u_sqrt { __device__ T operator()(T x) const { return T(sqrt(double(x))); } };
template <> struct u_sqrt<float> { __device__ float operator()(float x) const { return sqrtf(x); } };
template <class T> struct u_lnot { __device__ T operator()(T x) const { return T(!x); } };
template <class T> struct u_bnot { __device__ T operator()(T x) const { return T(~x); } };

template <class T> struct b_plus { __device__ T operator()(T a, T b) const { return T(a + b); } };
template <class T> struct b_minus { __device__ T operator()(T a, T b) const { return T(a - b); } };
template <class T> struct b_mul { __device__ T operator()(T a, T b) const { return T(a * b); } };
template <class T> struct b_div { __device__ T operator()(T a, T b) const { return T(a / b); } };
template <class T> struct b_mod { __device__ T operator()(T a, T b) const { return T(a % b); } };
template <class T> struct b_min { __device__ T operator()(T a, T b) const { return op_min<T>()(a, b); } };
template <class T> struct b_max { __device__ T operator()(T a, T b) const { return op_max<T>()(a, b); } };
template <class T> struct b_and { __device__ T operator()(T a, T b) const { return T(a & b); } };
template <class T> struct b_or { __device__ T operator()(T a, T b) const { return T(a | b); } };
template <class T> struct b_xor { __device__ T operator()(T a, T b) const { return T(a ^ b); } };
template <class T> struct b_saxpy {
  T alpha;
  __device__ T operator()(T x, T y) const { return fma(alpha, x, y); }
};
template <> struct b_saxpy<float> {
  float alpha;
  __device__ float operator()(float x, float y) const { return fmaf(alpha, x, y); }
};

// out[i] = f(in0[i]) or f(in0[i], in1[i]); head_pad aligns the 16-byte phase.
template <class T, class F, bool BINARY>
__global__ void __launch_bounds__(kTfThreads)
transform_kernel(const T *__restrict__ in0, const T *__restrict__ in1, T *__restrict__ out,
                 size_t n, size_t head, int vec_ok, F f) {
  constexpr int N = 16 / sizeof(T);
  const size_t gtid = size_t(blockIdx.x) * kTfThreads + threadIdx.x;
  const size_t stride = size_t(gridDim.x) * kTfThreads;
  if (!vec_ok) {
    for (size_t i = gtid; i < n; i += stride) {
      if constexpr (BINARY) out[i] = f(in0[i], in1[i]);
      else out[i] = f(in0[i]);
    }
    return;
  }
  for (size_t i = gtid; i < head; i += stride) {
    if constexpr (BINARY) out[i] = f(in0[i], in1[i]);
    else out[i] = f(in0[i]);
  }
  const size_t nvec = (n - head) / N;
  const size_t tail = head + nvec * N;
  for (size_t i = tail + gtid; i < n; i += stride) {
    if constexpr (BINARY) out[i] = f(in0[i], in1[i]);
    else out[i] = f(in0[i]);
  }
  const vec16<T> *a = reinterpret_cast<const vec16<T> *>(in0 + head);
  const vec16<T> *b = reinterpret_cast<const vec16<T> *>(in1 + head);
  vec16<T> *o = reinterpret_cast<vec16<T> *>(out + head);
  size_t v = gtid;
  for (; v + stride < nvec; v += 2 * stride) {
    vec16<T> x0 = ld_stream16(a + v), x1 = ld_stream16(a + v + stride);
    vec16<T> y0, y1;
    if constexpr (BINARY) {
      y0 = ld_stream16(b + v);
      y1 = ld_stream16(b + v + stride);
    }
    vec16<T> r0, r1;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      if constexpr (BINARY) {
        r0.v[k] = f(x0.v[k], y0.v[k]);
        r1.v[k] = f(x1.v[k], y1.v[k]);
      } else {
        r0.v[k] = f(x0.v[k]);
        r1.v[k] = f(x1.v[k]);
      }
    }
    st_stream16(o + v, r0);
    st_stream16(o + v + stride, r1);
  }
  for (; v < nvec; v += stride) {
    vec16<T> x0 = ld_stream16(a + v), y0;
    if constexpr (BINARY) y0 = ld_stream16(b + v);
    vec16<T> r0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      if constexpr (BINARY) r0.v[k] = f(x0.v[k], y0.v[k]);
      else r0.v[k] = f(x0.v[k]);
    }
    st_stream16(o + v, r0);
  }
}

template <class T, class F, bool BINARY>
bcx_status launch_transform(cudaStream_t s, const void *in0, const void *in1, void *out, size_t n,
                            F f, const char *name) {
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(in0), ao = reinterpret_cast<uintptr_t>(out);
  const uintptr_t a1 = BINARY ? reinterpret_cast<uintptr_t>(in1) : a0;
  bool vec_ok = (a0 % sizeof(T) == 0) && (ao % sizeof(T) == 0) && (a1 % sizeof(T) == 0) &&
                ((a0 & 15u) == (ao & 15u)) && ((a1 & 15u) == (ao & 15u));
  size_t head = vec_ok ? (((16u - (ao & 15u)) & 15u) / sizeof(T)) : 0;
  if (head > n) head = n;
  constexpr int N = 16 / sizeof(T);
  size_t work = div_up(n, size_t(N) * 2);
  size_t blocks = div_up(work, kTfThreads);
  size_t cap = size_t(ds->sm_count) * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  KernelScope ks(name, s);
  transform_kernel<T, F, BINARY><<<unsigned(blocks), kTfThreads, 0, s>>>(
      static_cast<const T *>(in0), static_cast<const T *>(in1), static_cast<T *>(out), n, head,
      vec_ok ? 1 : 0, f);
  return launch_status(name);
}

template <class T>
bcx_status unary_t(cudaStream_t s, int op, const void *in, void *out, size_t n) {
  switch (op) {
    case BCX_IDENTITY: return launch_transform<T, u_identity<T>, false>(s, in, nullptr, out, n, u_identity<T>(), "transform_unary");
    case BCX_NEGATE: return launch_transform<T, u_negate<T>, false>(s, in, nullptr, out, n, u_negate<T>(), "transform_unary");
    case BCX_ABS: return launch_transform<T, u_abs<T>, false>(s, in, nullptr, out, n, u_abs<T>(), "transform_unary");
    case BCX_SQRT:
      if constexpr (type_traits<T>::is_float)
        return launch_transform<T, u_sqrt<T>, false>(s, in, nullptr, out, n, u_sqrt<T>(), "transform_unary");
      return BCX_UNSUPPORTED;
    case BCX_LOGICAL_NOT: return launch_transform<T, u_lnot<T>, false>(s, in, nullptr, out, n, u_lnot<T>(), "transform_unary");
  }
  return BCX_UNSUPPORTED;
}
template <class T>
bcx_status unary_int_t(cudaStream_t s, int op, const void *in, void *out, size_t n) {
  if (op == BCX_BIT_NOT) return launch_transform<T, u_bnot<T>, false>(s, in, nullptr, out, n, u_bnot<T>(), "transform_unary");
  if (op == BCX_SQRT) return BCX_UNSUPPORTED;
  return unary_t<T>(s, op, in, out, n);
}

template <class T>
bcx_status binary_common_t(cudaStream_t s, int op, const void *a, const void *b, void *out, size_t n) {
  switch (op) {
    case BCX_PLUS: return launch_transform<T, b_plus<T>, true>(s, a, b, out, n, b_plus<T>(), "transform_binary");
    case BCX_MINUS: return launch_transform<T, b_minus<T>, true>(s, a, b, out, n, b_minus<T>(), "transform_binary");
    case BCX_MULTIPLIES: return launch_transform<T, b_mul<T>, true>(s, a, b, out, n, b_mul<T>(), "transform_binary");
    case BCX_DIVIDES: return launch_transform<T, b_div<T>, true>(s, a, b, out, n, b_div<T>(), "transform_binary");
    case BCX_MIN: return launch_transform<T, b_min<T>, true>(s, a, b, out, n, b_min<T>(), "transform_binary");
    case BCX_MAX: return launch_transform<T, b_max<T>, true>(s, a, b, out, n, b_max<T>(), "transform_binary");
  }
  return BCX_UNSUPPORTED;
}
template <class T>
bcx_status binary_int_t(cudaStream_t s, int op, const void *a, const void *b, void *out, size_t n) {
  switch (op) {
    case BCX_MODULUS: return launch_transform<T, b_mod<T>, true>(s, a, b, out, n, b_mod<T>(), "transform_binary");
    case BCX_BIT_AND: return launch_transform<T, b_and<T>, true>(s, a, b, out, n, b_and<T>(), "transform_binary");
    case BCX_BIT_OR: return launch_transform<T, b_or<T>, true>(s, a, b, out, n, b_or<T>(), "transform_binary");
    case BCX_BIT_XOR: return launch_transform<T, b_xor<T>, true>(s, a, b, out, n, b_xor<T>(), "transform_binary");
  }
  return binary_common_t<T>(s, op, a, b, out, n);
}

// One block per piece.  Pieces whose ends are 16-byte aligned move in 16-byte
// vectors; 4-byte aligned pieces (a request's elements packed at an arbitrary
// element offset of a batch) in words; anything else in bytes.
__global__ void __launch_bounds__(256) copy_chunks_kernel(const CopyChunk *__restrict__ chunks) {
  const CopyChunk c = chunks[blockIdx.x];
  const uintptr_t a = reinterpret_cast<uintptr_t>(c.src) | reinterpret_cast<uintptr_t>(c.dst) | c.bytes;
  if ((a & 15) == 0) {
    const uint4 *src = static_cast<const uint4 *>(c.src);
    uint4 *dst = static_cast<uint4 *>(c.dst);
    const uint32_t n = uint32_t(c.bytes >> 4);
#pragma unroll 4
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  } else if ((a & 3) == 0) {
    const uint32_t *src = static_cast<const uint32_t *>(c.src);
    uint32_t *dst = static_cast<uint32_t *>(c.dst);
    const uint32_t n = uint32_t(c.bytes >> 2);
#pragma unroll 4
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  } else {
    const unsigned char *src = static_cast<const unsigned char *>(c.src);
    unsigned char *dst = static_cast<unsigned char *>(c.dst);
    for (uint32_t i = threadIdx.x; i < c.bytes; i += blockDim.x) dst[i] = src[i];
  }
}

}  // namespace

bcx_status copy_chunks(const CopyChunk *chunks, size_t count, cudaStream_t s) {
  if (count == 0) return BCX_SUCCESS;
  BCX_CHECK(count <= 0x7fffffffu, BCX_INVALID_VALUE, "too many copy pieces");
  KernelScope ks("copy_chunks", s);
  copy_chunks_kernel<<<unsigned(count), 256, 0, s>>>(chunks);
  return launch_status("copy_chunks");
}

}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_transform_unary(bcx_stream stream, bcx_dtype type, bcx_unary_op op, const void *in,
                               void *out, size_t n) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (n == 0) return BCX_SUCCESS;
  BCX_CHECK(in && out, BCX_INVALID_VALUE, "NULL input or output");
  cudaStream_t s = (cudaStream_t)stream;
  bcx_status rc = BCX_UNSUPPORTED;
#define INT_FN(T) unary_int_t<T>(s, op, in, out, n)
#define FLT_FN(T) unary_t<T>(s, op, in, out, n)
  switch (type) {
    case BCX_CHAR: rc = INT_FN(int8_t); break;
    case BCX_UCHAR: rc = INT_FN(uint8_t); break;
    case BCX_SHORT: rc = INT_FN(int16_t); break;
    case BCX_USHORT: rc = INT_FN(uint16_t); break;
    case BCX_INT: rc = INT_FN(int32_t); break;
    case BCX_UINT: rc = INT_FN(uint32_t); break;
    case BCX_LONG: rc = INT_FN(long long); break;
    case BCX_ULONG: rc = INT_FN(unsigned long long); break;
    case BCX_FLOAT: rc = FLT_FN(float); break;
    case BCX_DOUBLE: rc = FLT_FN(double); break;
  }
#undef INT_FN
#undef FLT_FN
  if (rc == BCX_UNSUPPORTED) set_error("transform: unary functor %d not provided for dtype %d", int(op), int(type));
  return rc;
}

bcx_status bcx_transform_binary(bcx_stream stream, bcx_dtype type, bcx_op op, const void *in0,
                                const void *in1, void *out, size_t n) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (n == 0) return BCX_SUCCESS;
  BCX_CHECK(in0 && in1 && out, BCX_INVALID_VALUE, "NULL input or output");
  cudaStream_t s = (cudaStream_t)stream;
  bcx_status rc = BCX_UNSUPPORTED;
#define INT_FN(T) binary_int_t<T>(s, op, in0, in1, out, n)
#define FLT_FN(T) binary_common_t<T>(s, op, in0, in1, out, n)
  switch (type) {
    case BCX_CHAR: rc = INT_FN(int8_t); break;
    case BCX_UCHAR: rc = INT_FN(uint8_t); break;
    case BCX_SHORT: rc = INT_FN(int16_t); break;
    case BCX_USHORT: rc = INT_FN(uint16_t); break;
    case BCX_INT: rc = INT_FN(int32_t); break;
    case BCX_UINT: rc = INT_FN(uint32_t); break;
    case BCX_LONG: rc = INT_FN(long long); break;
    case BCX_ULONG: rc = INT_FN(unsigned long long); break;
    case BCX_FLOAT: rc = FLT_FN(float); break;
    case BCX_DOUBLE: rc = FLT_FN(double); break;
  }
#undef INT_FN
#undef FLT_FN
  if (rc == BCX_UNSUPPORTED) set_error("transform: binary functor %d not provided for dtype %d", int(op), int(type));
  return rc;
}

bcx_status bcx_transform_saxpy(bcx_stream stream, bcx_dtype type, const void *alpha, const void *x,
                               const void *y, void *out, size_t n) {
  clear_error();
  BCX_CHECK(type == BCX_FLOAT || type == BCX_DOUBLE, BCX_UNSUPPORTED, "saxpy: float or double only");
  BCX_CHECK(alpha != nullptr, BCX_INVALID_VALUE, "alpha is NULL");
  if (n == 0) return BCX_SUCCESS;
  BCX_CHECK(x && y && out, BCX_INVALID_VALUE, "NULL input or output");
  cudaStream_t s = (cudaStream_t)stream;
  if (type == BCX_FLOAT) {
    b_saxpy<float> f{*static_cast<const float *>(alpha)};
    return launch_transform<float, b_saxpy<float>, true>(s, x, y, out, n, f, "transform_saxpy");
  }
  b_saxpy<double> f{*static_cast<const double *>(alpha)};
  return launch_transform<double, b_saxpy<double>, true>(s, x, y, out, n, f, "transform_saxpy");
}

}  // extern "C"
