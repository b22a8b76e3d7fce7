// bcx_reduce.cu -- reduce / accumulate.
//
// Reference: reduce(first, last, result, op) (algorithm/reduce.hpp:205-305)
// runs reduce_on_gpu for plus (detail/reduce_on_gpu.hpp:169-280: VPT=8 strided
// scalar loads, a 128-wide local tree, ping/pong passes while count > 1024) and
// generic_reduce for other functors (reduce.hpp:37-203: block_reduce +
// inplace_reduce).  accumulate (accumulate.hpp:102-188) uses reduce for
// integer plus/multiplies/min/max with an identity init and a single
// work-item loop (serial_accumulate.hpp:33-49) for everything else.
//
// GB300 design: one pass over HBM.  Kernel 1 runs a fixed grid (blocks per SM
// x SM count) whose threads stream 16-byte vectors with four loads in flight,
// fold them in registers, then reduce through warp shuffles and one shared
// memory step into one partial per block.  Kernel 2 (one block) folds the
// partials in block order and applies init.  Inputs that fit one block's share
// run as a single launch.  The grid depends only on n and the SM count, so the
// association order -- and therefore a float result -- is reproducible run to
// run.  Integers are exact modulo 2^bits whatever the order.  For float plus
// with compensated=1 every thread keeps a Neumaier (s, c) pair, warps and
// blocks merge pairs with TwoSum, and the block partials are combined in FP64.
// Non-associative functors (minus, divides, modulus) are folded left to right
// by one thread, exactly like serial_accumulate.
#include <cuda_runtime.h>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"

namespace bcx {
namespace {

constexpr int kReduceThreads = 256;
constexpr int kUnroll = 4;

// ---- accumulator policies -------------------------------------------------
// Plain: fold in the (widened) element type with the functor.
template <class T, template <class> class OpT>
struct PlainAcc {
  typedef typename widen<T>::type A;
  typedef A Partial;
  typedef OpT<A> Op;
  A v;
  __device__ __forceinline__ void init() { v = Op::identity(); }
  __device__ __forceinline__ void add(T x) { v = Op()(v, A(x)); }
  __device__ __forceinline__ void merge(const PlainAcc &o) { v = Op()(v, o.v); }
  __device__ __forceinline__ PlainAcc shfl_xor(int m) const {
    PlainAcc r;
    r.v = __shfl_xor_sync(0xffffffffu, v, m);
    return r;
  }
  __device__ __forceinline__ Partial partial() const { return v; }
  __device__ __forceinline__ static Partial partial_identity() { return Op::identity(); }
  __device__ __forceinline__ static Partial partial_merge(Partial a, Partial b) { return Op()(a, b); }
  __device__ __forceinline__ static T finish(Partial p, const T *init) {
    return init ? T(Op()(A(*init), p)) : T(p);
  }
};

// Compensated FP32 plus: Neumaier pairs in registers/warps/blocks, FP64
// partials.
struct CompF32Acc {
  typedef double Partial;
  comp_f32 v;
  __device__ __forceinline__ void init() { v = comp_f32{0.f, 0.f}; }
  __device__ __forceinline__ void add(float x) { v = comp_add(v, x); }
  __device__ __forceinline__ void merge(const CompF32Acc &o) { v = comp_merge(v, o.v); }
  __device__ __forceinline__ CompF32Acc shfl_xor(int m) const {
    CompF32Acc r;
    r.v.s = __shfl_xor_sync(0xffffffffu, v.s, m);
    r.v.c = __shfl_xor_sync(0xffffffffu, v.c, m);
    return r;
  }
  __device__ __forceinline__ Partial partial() const { return double(v.s) + double(v.c); }
  __device__ __forceinline__ static Partial partial_identity() { return 0.0; }
  __device__ __forceinline__ static Partial partial_merge(Partial a, Partial b) { return a + b; }
  __device__ __forceinline__ static float finish(Partial p, const float *init) {
    return init ? float(double(*init) + p) : float(p);
  }
};

struct CompF64Acc {
  typedef comp_f64 Partial;
  comp_f64 v;
  __device__ __forceinline__ void init() { v = comp_f64{0.0, 0.0}; }
  __device__ __forceinline__ void add(double x) { v = comp_add(v, x); }
  __device__ __forceinline__ void merge(const CompF64Acc &o) { v = comp_merge(v, o.v); }
  __device__ __forceinline__ CompF64Acc shfl_xor(int m) const {
    CompF64Acc r;
    r.v.s = __shfl_xor_sync(0xffffffffu, v.s, m);
    r.v.c = __shfl_xor_sync(0xffffffffu, v.c, m);
    return r;
  }
  __device__ __forceinline__ Partial partial() const { return v; }
  __device__ __forceinline__ static Partial partial_identity() { return comp_f64{0.0, 0.0}; }
  __device__ __forceinline__ static Partial partial_merge(Partial a, Partial b) { return comp_merge(a, b); }
  __device__ __forceinline__ static double finish(Partial p, const double *init) {
    comp_f64 r = p;
    if (init) r = comp_add(r, *init);
    return r.s + r.c;
  }
};

template <class P> struct partial_shfl {
  __device__ __forceinline__ static P xor_(P v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
};
template <> struct partial_shfl<comp_f64> {
  __device__ __forceinline__ static comp_f64 xor_(comp_f64 v, int m) {
    return comp_f64{__shfl_xor_sync(0xffffffffu, v.s, m), __shfl_xor_sync(0xffffffffu, v.c, m)};
  }
};

// Block-wide fold of one accumulator per thread; the result is valid in
// thread 0.
template <class Acc>
__device__ __forceinline__ Acc block_fold(Acc a) {
  __shared__ Acc warp_acc[kReduceThreads / kWarp];
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) a.merge(a.shfl_xor(m));
  const int w = threadIdx.x / kWarp;
  if (lane_id() == 0) warp_acc[w] = a;
  __syncthreads();
  if (w == 0) {
    Acc b;
    if (lane_id() < kReduceThreads / kWarp) b = warp_acc[lane_id()];
    else b.init();
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) b.merge(b.shfl_xor(m));
    a = b;
  }
  return a;
}

// Kernel 1: every block folds a strided share of the 16-byte vectors plus any
// unaligned head/tail elements, and writes one partial (or, with a single
// block, the final value).
template <class T, class Acc, bool FINAL>
__global__ void __launch_bounds__(kReduceThreads)
reduce_partials_kernel(const T *__restrict__ in, size_t n, size_t head, size_t nvec,
                       typename Acc::Partial *__restrict__ partials, T *__restrict__ out,
                       const T init_value, int has_init) {
  constexpr int N = 16 / sizeof(T);
  typedef vec16<T> V;
  Acc acc;
  acc.init();
  const size_t gtid = size_t(blockIdx.x) * kReduceThreads + threadIdx.x;
  const size_t stride = size_t(gridDim.x) * kReduceThreads;
  // Unaligned head and tail (fewer than 2N scalars unless the pointer is not
  // even element-aligned, in which case everything takes this path).
  const size_t tail_start = head + nvec * N;
  for (size_t i = gtid; i < head; i += stride) acc.add(in[i]);
  for (size_t i = tail_start + gtid; i < n; i += stride) acc.add(in[i]);
  const V *vin = reinterpret_cast<const V *>(in + head);
  size_t v = gtid;
  for (; v + (kUnroll - 1) * stride < nvec; v += kUnroll * stride) {
    V r[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) r[u] = ld_stream16(&vin[v + u * stride]);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int k = 0; k < N; ++k) acc.add(r[u].v[k]);
  }
  for (; v < nvec; v += stride) {
    V r = ld_stream16(&vin[v]);
#pragma unroll
    for (int k = 0; k < N; ++k) acc.add(r.v[k]);
  }
  acc = block_fold(acc);
  if (threadIdx.x == 0) {
    if (FINAL) {
      out[0] = Acc::finish(acc.partial(), has_init ? &init_value : nullptr);
    } else {
      partials[blockIdx.x] = acc.partial();
    }
  }
}

// Kernel 2: one block folds the partials in block order and applies init.
template <class T, class Acc>
__global__ void __launch_bounds__(kReduceThreads)
reduce_final_kernel(const typename Acc::Partial *__restrict__ partials, int count,
                    T *__restrict__ out, const T init_value, int has_init) {
  typedef typename Acc::Partial P;
  __shared__ P sp[kReduceThreads / kWarp];
  P p = Acc::partial_identity();
  for (int i = threadIdx.x; i < count; i += kReduceThreads) p = Acc::partial_merge(p, partials[i]);
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) p = Acc::partial_merge(p, partial_shfl<P>::xor_(p, m));
  if (lane_id() == 0) sp[threadIdx.x / kWarp] = p;
  __syncthreads();
  if (threadIdx.x == 0) {
    P r = sp[0];
    for (int w = 1; w < kReduceThreads / kWarp; ++w) r = Acc::partial_merge(r, sp[w]);
    out[0] = Acc::finish(r, has_init ? &init_value : nullptr);
  }
}

// Left-to-right fold by one thread for functors that are not associative
// (serial_accumulate.hpp:33-49).
template <class T, int OP>
__global__ void serial_fold_kernel(const T *__restrict__ in, size_t n, T *__restrict__ out,
                                   const T init_value) {
  typedef typename widen<T>::type A;
  A r = A(init_value);
  for (size_t i = 0; i < n; ++i) {
    A x = A(in[i]);
    if (OP == BCX_MINUS) r = A(r - x);
    else r = A(r / x);
  }
  out[0] = T(r);
}

struct ReducePlan {
  size_t head = 0, nvec = 0;
  int blocks = 1;
  bool single = true;
};

template <class T>
ReducePlan plan_reduce(const void *in, size_t n, int sm_count) {
  constexpr int N = 16 / sizeof(T);
  ReducePlan p;
  uintptr_t a = reinterpret_cast<uintptr_t>(in);
  size_t mis = (a & 15u) ? (16u - (a & 15u)) / sizeof(T) : 0;
  if ((a % sizeof(T)) != 0) mis = n;  // unaligned element pointer: scalar path only
  p.head = mis < n ? mis : n;
  p.nvec = (n - p.head) / N;
  const size_t per_block = size_t(kReduceThreads) * N * kUnroll * 2;
  size_t want = div_up(n, per_block);
  size_t cap = size_t(sm_count) * 4;
  p.blocks = int(want < 1 ? 1 : (want > cap ? cap : want));
  p.single = (p.blocks == 1);
  return p;
}

template <class T, class Acc>
bcx_status run_reduce_t(cudaStream_t s, const void *in, size_t n, void *out, const void *init,
                        void *temp, size_t *temp_bytes) {
  DeviceState *st = nullptr;
  bcx_status rc = current_device_state(&st);
  if (rc) return rc;
  ReducePlan p = plan_reduce<T>(in, n, st->sm_count);
  size_t need = p.single ? 0 : align256(sizeof(typename Acc::Partial) * p.blocks);
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, need, s, &query);
  if (rc || query) return rc;
  T init_value = init ? *static_cast<const T *>(init) : T(0);
  int has_init = init ? 1 : 0;
  if (p.single) {
    KernelScope ks("reduce_single", s);
    reduce_partials_kernel<T, Acc, true><<<1, kReduceThreads, 0, s>>>(
        static_cast<const T *>(in), n, p.head, p.nvec, nullptr, static_cast<T *>(out),
        init_value, has_init);
    return launch_status("reduce_single");
  }
  typedef typename Acc::Partial P;
  P *partials = static_cast<P *>(ts.ptr());
  {
    KernelScope ks("reduce_partials", s);
    reduce_partials_kernel<T, Acc, false><<<p.blocks, kReduceThreads, 0, s>>>(
        static_cast<const T *>(in), n, p.head, p.nvec, partials, nullptr, init_value, has_init);
    rc = launch_status("reduce_partials");
    if (rc) return rc;
  }
  KernelScope ks("reduce_final", s);
  reduce_final_kernel<T, Acc><<<1, kReduceThreads, 0, s>>>(partials, p.blocks,
                                                           static_cast<T *>(out), init_value,
                                                           has_init);
  return launch_status("reduce_final");
}

template <class T>
bcx_status run_serial_fold(cudaStream_t s, int op, const void *in, size_t n, void *out,
                           const void *init) {
  T init_value = init ? *static_cast<const T *>(init) : T(0);
  KernelScope ks("serial_fold", s);
  const T *pin = static_cast<const T *>(in);
  T *pout = static_cast<T *>(out);
  if (op == BCX_MINUS) serial_fold_kernel<T, BCX_MINUS><<<1, 1, 0, s>>>(pin, n, pout, init_value);
  else if (op == BCX_DIVIDES) serial_fold_kernel<T, BCX_DIVIDES><<<1, 1, 0, s>>>(pin, n, pout, init_value);
  else return BCX_UNSUPPORTED;
  return launch_status("serial_fold");
}

template <class T>
bcx_status dispatch_int(cudaStream_t s, int op, const void *in, size_t n, void *out,
                        const void *init, void *temp, size_t *tb) {
  switch (op) {
    case BCX_PLUS: return run_reduce_t<T, PlainAcc<T, op_plus>>(s, in, n, out, init, temp, tb);
    case BCX_MULTIPLIES: return run_reduce_t<T, PlainAcc<T, op_multiplies>>(s, in, n, out, init, temp, tb);
    case BCX_MIN: return run_reduce_t<T, PlainAcc<T, op_min>>(s, in, n, out, init, temp, tb);
    case BCX_MAX: return run_reduce_t<T, PlainAcc<T, op_max>>(s, in, n, out, init, temp, tb);
    case BCX_BIT_AND: return run_reduce_t<T, PlainAcc<T, op_bit_and>>(s, in, n, out, init, temp, tb);
    case BCX_BIT_OR: return run_reduce_t<T, PlainAcc<T, op_bit_or>>(s, in, n, out, init, temp, tb);
    case BCX_BIT_XOR: return run_reduce_t<T, PlainAcc<T, op_bit_xor>>(s, in, n, out, init, temp, tb);
  }
  return BCX_UNSUPPORTED;
}

template <class T>
bcx_status dispatch_float(cudaStream_t s, int op, const void *in, size_t n, void *out,
                          const void *init, int compensated, void *temp, size_t *tb) {
  switch (op) {
    case BCX_PLUS:
      if (compensated) {
        if (sizeof(T) == 4) return run_reduce_t<float, CompF32Acc>(s, in, n, out, init, temp, tb);
        return run_reduce_t<double, CompF64Acc>(s, in, n, out, init, temp, tb);
      }
      return run_reduce_t<T, PlainAcc<T, op_plus>>(s, in, n, out, init, temp, tb);
    case BCX_MULTIPLIES: return run_reduce_t<T, PlainAcc<T, op_multiplies>>(s, in, n, out, init, temp, tb);
    case BCX_MIN: return run_reduce_t<T, PlainAcc<T, op_min>>(s, in, n, out, init, temp, tb);
    case BCX_MAX: return run_reduce_t<T, PlainAcc<T, op_max>>(s, in, n, out, init, temp, tb);
  }
  return BCX_UNSUPPORTED;
}

bcx_status reduce_entry(cudaStream_t s, bcx_dtype type, bcx_op op, const void *in, size_t n,
                        const void *init, void *out, int compensated, void *temp,
                        size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  const bool serial = (op == BCX_MINUS || op == BCX_DIVIDES);
  if (temp == nullptr && temp_bytes != nullptr) {
    if (n == 0 || serial) {
      *temp_bytes = 0;
      return BCX_SUCCESS;
    }
  }
  if (n == 0) {
    // reduce() of an empty range writes nothing (reduce.hpp:291-296);
    // accumulate() returns init (accumulate.hpp:108-111).
    if (init) BCX_CUDA(cudaMemcpyAsync(out, init, dtype_size(type), cudaMemcpyHostToDevice, s));
    return BCX_SUCCESS;
  }
  BCX_CHECK(in != nullptr && out != nullptr, BCX_INVALID_VALUE, "NULL input or output");
  if (serial) {
    BCX_CHECK(init != nullptr, BCX_INVALID_VALUE, "%s needs an init value",
              op == BCX_MINUS ? "minus" : "divides");
    switch (type) {
      case BCX_CHAR: return run_serial_fold<int8_t>(s, op, in, n, out, init);
      case BCX_UCHAR: return run_serial_fold<uint8_t>(s, op, in, n, out, init);
      case BCX_SHORT: return run_serial_fold<int16_t>(s, op, in, n, out, init);
      case BCX_USHORT: return run_serial_fold<uint16_t>(s, op, in, n, out, init);
      case BCX_INT: return run_serial_fold<int32_t>(s, op, in, n, out, init);
      case BCX_UINT: return run_serial_fold<uint32_t>(s, op, in, n, out, init);
      case BCX_LONG: return run_serial_fold<long long>(s, op, in, n, out, init);
      case BCX_ULONG: return run_serial_fold<unsigned long long>(s, op, in, n, out, init);
      case BCX_FLOAT: return run_serial_fold<float>(s, op, in, n, out, init);
      case BCX_DOUBLE: return run_serial_fold<double>(s, op, in, n, out, init);
    }
  }
  bcx_status rc = BCX_UNSUPPORTED;
  switch (type) {
    case BCX_CHAR: rc = dispatch_int<int8_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_UCHAR: rc = dispatch_int<uint8_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_SHORT: rc = dispatch_int<int16_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_USHORT: rc = dispatch_int<uint16_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_INT: rc = dispatch_int<int32_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_UINT: rc = dispatch_int<uint32_t>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_LONG: rc = dispatch_int<long long>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_ULONG: rc = dispatch_int<unsigned long long>(s, op, in, n, out, init, temp, temp_bytes); break;
    case BCX_FLOAT: rc = dispatch_float<float>(s, op, in, n, out, init, compensated, temp, temp_bytes); break;
    case BCX_DOUBLE: rc = dispatch_float<double>(s, op, in, n, out, init, compensated, temp, temp_bytes); break;
  }
  if (rc == BCX_UNSUPPORTED) set_error("reduce: functor %d not provided for dtype %d", int(op), int(type));
  return rc;
}

}  // namespace
}  // namespace bcx

extern "C" {

bcx_status bcx_reduce(bcx_stream stream, bcx_dtype type, bcx_op op, const void *in, size_t n,
                      void *out_dev, int compensated, void *temp, size_t *temp_bytes) {
  BCX_CHECK(op != BCX_MINUS && op != BCX_DIVIDES && op != BCX_MODULUS, BCX_INVALID_VALUE,
            "reduce needs an associative functor");
  return bcx::reduce_entry((cudaStream_t)stream, type, op, in, n, nullptr, out_dev, compensated,
                           temp, temp_bytes);
}

bcx_status bcx_accumulate(bcx_stream stream, bcx_dtype type, bcx_op op, const void *in,
                          size_t n, const void *init, void *out_dev, int compensated, void *temp,
                          size_t *temp_bytes) {
  BCX_CHECK(init != nullptr, BCX_INVALID_VALUE, "accumulate needs an init value");
  BCX_CHECK(op != BCX_MODULUS, BCX_UNSUPPORTED, "accumulate: modulus not provided");
  return bcx::reduce_entry((cudaStream_t)stream, type, op, in, n, init, out_dev, compensated,
                           temp, temp_bytes);
}

}  // extern "C"
