// bcx_scan.cuh -- exclusive_scan / inclusive_scan as ONE pass over HBM.
//
// Reference: detail::scan_on_gpu (algorithm/detail/scan_on_gpu.hpp:187-324):
// a 256-wide Hillis-Steele scan per work-group in local memory, a recursive
// scan of the block sums, then a uniform-add pass (about three global passes,
// ~12 launches at 2^30).  Exclusive output[0] = init (:59-66); in-place scans
// go through a temporary copy (:281-308).
//
// GB300 design: single-pass decoupled look-back over tiles staged in shared
// memory.  Each 256-thread block takes the next tile from an atomic ticket (so
// a block only ever waits on tiles that were handed out before it, which
// guarantees forward progress) and moves the whole tile (64 KB; 96 KB for
// 8-byte elements) into shared memory with bulk asynchronous copies completed
// on an mbarrier, while asking L2 to prefetch the tile 16 MB further on.  Each
// thread folds its contiguous run of the tile from shared memory, a block scan
// of the run totals gives the tile aggregate, which is published; warp 0 looks
// back over 32 predecessors at a time for the nearest inclusive prefix; each
// thread then rewrites its run in place with its outputs, and bulk copies move
// the tile out.  DRAM sees 8 bytes per element and nothing is re-read.
// In-place scans need no copy: a tile is read whole before any of it is
// written, and other tiles never touch it.
//
// Inputs that fit one tile, and inputs or outputs that are not 16-byte
// aligned (bulk copies need that), take a register-tiled form instead: 16-byte
// loads with lane runs per warp chunk, a first read (cached in L2) that only
// forms per-lane prefixes and the aggregate, and a second read for the
// outputs after the look-back.  Every wait on a predecessor or on a bulk copy
// is bounded (kSpinLimit polls); on expiry the block records a device error
// and finishes.
//
// Float plus with compensated=1 keeps Neumaier (s, c) pairs for every sum
// inside a tile and carries tile prefixes between blocks in FP64.
#ifndef BCX_SCAN_CUH
#define BCX_SCAN_CUH
#include <cuda_runtime.h>

#include <string.h>

#include <map>
#include <mutex>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"

namespace bcx {
// Internal linkage on purpose: each translation unit that includes this header
// instantiates the kernels it dispatches to as its own private copies, so no
// kernel symbol or launch stub is shared between separately compiled device
// images.
namespace {

// Block size of the allocating scan (the no-alloc entry point keeps its own
// fixed shape).
constexpr int kScanThreads = 256;
// 16-byte vectors a lane owns consecutively per chunk (its serial run before
// the chunk's warp scan).
constexpr int kScanRunVectors = 2;

enum : uint32_t { kFlagInvalid = 0, kFlagAggregate = 1, kFlagPrefix = 2 };

// ---- policies --------------------------------------------------------------
template <class T, template <class> class OpT>
struct ScanPlain {
  typedef typename widen<T>::type Acc;
  typedef Acc Carry;
  typedef OpT<Acc> Op;
  __device__ __forceinline__ static Acc ident() { return Op::identity(); }
  __device__ __forceinline__ static Acc add(Acc a, T x) { return Op()(a, Acc(x)); }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return Op()(a, b); }
  __device__ __forceinline__ static Carry to_carry(Acc a) { return a; }
  __device__ __forceinline__ static Acc from_carry(Carry c) { return c; }
  __device__ __forceinline__ static Carry carry_comb(Carry a, Carry b) { return Op()(a, b); }
  __device__ __forceinline__ static Carry carry_ident() { return Op::identity(); }
  __device__ __forceinline__ static T out(Acc a) { return T(a); }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
  __device__ __forceinline__ static Acc shfl(Acc a, int src) { return __shfl_sync(0xffffffffu, a, src); }
  __device__ __forceinline__ static Carry carry_shfl_down(Carry a, int d) {
    return __shfl_down_sync(0xffffffffu, a, d);
  }
  __device__ __forceinline__ static Carry carry_bcast(Carry a) { return __shfl_sync(0xffffffffu, a, 0); }
  static Carry host_carry(const void *init) {
    T v;
    memcpy(&v, init, sizeof(T));
    return Carry(v);
  }
};

struct ScanCompF32 {
  typedef comp_f32 Acc;
  typedef double Carry;
  __device__ __forceinline__ static Acc ident() { return comp_f32{0.f, 0.f}; }
  __device__ __forceinline__ static Acc add(Acc a, float x) { return comp_add(a, x); }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return comp_merge(a, b); }
  __device__ __forceinline__ static Carry to_carry(Acc a) { return double(a.s) + double(a.c); }
  __device__ __forceinline__ static Acc from_carry(Carry c) {
    float hi = float(c);
    return comp_f32{hi, float(c - double(hi))};
  }
  __device__ __forceinline__ static Carry carry_comb(Carry a, Carry b) { return a + b; }
  __device__ __forceinline__ static Carry carry_ident() { return 0.0; }
  __device__ __forceinline__ static float out(Acc a) { return a.s + a.c; }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) {
    return comp_f32{__shfl_up_sync(0xffffffffu, a.s, d), __shfl_up_sync(0xffffffffu, a.c, d)};
  }
  __device__ __forceinline__ static Acc shfl(Acc a, int src) {
    return comp_f32{__shfl_sync(0xffffffffu, a.s, src), __shfl_sync(0xffffffffu, a.c, src)};
  }
  __device__ __forceinline__ static Carry carry_shfl_down(Carry a, int d) {
    return __shfl_down_sync(0xffffffffu, a, d);
  }
  __device__ __forceinline__ static Carry carry_bcast(Carry a) { return __shfl_sync(0xffffffffu, a, 0); }
  static Carry host_carry(const void *init) {
    float v;
    memcpy(&v, init, sizeof(float));
    return double(v);
  }
};

struct ScanCompF64 {
  typedef comp_f64 Acc;
  typedef comp_f64 Carry;
  __device__ __forceinline__ static Acc ident() { return comp_f64{0.0, 0.0}; }
  __device__ __forceinline__ static Acc add(Acc a, double x) { return comp_add(a, x); }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return comp_merge(a, b); }
  __device__ __forceinline__ static Carry to_carry(Acc a) { return a; }
  __device__ __forceinline__ static Acc from_carry(Carry c) { return c; }
  __device__ __forceinline__ static Carry carry_comb(Carry a, Carry b) { return comp_merge(a, b); }
  __device__ __forceinline__ static Carry carry_ident() { return comp_f64{0.0, 0.0}; }
  __device__ __forceinline__ static double out(Acc a) { return a.s + a.c; }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) {
    return comp_f64{__shfl_up_sync(0xffffffffu, a.s, d), __shfl_up_sync(0xffffffffu, a.c, d)};
  }
  __device__ __forceinline__ static Acc shfl(Acc a, int src) {
    return comp_f64{__shfl_sync(0xffffffffu, a.s, src), __shfl_sync(0xffffffffu, a.c, src)};
  }
  __device__ __forceinline__ static Carry carry_shfl_down(Carry a, int d) {
    return comp_f64{__shfl_down_sync(0xffffffffu, a.s, d), __shfl_down_sync(0xffffffffu, a.c, d)};
  }
  __device__ __forceinline__ static Carry carry_bcast(Carry a) {
    return comp_f64{__shfl_sync(0xffffffffu, a.s, 0), __shfl_sync(0xffffffffu, a.c, 0)};
  }
  static Carry host_carry(const void *init) {
    double v;
    memcpy(&v, init, sizeof(double));
    return comp_f64{v, 0.0};
  }
};

// L2-coherent payload loads (issued after an acquire of the flag word).  FP64
// carries need none: they live in self-validating words.
__device__ __forceinline__ long long ldcg(const long long *p) { return __ldcg(p); }
__device__ __forceinline__ unsigned long long ldcg(const unsigned long long *p) { return __ldcg(p); }
__device__ __forceinline__ comp_f64 ldcg(const comp_f64 *p) {
  return comp_f64{__ldcg(&p->s), __ldcg(&p->c)};
}

// ---- tile status -----------------------------------------------------------
// 4-byte carries are packed with their flag into one 64-bit word, published
// and read as a single 64-bit access.  Wider carries use a flag word plus
// separate aggregate/inclusive arrays ordered by release/acquire.
template <class Carry, bool PACKED = (sizeof(Carry) == 4)>
struct TileStatus;

template <class Carry>
struct TileStatus<Carry, true> {
  unsigned long long *words;
  static constexpr size_t bytes(size_t tiles) { return align256(tiles * 8); }
  static size_t zero_bytes(size_t tiles) { return bytes(tiles); }
  void bind(char *base, size_t) { words = reinterpret_cast<unsigned long long *>(base); }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(words, 0, zero_bytes(tiles), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, Carry v) {
    uint32_t bits;
    memcpy(&bits, &v, 4);
    unsigned long long w = (static_cast<unsigned long long>(bits) << 32) | flag;
    // Flag and value travel in one 64-bit word, so relaxed ordering suffices.
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(&words[t]), "l"(w) : "memory");
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Carry *v) const {
    unsigned long long w = ld_relaxed_u64(&words[t]);
    uint32_t bits = uint32_t(w >> 32);
    memcpy(v, &bits, 4);
    return uint32_t(w & 0xffffffffu);
  }
};

template <class Carry>
struct TileStatus<Carry, false> {
  uint32_t *flags;
  Carry *agg;
  Carry *inc;
  static constexpr size_t bytes(size_t tiles) {
    return align256(tiles * 4) + 2 * align256(tiles * sizeof(Carry));
  }
  static size_t zero_bytes(size_t tiles) { return align256(tiles * 4); }
  void bind(char *base, size_t tiles) {
    flags = reinterpret_cast<uint32_t *>(base);
    agg = reinterpret_cast<Carry *>(base + align256(tiles * 4));
    inc = reinterpret_cast<Carry *>(base + align256(tiles * 4) + align256(tiles * sizeof(Carry)));
  }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(flags, 0, zero_bytes(tiles), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, Carry v) {
    if (flag == kFlagAggregate) agg[t] = v;
    else inc[t] = v;
    st_release_u32(&flags[t], flag);
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Carry *v) const {
    uint32_t f = ld_acquire_u32(&flags[t]);
    if (f == kFlagAggregate) *v = ldcg(&agg[t]);
    else if (f == kFlagPrefix) *v = ldcg(&inc[t]);
    return f;
  }
};

// FP64 carries (double scans, compensated float scans): the aggregate and the
// inclusive prefix of a tile each live in one 64-bit word that holds either the
// value or an all-ones bit pattern meaning "not published yet".  All ones is a
// NaN with a full payload, which GPU arithmetic never produces (computed NaNs
// are canonical), and a relaxed 64-bit load returns either the marker or the
// whole value, so no fence has to order a separate flag after the value.
template <>
struct TileStatus<double, false> {
  unsigned long long *agg;
  unsigned long long *inc;
  static constexpr unsigned long long kUnset = ~0ull;
  static constexpr size_t bytes(size_t tiles) { return 2 * align256(tiles * 8); }
  void bind(char *base, size_t tiles) {
    agg = reinterpret_cast<unsigned long long *>(base);
    inc = reinterpret_cast<unsigned long long *>(base + align256(tiles * 8));
  }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(agg, 0xff, bytes(tiles), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, double v) {
    unsigned long long w;
    memcpy(&w, &v, 8);
    unsigned long long *dst = flag == kFlagAggregate ? &agg[t] : &inc[t];
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(dst), "l"(w) : "memory");
  }
  __device__ __forceinline__ uint32_t poll(size_t t, double *v) const {
    const unsigned long long wi = ld_relaxed_u64(&inc[t]);
    const unsigned long long wa = ld_relaxed_u64(&agg[t]);
    if (wi != kUnset) {
      memcpy(v, &wi, 8);
      return kFlagPrefix;
    }
    if (wa != kUnset) {
      memcpy(v, &wa, 8);
      return kFlagAggregate;
    }
    return kFlagInvalid;
  }
};

// Warp 0 of a block: publish this tile's aggregate, look back for the
// exclusive prefix, publish the inclusive prefix.  Lane l watches the
// predecessors pred - l - 32*j for j < kLookbackDepth, all loaded at once, so
// one L2 round trip covers 32 * kLookbackDepth predecessors: the walk back to
// the nearest inclusive prefix stays short even when many tiles are in flight.
// Returns the exclusive prefix (valid in every lane of warp 0).
constexpr int kLookbackDepth = 4;

template <class P, class Status>
__device__ __forceinline__ typename P::Carry lookback(Status &st, size_t tile,
                                                      typename P::Carry agg, uint32_t *err,
                                                      uint32_t limit = kSpinLimit) {
  typedef typename P::Carry C;
  const unsigned lane = lane_id();
  if (lane == 0) st.publish(tile, kFlagAggregate, agg);
  C excl = P::carry_ident();
  long long pred = (long long)tile - 1;
  bool gave_up = false;
  while (true) {
    C v[kLookbackDepth];
    uint32_t f[kLookbackDepth];
#pragma unroll
    for (int j = 0; j < kLookbackDepth; ++j) {
      const long long t = pred - (long long)lane - (long long)kWarp * j;
      v[j] = P::carry_ident();
      f[j] = kFlagPrefix;  // beyond tile 0: nothing to add
      if (t >= 0) f[j] = st.poll(size_t(t), &v[j]);
    }
    bool done = false;
#pragma unroll
    for (int j = 0; j < kLookbackDepth; ++j) {
      if (done) break;
      const long long t = pred - (long long)lane - (long long)kWarp * j;
      uint32_t spins = 0;
      while (f[j] == kFlagInvalid) {
        if (++spins > limit) {
          gave_up = true;
          f[j] = kFlagPrefix;
          v[j] = P::carry_ident();
          break;
        }
        if (spins > 32) __nanosleep(spins < 256 ? 32 : 256);
        f[j] = st.poll(size_t(t), &v[j]);
      }
      const unsigned pmask = __ballot_sync(0xffffffffu, f[j] == kFlagPrefix);
      const int first = pmask ? __ffs(pmask) - 1 : kWarp - 1;
      C w = (int(lane) > first) ? P::carry_ident() : v[j];
      // Lane 0 folds lanes 0..first: this window's predecessors up to the
      // nearest inclusive prefix.
#pragma unroll
      for (int d = 16; d >= 1; d >>= 1) {
        C o = P::carry_shfl_down(w, d);
        if (int(lane) + d < kWarp) w = P::carry_comb(w, o);
      }
      excl = P::carry_comb(P::carry_bcast(w), excl);
      done = pmask != 0;
    }
    if (done) break;
    pred -= (long long)kWarp * kLookbackDepth;
  }
  if (__any_sync(0xffffffffu, gave_up) && lane == 0) report_error(err, kErrLookbackTimeout);
  if (lane == 0) st.publish(tile, kFlagPrefix, P::carry_comb(excl, agg));
  return excl;
}

template <class T>
__device__ __forceinline__ void load_chunk(const T *__restrict__ in, size_t vi, size_t head_pad,
                                           size_t nv, bool vec_ok, T (&x)[16 / sizeof(T)]) {
  constexpr int N = 16 / sizeof(T);
  const size_t u0 = vi * N;
  if (vec_ok && u0 >= head_pad && u0 + N <= nv) {
    vec16<T> r = ld_stream16(reinterpret_cast<const vec16<T> *>(in - head_pad) + vi);
#pragma unroll
    for (int k = 0; k < N; ++k) x[k] = r.v[k];
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const size_t u = u0 + k;
      x[k] = (u >= head_pad && u < nv) ? in[u - head_pad] : T(0);
    }
  }
}

// First read of a chunk: cached in L2 (not L1) so that the second read after
// the look-back hits L2.
template <class T>
__device__ __forceinline__ void load_chunk_l2(const T *__restrict__ in, size_t vi, size_t head_pad,
                                              size_t nv, bool vec_ok, T (&x)[16 / sizeof(T)]) {
  constexpr int N = 16 / sizeof(T);
  const size_t u0 = vi * N;
  if (vec_ok && u0 >= head_pad && u0 + N <= nv) {
    uint4 u = __ldcg(reinterpret_cast<const uint4 *>(reinterpret_cast<const vec16<T> *>(in - head_pad) + vi));
    vec16<T> r;
    memcpy(&r, &u, 16);
#pragma unroll
    for (int k = 0; k < N; ++k) x[k] = r.v[k];
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const size_t u = u0 + k;
      x[k] = (u >= head_pad && u < nv) ? in[u - head_pad] : T(0);
    }
  }
}

// One block = one tile of THREADS * V vectors.
template <class T, class P, int THREADS, int V, bool SINGLE, class Status>
__global__ void __launch_bounds__(THREADS, (THREADS >= 256 ? 4 : 8))
scan_tile_kernel(const T *__restrict__ in, T *__restrict__ out, size_t n, size_t head_pad,
                 int vec_ok, int exclusive, typename P::Carry init_carry, Status st,
                 uint32_t *tile_counter, uint32_t *err) {
  typedef typename P::Acc Acc;
  typedef typename P::Carry Carry;
  constexpr int N = 16 / sizeof(T);
  constexpr int WARPS = THREADS / kWarp;
  __shared__ Acc warp_tot[WARPS];
  __shared__ Carry tile_prefix;
  __shared__ uint32_t tile_slot;

  const unsigned lane = lane_id();
  const unsigned warp = threadIdx.x / kWarp;
  size_t tile = 0;
  if (!SINGLE) {
    if (threadIdx.x == 0) tile_slot = atomicAdd(tile_counter, 1u);
    __syncthreads();
    tile = tile_slot;
  }
  const size_t nv = n + head_pad;
  const size_t tile_vec0 = tile * size_t(THREADS) * V;
  const size_t warp_vec0 = tile_vec0 + size_t(warp) * kWarp * V;

  // A lane owns R consecutive vectors per chunk (its serial run); a warp's
  // chunk is 32*R consecutive vectors; G chunks are loaded together.
  constexpr int R = kScanRunVectors < V ? kScanRunVectors : V;
  static_assert(V % R == 0, "whole runs per thread");
  constexpr int CH = V / R;
  constexpr int G0 = (16 / N) / R > 0 ? (16 / N) / R : 1;
  constexpr int G = G0 < CH ? G0 : CH;
  static_assert(CH % G == 0, "whole groups per thread");
  Acc lane_pre[CH];  // prefix of this lane's first element within the warp's part of the tile
  Acc run = P::ident();
  const bool interior = (warp_vec0 * N >= head_pad) && (warp_vec0 + size_t(V) * kWarp) * N <= nv;
#pragma unroll
  for (int g = 0; g < CH; g += G) {
    T x[G][R][N];
#pragma unroll
    for (int c = 0; c < G; ++c)
#pragma unroll
      for (int q = 0; q < R; ++q)
        load_chunk_l2<T>(in, warp_vec0 + size_t(g + c) * kWarp * R + size_t(lane) * R + q, head_pad, nv,
                         vec_ok != 0, x[c][q]);
#pragma unroll
    for (int c = 0; c < G; ++c) {
      const int j = g + c;
      const size_t u0 = (warp_vec0 + size_t(j) * kWarp * R + size_t(lane) * R) * N;
      Acc t = P::ident();
#pragma unroll
      for (int q = 0; q < R; ++q)
#pragma unroll
        for (int k = 0; k < N; ++k)
          if (interior || (u0 + q * N + k >= head_pad && u0 + q * N + k < nv)) t = P::add(t, x[c][q][k]);
      Acc incl = t;
#pragma unroll
      for (int d = 1; d < kWarp; d <<= 1) {
        Acc o = P::shfl_up(incl, d);
        if (int(lane) >= d) incl = P::comb(o, incl);
      }
      Acc ex = P::shfl_up(incl, 1);
      lane_pre[j] = (lane == 0) ? run : P::comb(run, ex);
      run = P::comb(run, P::shfl(incl, kWarp - 1));
    }
  }
  if (lane == 0) warp_tot[warp] = run;
  __syncthreads();
  Acc warp_excl = P::ident();
  Acc tile_agg = P::ident();
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w == int(warp)) warp_excl = tile_agg;
    tile_agg = P::comb(tile_agg, warp_tot[w]);
  }
  // Tile 0 starts from init (exclusive) or the functor's identity (inclusive).
  const Carry first_prefix = exclusive ? init_carry : P::carry_ident();
  if (SINGLE) {
    if (threadIdx.x == 0) tile_prefix = first_prefix;
  } else if (warp == 0) {
    Carry pre;
    if (tile == 0) {
      pre = first_prefix;
      if (lane == 0) st.publish(0, kFlagPrefix, P::carry_comb(first_prefix, P::to_carry(tile_agg)));
    } else {
      pre = lookback<P>(st, tile, P::to_carry(tile_agg), err);
    }
    if (lane == 0) tile_prefix = pre;
  }
  __syncthreads();
  const Acc base = P::comb(P::from_carry(tile_prefix), warp_excl);
  T *vout_base = out - head_pad;
#pragma unroll
  for (int g = 0; g < CH; g += G) {
    T x[G][R][N];
#pragma unroll
    for (int c = 0; c < G; ++c)
#pragma unroll
      for (int q = 0; q < R; ++q)
        load_chunk<T>(in, warp_vec0 + size_t(g + c) * kWarp * R + size_t(lane) * R + q, head_pad, nv, vec_ok != 0,
                      x[c][q]);
#pragma unroll
    for (int c = 0; c < G; ++c) {
      const int j = g + c;
      Acc r = P::comb(base, lane_pre[j]);
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const size_t vi = warp_vec0 + size_t(j) * kWarp * R + size_t(lane) * R + q;
        const size_t u0 = vi * N;
        T y[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const bool ok = interior || (u0 + k >= head_pad && u0 + k < nv);
          if (exclusive) {
            y[k] = P::out(r);
            if (ok) r = P::add(r, x[c][q][k]);
          } else {
            if (ok) r = P::add(r, x[c][q][k]);
            y[k] = P::out(r);
          }
        }
        if (vec_ok && u0 >= head_pad && u0 + N <= nv) {
          vec16<T> w;
#pragma unroll
          for (int k = 0; k < N; ++k) w.v[k] = y[k];
          st_stream16(reinterpret_cast<vec16<T> *>(vout_base) + vi, w);
        } else {
#pragma unroll
          for (int k = 0; k < N; ++k)
            if (u0 + k >= head_pad && u0 + k < nv) vout_base[u0 + k] = y[k];
        }
      }
    }
  }
}

// ---- shared-memory staged tiles --------------------------------------------
// Tile bytes of the staged scan (three resident tiles per SM) and the size of
// each bulk copy that moves a tile in or out.
constexpr uint32_t kStagedPieceBytes = 16 * 1024;
constexpr int kStagedThreads = 256;
// Tile bytes (measured on GB300 at 2^30 elements): 64 KB, three resident per
// SM; 96 KB for 8-byte elements, whose fenced status words make each look-back
// step dearer, so fewer and larger tiles pay (2.08 ms against 2.40 ms for an
// int64 scan of 2^30 elements).
template <class T> struct staged_tile_bytes {
  static constexpr uint32_t value = sizeof(T) == 8 ? 96u * 1024u : 64u * 1024u;
};
// A block that takes tile i asks L2 to prefetch the tile kStagedPrefetchBytes
// further on, so by the time that tile's block starts, its bulk load is served
// from L2: short, even load times keep the look-back waits short (they wait
// for the slowest predecessor's load), and the DRAM latency is absorbed by the
// 129 MB L2 rather than by shared memory held idle.  16 MB ahead took a 2^30
// int32 scan from 2.02 ms to 1.63 ms; 32 MB and more ahead gained nothing.
constexpr size_t kStagedPrefetchBytes = size_t(16) << 20;
// Resident tiles per SM that the shared memory allows (1 KB per block is
// reserved by the hardware; at most 8 blocks are asked for).
constexpr int staged_blocks_per_sm(uint32_t tile_bytes) {
  return int((227u * 1024u) / (tile_bytes + 1024u)) < 8 ? int((227u * 1024u) / (tile_bytes + 1024u)) : 8;
}

// One block = one tile of TILE_BYTES, moved into shared memory by bulk
// copies (the whole tile in flight at once, no registers held for it) and
// out again by bulk copies after the scan.  Thread t owns the contiguous run
// of VPT 16-byte vectors starting at vector t*VPT.  A thread visits its
// vectors starting at vector (t mod VPT) and wrapping around, so the eight
// threads of each shared-memory phase touch eight different bank groups; the
// fold still combines the run in element order: `part_a` holds vectors
// [r, VPT) and `part_b` vectors [0, r), and the run total is part_b op part_a.
// The second pass rewrites the run in place with its outputs.  DRAM sees each
// input byte once and each output byte once; L2 sees no re-read.
template <class T, class P, class Status, uint32_t TILE_BYTES = staged_tile_bytes<T>::value>
__global__ void __launch_bounds__(kStagedThreads, staged_blocks_per_sm(TILE_BYTES))
scan_staged_kernel(const T *__restrict__ in, T *__restrict__ out, size_t n, int exclusive,
                   typename P::Carry init_carry, Status st, uint32_t *tile_counter, uint32_t *err) {
  typedef typename P::Acc Acc;
  typedef typename P::Carry Carry;
  constexpr int N = 16 / sizeof(T);
  constexpr int VPT = int(TILE_BYTES / (kStagedThreads * 16u));
  constexpr int ITEMS = VPT * N;
  constexpr uint32_t TILE = uint32_t(kStagedThreads) * ITEMS;
  constexpr int WARPS = kStagedThreads / kWarp;
  constexpr size_t PREFETCH_TILES = kStagedPrefetchBytes / TILE_BYTES;
  static_assert(VPT >= 1 && TILE_BYTES % kStagedPieceBytes == 0, "whole pieces per tile");
  extern __shared__ __align__(128) unsigned char staged_smem[];
  vec16<T> *tv = reinterpret_cast<vec16<T> *>(staged_smem);
  T *te = reinterpret_cast<T *>(staged_smem);
  __shared__ unsigned long long bar;
  __shared__ Acc warp_tot[WARPS];
  __shared__ Carry tile_prefix;
  __shared__ uint32_t tile_slot;

  if (threadIdx.x == 0) {
    tile_slot = atomicAdd(tile_counter, 1u);
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const size_t tile = tile_slot;
  const size_t base = tile * TILE;
  const uint32_t cnt = uint32_t((n - base) < TILE ? (n - base) : TILE);
  const uint32_t bulk = (cnt * uint32_t(sizeof(T))) & ~15u;
  const uint32_t bulk_elems = bulk / uint32_t(sizeof(T));
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, bulk);
    const char *src = reinterpret_cast<const char *>(in + base);
    for (uint32_t off = 0; off < bulk; off += kStagedPieceBytes)
      bulk_load_smem(staged_smem + off, src + off, (bulk - off) < kStagedPieceBytes ? (bulk - off) : kStagedPieceBytes,
                     &bar);
    const size_t ahead = tile + PREFETCH_TILES;
    if (PREFETCH_TILES > 0 && ahead * TILE < n) {
      const size_t rest = n - ahead * TILE;
      const uint32_t pf = uint32_t((rest < TILE ? rest : size_t(TILE)) * sizeof(T)) & ~15u;
      const char *pfs = reinterpret_cast<const char *>(in + ahead * TILE);
      for (uint32_t off = 0; off < pf; off += kStagedPieceBytes)
        bulk_prefetch_l2(pfs + off, (pf - off) < kStagedPieceBytes ? (pf - off) : kStagedPieceBytes);
    }
  }
  // The last tile's ragged end (under 16 bytes) comes in by plain loads.
  for (uint32_t i = bulk_elems + threadIdx.x; i < cnt; i += kStagedThreads) te[i] = in[base + i];
  const bool arrived = mbar_wait_bounded(&bar, 0);
  if (__syncthreads_or(!arrived)) {
    // Leave only after the copies into this block's shared memory are done.
    if (threadIdx.x == 0) {
      report_error(err, kErrCopyTimeout);
      mbar_wait_bounded(&bar, 0);
    }
    return;
  }

  const unsigned t = threadIdx.x, lane = lane_id(), warp = t / kWarp;
  const bool full = (cnt == TILE);
  const uint32_t e_first = t * uint32_t(ITEMS);
  const int r = int(t % unsigned(VPT));
  Acc a = P::ident(), part_a = P::ident();
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    int v = k + r;
    if (v >= VPT) v -= VPT;
    if (k > 0 && v == 0) {
      part_a = a;
      a = P::ident();
    }
    const vec16<T> x = tv[t * VPT + v];
#pragma unroll
    for (int m = 0; m < N; ++m)
      if (full || e_first + uint32_t(v * N + m) < cnt) a = P::add(a, x.v[m]);
  }
  Acc part_b = P::ident();
  if (r == 0) part_a = a;
  else part_b = a;
  // Block scan of the run totals.
  Acc incl = P::comb(part_b, part_a);
#pragma unroll
  for (int d = 1; d < kWarp; d <<= 1) {
    const Acc o = P::shfl_up(incl, d);
    if (int(lane) >= d) incl = P::comb(o, incl);
  }
  Acc lane_excl = P::shfl_up(incl, 1);
  if (lane == 0) lane_excl = P::ident();
  if (lane == kWarp - 1) warp_tot[warp] = incl;
  __syncthreads();
  Acc warp_excl = P::ident(), tile_agg = P::ident();
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    if (w == int(warp)) warp_excl = tile_agg;
    tile_agg = P::comb(tile_agg, warp_tot[w]);
  }
  if (warp == 0) {
    const Carry first_prefix = exclusive ? init_carry : P::carry_ident();
    Carry pre;
    if (tile == 0) {
      pre = first_prefix;
      if (lane == 0) st.publish(0, kFlagPrefix, P::carry_comb(first_prefix, P::to_carry(tile_agg)));
    } else {
      pre = lookback<P>(st, tile, P::to_carry(tile_agg), err);
    }
    if (lane == 0) tile_prefix = pre;
  }
  __syncthreads();
  const Acc pre = P::comb(P::comb(P::from_carry(tile_prefix), warp_excl), lane_excl);
  Acc run = P::comb(pre, part_b);
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    int v = k + r;
    if (v >= VPT) v -= VPT;
    if (k > 0 && v == 0) run = pre;
    const vec16<T> x = tv[t * VPT + v];
    vec16<T> y;
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const bool ok = full || e_first + uint32_t(v * N + m) < cnt;
      if (exclusive) {
        y.v[m] = P::out(run);
        if (ok) run = P::add(run, x.v[m]);
      } else {
        if (ok) run = P::add(run, x.v[m]);
        y.v[m] = P::out(run);
      }
    }
    tv[t * VPT + v] = y;
  }
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    char *dst = reinterpret_cast<char *>(out + base);
    for (uint32_t off = 0; off < bulk; off += kStagedPieceBytes)
      bulk_store_global(dst + off, staged_smem + off, (bulk - off) < kStagedPieceBytes ? (bulk - off) : kStagedPieceBytes);
    bulk_commit_group();
    bulk_wait_group_read0();
  }
  for (uint32_t i = bulk_elems + threadIdx.x; i < cnt; i += kStagedThreads) out[base + i] = te[i];
}

// Opts scan_staged_kernel<T, P, Status> into its tile bytes of dynamic
// shared memory on the current device (once per device and instantiation:
// the flags are per instantiation, not per kernel signature, which several
// functors share).
template <class T, class P, class Status>
cudaError_t staged_smem_optin() {
  auto kernel = scan_staged_kernel<T, P, Status>;
  static std::mutex mu;
  static uint64_t done = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && (done >> dev) & 1u) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(staged_tile_bytes<T>::value));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, int(cudaSharedmemCarveoutMaxShared));
  if (e == cudaSuccess && dev < 64) done |= uint64_t(1) << dev;
  return e;
}

// Tile shape of the allocating scan (measured on GB300 at 2^30 elements):
// 96 elements per thread when the accumulator is at most 4 bytes (96 KB tiles
// of 4-byte elements; 64 and 128 per thread were slower), 32 compensated FP32
// pairs per thread in 512-thread blocks, 8 elements of 8-byte types.
template <class T, class P> struct scan_vectors_per_thread {
  static constexpr int value = sizeof(typename P::Acc) <= 4 ? int(96 / (16 / sizeof(T))) : (sizeof(T) == 4 ? 8 : 4);
};
template <class P> struct scan_threads {
  static constexpr int value = kScanThreads;
};
template <> struct scan_threads<ScanCompF32> {
  static constexpr int value = 512;
};

template <class T, class P>
bcx_status run_scan_t(cudaStream_t s, int exclusive, const void *init, const void *in, void *out,
                      size_t n, void *temp, size_t *temp_bytes) {
  typedef typename P::Carry Carry;
  typedef TileStatus<Carry> Status;
  constexpr int N = 16 / sizeof(T);
  constexpr int V = scan_vectors_per_thread<T, P>::value;
  constexpr int THREADS = scan_threads<P>::value;
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const uintptr_t ain = reinterpret_cast<uintptr_t>(in), aout = reinterpret_cast<uintptr_t>(out);
  const bool elem_aligned = (ain % sizeof(T) == 0) && (aout % sizeof(T) == 0);
  const bool vec_ok = elem_aligned && ((ain & 15u) == (aout & 15u));
  const size_t head_pad = vec_ok ? (ain & 15u) / sizeof(T) : 0;
  const size_t nv = n + head_pad;
  const size_t tile_elems = size_t(THREADS) * V * N;
  const size_t tiles = div_up(nv, tile_elems);
  const bool single = (tiles <= 1);
  // Staged tiles need 16-byte aligned input and output (bulk copies); the
  // temporary is sized for either shape, so a size query holds for both.
  const size_t staged_tile_elems = staged_tile_bytes<T>::value / sizeof(T);
  const size_t staged_tiles = div_up(n, staged_tile_elems);
  const bool staged = !single && ((ain | aout) & 15u) == 0;
  const size_t need = single ? 0 : (256 + Status::bytes(tiles > staged_tiles ? tiles : staged_tiles));
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, need, s, &query);
  if (rc || query) return rc;
  Carry init_carry = P::host_carry(init);
  const T *pin = static_cast<const T *>(in);
  T *pout = static_cast<T *>(out);
  if (single) {
    Status st{};
    KernelScope ks("scan_single", s);
    scan_tile_kernel<T, P, THREADS, V, true, Status><<<1, THREADS, 0, s>>>(
        pin, pout, n, head_pad, vec_ok ? 1 : 0, exclusive, init_carry, st, nullptr, ds->err_word);
    return launch_status("scan_single");
  }
  char *base = static_cast<char *>(ts.ptr());
  uint32_t *counter = reinterpret_cast<uint32_t *>(base);
  Status st;
  if (staged) {
    st.bind(base + 256, staged_tiles);
    BCX_CUDA(cudaMemsetAsync(base, 0, 256, s));
    BCX_CUDA(st.clear(staged_tiles, s));
    BCX_CHECK(staged_tiles < (size_t(1) << 31), BCX_INVALID_VALUE, "scan: input too large");
    BCX_CUDA((staged_smem_optin<T, P, Status>()));
    auto kernel = scan_staged_kernel<T, P, Status>;
    KernelScope ks("scan_lookback", s);
    kernel<<<unsigned(staged_tiles), kStagedThreads, staged_tile_bytes<T>::value, s>>>(pin, pout, n, exclusive,
                                                                                        init_carry, st,
                                                                            counter, ds->err_word);
    return launch_status("scan_lookback");
  }
  st.bind(base + 256, tiles);
  BCX_CUDA(cudaMemsetAsync(base, 0, 256, s));
  BCX_CUDA(st.clear(tiles, s));
  BCX_CHECK(tiles < (size_t(1) << 31), BCX_INVALID_VALUE, "scan: input too large");
  KernelScope ks("scan_lookback", s);
  scan_tile_kernel<T, P, THREADS, V, false, Status><<<unsigned(tiles), THREADS, 0, s>>>(
      pin, pout, n, head_pad, vec_ok ? 1 : 0, exclusive, init_carry, st, counter, ds->err_word);
  return launch_status("scan_lookback");
}

template <class T>
bcx_status dispatch_int(cudaStream_t s, int op, int ex, const void *init, const void *in,
                        void *out, size_t n, void *temp, size_t *tb) {
  switch (op) {
    case BCX_PLUS: return run_scan_t<T, ScanPlain<T, op_plus>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MULTIPLIES: return run_scan_t<T, ScanPlain<T, op_multiplies>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MIN: return run_scan_t<T, ScanPlain<T, op_min>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MAX: return run_scan_t<T, ScanPlain<T, op_max>>(s, ex, init, in, out, n, temp, tb);
    case BCX_BIT_AND: return run_scan_t<T, ScanPlain<T, op_bit_and>>(s, ex, init, in, out, n, temp, tb);
    case BCX_BIT_OR: return run_scan_t<T, ScanPlain<T, op_bit_or>>(s, ex, init, in, out, n, temp, tb);
    case BCX_BIT_XOR: return run_scan_t<T, ScanPlain<T, op_bit_xor>>(s, ex, init, in, out, n, temp, tb);
  }
  return BCX_UNSUPPORTED;
}

template <class T>
bcx_status dispatch_float(cudaStream_t s, int op, int ex, const void *init, const void *in,
                          void *out, size_t n, int comp, void *temp, size_t *tb) {
  switch (op) {
    case BCX_PLUS:
      if (comp) {
        if (sizeof(T) == 4) return run_scan_t<float, ScanCompF32>(s, ex, init, in, out, n, temp, tb);
        return run_scan_t<double, ScanCompF64>(s, ex, init, in, out, n, temp, tb);
      }
      return run_scan_t<T, ScanPlain<T, op_plus>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MULTIPLIES: return run_scan_t<T, ScanPlain<T, op_multiplies>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MIN: return run_scan_t<T, ScanPlain<T, op_min>>(s, ex, init, in, out, n, temp, tb);
    case BCX_MAX: return run_scan_t<T, ScanPlain<T, op_max>>(s, ex, init, in, out, n, temp, tb);
  }
  return BCX_UNSUPPORTED;
}

}  // namespace
}  // namespace bcx

namespace bcx {
// The allocating scan for one group of element types each (the group's
// kernels are compiled in their own translation unit, so the library builds
// in parallel): 1- and 2-byte integers, 4-byte integers, 8-byte integers,
// float and double.  Arguments as bcx_scan, after its checks; init points to
// the initial value (zeros when absent).
bcx_status scan_small_ints(cudaStream_t s, bcx_dtype type, int op, int exclusive, const void *init,
                           const void *in, void *out, size_t n, void *temp, size_t *temp_bytes);
bcx_status scan_word_ints(cudaStream_t s, bcx_dtype type, int op, int exclusive, const void *init,
                          const void *in, void *out, size_t n, void *temp, size_t *temp_bytes);
bcx_status scan_wide_ints(cudaStream_t s, bcx_dtype type, int op, int exclusive, const void *init,
                          const void *in, void *out, size_t n, void *temp, size_t *temp_bytes);
bcx_status scan_floats(cudaStream_t s, bcx_dtype type, int op, int exclusive, const void *init,
                       const void *in, void *out, size_t n, int compensated, void *temp, size_t *temp_bytes);
}  // namespace bcx

#endif  // BCX_SCAN_CUH
