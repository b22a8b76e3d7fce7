// bcx_segmented.cu -- segmented scan and segmented reduce in one launch each.
//
// The reference has no segmented algorithms: a caller loops over segments and
// issues one exclusive_scan / reduce per segment (each several launches, see
// algorithm/detail/scan_on_gpu.hpp:187-267 and reduce_on_gpu.hpp:169-280), or
// uses reduce_by_key with segment ids as keys (reduce_by_key_with_scan.hpp).
// Segments here are CSR offsets: segment s is [offsets[s], offsets[s+1]),
// offsets[0] == 0, offsets[nseg] == n, non-decreasing (empty segments allowed).
//
// Segmented scan: the decoupled look-back scan with the segmented operator
// (head, value): (a then b) = (a.head | b.head, b.head ? b.value : a op b).
// Each tile marks the segment heads that fall inside it in a shared-memory
// bitmap (one binary search per tile, then one pass over those offsets), so a
// tile costs one read and one write of its elements whatever the segment
// sizes.  Exclusive scans start every segment at init.
//
// Segmented reduce: persistent blocks take segments from a ticket counter and
// fold each with every thread striding the segment, four independent
// accumulators per thread; one output per segment (init for an empty one).
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <type_traits>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"

namespace bcx {
namespace {

constexpr int kSegThreads = 256;
constexpr int kSegWarps = kSegThreads / kWarp;
enum : uint32_t { kSgInvalid = 0, kSgAggregate = 1, kSgPrefix = 2 };

template <class T, template <class> class OpT>
struct SgPlain {
  typedef typename widen<T>::type Acc;
  typedef OpT<Acc> Op;
  __device__ __forceinline__ static Acc ident() { return Op::identity(); }
  __device__ __forceinline__ static Acc from(T x) { return Acc(x); }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return Op()(a, b); }
  __device__ __forceinline__ static T out(Acc a) { return T(a); }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
  __device__ __forceinline__ static Acc shfl_down(Acc a, int d) { return __shfl_down_sync(0xffffffffu, a, d); }
  __device__ __forceinline__ static Acc shfl(Acc a, int s) { return __shfl_sync(0xffffffffu, a, s); }
};
struct SgCompF32 {
  typedef comp_f32 Acc;
  __device__ __forceinline__ static Acc ident() { return comp_f32{0.f, 0.f}; }
  __device__ __forceinline__ static Acc from(float x) { return comp_f32{x, 0.f}; }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return comp_merge(a, b); }
  __device__ __forceinline__ static float out(Acc a) { return a.s + a.c; }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) {
    return comp_f32{__shfl_up_sync(0xffffffffu, a.s, d), __shfl_up_sync(0xffffffffu, a.c, d)};
  }
  __device__ __forceinline__ static Acc shfl_down(Acc a, int d) {
    return comp_f32{__shfl_down_sync(0xffffffffu, a.s, d), __shfl_down_sync(0xffffffffu, a.c, d)};
  }
  __device__ __forceinline__ static Acc shfl(Acc a, int s) {
    return comp_f32{__shfl_sync(0xffffffffu, a.s, s), __shfl_sync(0xffffffffu, a.c, s)};
  }
};

// (head flag, value); combine is "b restarts the segment if it holds a head".
template <class P>
struct Sg {
  uint32_t h;
  typename P::Acc v;
};
template <class P>
__device__ __forceinline__ Sg<P> sg_comb(const Sg<P> &a, const Sg<P> &b) {
  return Sg<P>{a.h | b.h, b.h ? b.v : P::comb(a.v, b.v)};
}
template <class P>
__device__ __forceinline__ Sg<P> sg_ident() {
  return Sg<P>{0u, P::ident()};
}
template <class P>
__device__ __forceinline__ Sg<P> sg_shfl_up(const Sg<P> &a, int d) {
  return Sg<P>{__shfl_up_sync(0xffffffffu, a.h, d), P::shfl_up(a.v, d)};
}
template <class P>
__device__ __forceinline__ Sg<P> sg_shfl_down(const Sg<P> &a, int d) {
  return Sg<P>{__shfl_down_sync(0xffffffffu, a.h, d), P::shfl_down(a.v, d)};
}
template <class P>
__device__ __forceinline__ Sg<P> sg_shfl(const Sg<P> &a, int s) {
  return Sg<P>{__shfl_sync(0xffffffffu, a.h, s), P::shfl(a.v, s)};
}

// Look-back status of one tile.  With a 4-byte value the flag, the head bit
// and the value travel in one 64-bit word (relaxed loads and stores suffice);
// wider values use a flag array plus aggregate/inclusive arrays ordered by
// release/acquire.
template <class P, bool PACK = (sizeof(typename P::Acc) == 4)>
struct SgStatus;

template <class P>
struct SgStatus<P, true> {
  unsigned long long *words;
  static size_t bytes(size_t tiles) { return align256(tiles * 8); }
  static size_t zero_bytes(size_t tiles) { return bytes(tiles); }
  void bind(char *base, size_t) { words = reinterpret_cast<unsigned long long *>(base); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, const Sg<P> &v) {
    uint32_t bits;
    memcpy(&bits, &v.v, 4);
    const unsigned long long w = (static_cast<unsigned long long>(bits) << 32) | (v.h << 2) | flag;
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(&words[t]), "l"(w) : "memory");
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Sg<P> *v) const {
    const unsigned long long w = ld_relaxed_u64(&words[t]);
    const uint32_t bits = uint32_t(w >> 32);
    memcpy(&v->v, &bits, 4);
    v->h = uint32_t(w >> 2) & 1u;
    return uint32_t(w & 3u);
  }
};

template <class P>
struct SgStatus<P, false> {
  uint32_t *flags;
  Sg<P> *agg;
  Sg<P> *inc;
  static size_t bytes(size_t tiles) { return align256(tiles * 4) + 2 * align256(tiles * sizeof(Sg<P>)); }
  static size_t zero_bytes(size_t tiles) { return align256(tiles * 4); }
  void bind(char *base, size_t tiles) {
    flags = reinterpret_cast<uint32_t *>(base);
    agg = reinterpret_cast<Sg<P> *>(base + align256(tiles * 4));
    inc = reinterpret_cast<Sg<P> *>(base + align256(tiles * 4) + align256(tiles * sizeof(Sg<P>)));
  }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, const Sg<P> &v) {
    if (flag == kSgAggregate) agg[t] = v;
    else inc[t] = v;
    st_release_u32(&flags[t], flag);
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Sg<P> *v) const {
    const uint32_t f = ld_acquire_u32(&flags[t]);
    if (f != kSgInvalid) {
      const Sg<P> *src = (f == kSgAggregate) ? &agg[t] : &inc[t];
      const volatile uint32_t *w = reinterpret_cast<const volatile uint32_t *>(src);
      uint32_t tmp[sizeof(Sg<P>) / 4];
#pragma unroll
      for (int i = 0; i < int(sizeof(Sg<P>) / 4); ++i) tmp[i] = w[i];
      memcpy(v, tmp, sizeof(Sg<P>));
    }
    return f;
  }
};

// First segment whose start is at or after each tile's first element: one
// thread per tile, so every tile's binary search is in flight at once instead
// of sitting on the scan kernel's critical path.
__global__ void seg_tile_first_kernel(const unsigned long long *__restrict__ offsets, size_t nseg, size_t tile,
                                      size_t tiles, uint32_t *__restrict__ tile_first_seg) {
  const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (t >= tiles) return;
  const unsigned long long x = t * tile;
  size_t lo = 0, hi = nseg;
  while (lo < hi) {
    const size_t mid = (lo + hi) / 2;
    if (offsets[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  tile_first_seg[t] = uint32_t(lo);
}

// Bytes of consecutive elements a lane owns per chunk of the segmented scan
// (a multiple of 16: one or more 16-byte vector loads).
constexpr int kSegRunBytes = 32;

template <class T, int N>
struct alignas(sizeof(T) * N) SegVec {
  T v[N];
};

// ITEMS elements per thread in ITEMS/N chunks; in chunk j lane l owns the N
// consecutive elements chunk_base + l*N .. + N-1 (one vector load and store
// when the arrays are aligned), so (j, l, m) is input order within a warp.
constexpr size_t kSegPrefetchBytes = kL2PrefetchBytes;

template <class T, class P, int ITEMS>
__global__ void __launch_bounds__(kSegThreads, 4)
segmented_scan_kernel(const T *__restrict__ in, T *__restrict__ out, size_t n,
                      const unsigned long long *__restrict__ offsets, size_t nseg,
                      const uint32_t *__restrict__ tile_first_seg, int exclusive, typename P::Acc init,
                      SgStatus<P> st, uint32_t *__restrict__ tile_counter, int vec_in, int vec_out, uint32_t *err) {
  typedef Sg<P> S;
  typedef typename P::Acc Acc;
  constexpr int N = kSegRunBytes / int(sizeof(T)) < ITEMS ? kSegRunBytes / int(sizeof(T)) : ITEMS;
  constexpr int CH = ITEMS / N;
  constexpr int TILE = kSegThreads * ITEMS;
  static_assert(32 % N == 0, "a lane's run sits inside one bitmap word");
  __shared__ uint32_t s_heads[TILE / 32];
  __shared__ S s_warp[kSegWarps];
  __shared__ S s_prefix;
  __shared__ uint32_t s_tile;
  const unsigned lane = lane_id(), warp = threadIdx.x / kWarp;
  for (int i = threadIdx.x; i < TILE / 32; i += kSegThreads) s_heads[i] = 0;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const size_t tile = s_tile;
  const size_t tile_base = tile * TILE;
  // Ask L2 for the tile kSegPrefetchBytes ahead, so that tile's first read is
  // served from L2 (short, even load times keep the look-back waits short).
  if (kSegPrefetchBytes > 0 && threadIdx.x == 0 && vec_in)
    prefetch_l2_range(in, (tile + kSegPrefetchBytes / (size_t(TILE) * sizeof(T))) * TILE, TILE, n);
  const size_t tile_end = (tile_base + TILE < n) ? tile_base + TILE : n;
  const uint32_t warp_first = warp * (kWarp * ITEMS);
  // Mark the segment starts inside this tile (offsets[0..nseg] are starts;
  // offsets[nseg] == n is not); the tile's first candidate segment comes from
  // the pre-pass, so this is one load and usually a single iteration.
  if (warp == 0) {
    const size_t first = tile_first_seg[tile];
    for (size_t k = first + lane; k < nseg; k += kWarp) {
      const unsigned long long o = offsets[k];
      if (o >= tile_end) break;
      const uint32_t local = uint32_t(o - tile_base);
      atomicOr(&s_heads[local >> 5], 1u << (local & 31u));
    }
  }
  __syncthreads();  // head bitmap complete
  // Pass 1: per chunk, serial fold of the lane's run and a warp scan of the
  // lane folds, G chunks loaded at a time (cached in L2 for the second read).
  // Only the per-chunk prefixes stay in registers across the look-back.
  constexpr int G = CH < 4 ? CH : 4;
  S lane_pre[CH];  // fold of everything before the lane's run in chunk j (within the warp)
  S run = sg_ident<P>();
#pragma unroll
  for (int g = 0; g < CH; g += G) {
    T x[G][N];
#pragma unroll
    for (int c = 0; c < G; ++c) {
      const size_t e0 = tile_base + warp_first + (g + c) * (kWarp * N) + lane * N;
      if (vec_in && e0 + N <= n) {
        SegVec<T, N> w;
        uint4 u[sizeof(w) / 16];
#pragma unroll
        for (int q = 0; q < int(sizeof(w) / 16); ++q) u[q] = __ldcg(reinterpret_cast<const uint4 *>(in + e0) + q);
        memcpy(&w, u, sizeof(w));
#pragma unroll
        for (int m = 0; m < N; ++m) x[c][m] = w.v[m];
      } else {
#pragma unroll
        for (int m = 0; m < N; ++m) x[c][m] = (e0 + m < n) ? in[e0 + m] : T(0);
      }
    }
#pragma unroll
    for (int c = 0; c < G; ++c) {
      const int j = g + c;
      const size_t e0 = tile_base + warp_first + j * (kWarp * N) + lane * N;
      const uint32_t local = warp_first + j * (kWarp * N) + lane * N;
      const uint32_t hb = (s_heads[local >> 5] >> (local & 31u)) & ((1u << N) - 1u);
      S a = sg_ident<P>();
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const S e{(hb >> m) & 1u, (e0 + m < n) ? P::from(x[c][m]) : P::ident()};
        a = sg_comb<P>(a, e);
      }
#pragma unroll
      for (int d = 1; d < kWarp; d <<= 1) {
        const S o = sg_shfl_up<P>(a, d);
        if (int(lane) >= d) a = sg_comb<P>(o, a);
      }
      const S ex = sg_shfl_up<P>(a, 1);
      lane_pre[j] = lane == 0 ? run : sg_comb<P>(run, ex);
      run = sg_comb<P>(run, sg_shfl<P>(a, kWarp - 1));
    }
  }
  if (lane == 0) s_warp[warp] = run;
  __syncthreads();
  S warp_excl = sg_ident<P>(), tile_agg = sg_ident<P>();
#pragma unroll
  for (int w = 0; w < kSegWarps; ++w) {
    if (w == int(warp)) warp_excl = tile_agg;
    tile_agg = sg_comb<P>(tile_agg, s_warp[w]);
  }
  if (warp == 0) {
    S excl = sg_ident<P>();
    if (tile == 0) {
      if (lane == 0) st.publish(0, kSgPrefix, tile_agg);
    } else {
      if (lane == 0) st.publish(tile, kSgAggregate, tile_agg);
      long long pred = (long long)tile - 1;
      bool gave_up = false;
      while (true) {
        const long long t = pred - (long long)lane;
        S val = sg_ident<P>();
        uint32_t f = kSgPrefix;
        if (t >= 0) {
          uint32_t spins = 0;
          f = st.poll(size_t(t), &val);
          while (f == kSgInvalid) {
            if (++spins > kSpinLimit) {
              gave_up = true;
              f = kSgPrefix;
              val = sg_ident<P>();
              break;
            }
            if (spins > 16) __nanosleep(64);
            f = st.poll(size_t(t), &val);
          }
        }
        const unsigned pmask = __ballot_sync(0xffffffffu, f == kSgPrefix);
        const int firstp = pmask ? __ffs(pmask) - 1 : kWarp - 1;
        if (int(lane) > firstp) val = sg_ident<P>();
#pragma unroll
        for (int d = 1; d < kWarp; d <<= 1) {
          const S o = sg_shfl_down<P>(val, d);
          if (int(lane) + d < kWarp) val = sg_comb<P>(o, val);
        }
        excl = sg_comb<P>(sg_shfl<P>(val, 0), excl);
        if (pmask) break;
        pred -= kWarp;
      }
      if (__any_sync(0xffffffffu, gave_up) && lane == 0) report_error(err, kErrLookbackTimeout);
      if (lane == 0) st.publish(tile, kSgPrefix, sg_comb<P>(excl, tile_agg));
    }
    if (lane == 0) s_prefix = excl;
  }
  __syncthreads();
  // Pass 2: inclusive output is the running value after each element;
  // exclusive output is init for a segment's first element, else init op the
  // running value before it.
  const S pre = sg_comb<P>(s_prefix, warp_excl);
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const size_t e0 = tile_base + warp_first + j * (kWarp * N) + lane * N;
    const uint32_t local = warp_first + j * (kWarp * N) + lane * N;
    const uint32_t hb = (s_heads[local >> 5] >> (local & 31u)) & ((1u << N) - 1u);
    T x[N];
    if (vec_in && e0 + N <= n) {
      const SegVec<T, N> w = *reinterpret_cast<const SegVec<T, N> *>(in + e0);
#pragma unroll
      for (int m = 0; m < N; ++m) x[m] = w.v[m];
    } else {
#pragma unroll
      for (int m = 0; m < N; ++m) x[m] = (e0 + m < n) ? in[e0 + m] : T(0);
    }
    S acc = sg_comb<P>(pre, lane_pre[j]);
    T y[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const uint32_t h = (hb >> m) & 1u;
      const Acc ex = h ? init : P::comb(init, acc.v);
      acc = sg_comb<P>(acc, S{h, (e0 + m < n) ? P::from(x[m]) : P::ident()});
      y[m] = P::out(exclusive ? ex : acc.v);
    }
    if (vec_out && e0 + N <= n) {
      SegVec<T, N> w;
#pragma unroll
      for (int m = 0; m < N; ++m) w.v[m] = y[m];
      *reinterpret_cast<SegVec<T, N> *>(out + e0) = w;
    } else {
#pragma unroll
      for (int m = 0; m < N; ++m)
        if (e0 + m < n) out[e0 + m] = y[m];
    }
  }
}

template <class T, class P>
__global__ void __launch_bounds__(kSegThreads)
segmented_reduce_kernel(const T *__restrict__ in, const unsigned long long *__restrict__ offsets, size_t nseg,
                        typename P::Acc init, T *__restrict__ out, uint32_t *__restrict__ seg_counter, int vec) {
  typedef typename P::Acc Acc;
  constexpr int N = 16 / int(sizeof(T));
  __shared__ Acc s_acc[kSegWarps];
  __shared__ uint32_t s_seg;
  while (true) {
    if (threadIdx.x == 0) s_seg = atomicAdd(seg_counter, 1u);
    __syncthreads();
    const size_t seg = s_seg;
    if (seg >= nseg) break;
    const size_t b = offsets[seg], e = offsets[seg + 1];
    Acc a0 = P::ident(), a1 = P::ident(), a2 = P::ident(), a3 = P::ident();
    // Scalar head up to the first 16-byte boundary, then 16-byte vectors,
    // four in flight per thread, then the scalar tail (the operators are
    // commutative, so the order of the partial folds is free).
    size_t hb = e;
    if (vec) {
      hb = b + ((16u - (reinterpret_cast<uintptr_t>(in + b) & 15u)) & 15u) / sizeof(T);
      if (hb > e) hb = e;
    }
    for (size_t i = b + threadIdx.x; i < hb; i += kSegThreads) a0 = P::comb(a0, P::from(in[i]));
    const size_t nvec = (e - hb) / N;
    const vec16<T> *vp = reinterpret_cast<const vec16<T> *>(in + hb);
    size_t v = threadIdx.x;
    for (; v + 3 * kSegThreads < nvec; v += 4 * kSegThreads) {
      const vec16<T> x0 = ld_stream16(vp + v), x1 = ld_stream16(vp + v + kSegThreads),
                     x2 = ld_stream16(vp + v + 2 * kSegThreads), x3 = ld_stream16(vp + v + 3 * kSegThreads);
#pragma unroll
      for (int m = 0; m < N; ++m) {
        a0 = P::comb(a0, P::from(x0.v[m]));
        a1 = P::comb(a1, P::from(x1.v[m]));
        a2 = P::comb(a2, P::from(x2.v[m]));
        a3 = P::comb(a3, P::from(x3.v[m]));
      }
    }
    for (; v < nvec; v += kSegThreads) {
      const vec16<T> x = ld_stream16(vp + v);
#pragma unroll
      for (int m = 0; m < N; ++m) a1 = P::comb(a1, P::from(x.v[m]));
    }
    for (size_t i = hb + nvec * N + threadIdx.x; i < e; i += kSegThreads) a2 = P::comb(a2, P::from(in[i]));
    Acc a = P::comb(P::comb(a0, a1), P::comb(a2, a3));
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) a = P::comb(a, P::shfl_down(a, d));
    if (lane_id() == 0) s_acc[threadIdx.x / kWarp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      Acc r = init;
      for (int w = 0; w < kSegWarps; ++w) r = P::comb(r, s_acc[w]);
      out[seg] = P::out(r);
    }
    __syncthreads();
  }
}

// Tile shapes the segmented scan is compiled for: 32 or 64 items per thread
// for 4-byte elements, 8 or 16 for wider ones (tunable "items_per_thread").
template <class T> struct SegScanShapes {
  static constexpr int small = sizeof(T) == 4 ? 32 : 8;
  static constexpr int large = sizeof(T) == 4 ? 64 : 16;
};

std::string seg_object(const char *what, bcx_dtype t) { return std::string(what) + "_" + dtype_name(t); }

template <class T, class P, int ITEMS>
bcx_status launch_segmented_scan(cudaStream_t s, int exclusive, const T &init_v, const void *in, void *out,
                                 size_t n, const unsigned long long *offsets, size_t nseg, char *base,
                                 uint32_t *tile_first_seg, const SgStatus<P> &st, DeviceState *ds) {
  const size_t tile = size_t(kSegThreads) * ITEMS;
  const size_t tiles = div_up(n, tile);
  {
    KernelScope ks("segmented_scan_plan", s);
    seg_tile_first_kernel<<<unsigned(div_up(tiles, size_t(256))), 256, 0, s>>>(offsets, nseg, tile, tiles,
                                                                               tile_first_seg);
    const bcx_status rc = launch_status("segmented_scan_plan");
    if (rc) return rc;
  }
  constexpr int N = kSegRunBytes / int(sizeof(T)) < ITEMS ? kSegRunBytes / int(sizeof(T)) : ITEMS;
  const int vec_in = reinterpret_cast<uintptr_t>(in) % (sizeof(T) * N) == 0;
  const int vec_out = reinterpret_cast<uintptr_t>(out) % (sizeof(T) * N) == 0;
  KernelScope ks("segmented_scan", s);
  segmented_scan_kernel<T, P, ITEMS><<<unsigned(tiles), kSegThreads, 0, s>>>(
      static_cast<const T *>(in), static_cast<T *>(out), n, offsets, nseg, tile_first_seg, exclusive,
      P::from_host(init_v), st, reinterpret_cast<uint32_t *>(base), vec_in, vec_out, ds->err_word);
  return launch_status("segmented_scan");
}

template <class T, class P>
bcx_status run_segmented_scan(cudaStream_t s, bcx_dtype type, int exclusive, const void *init, const void *in,
                              void *out, size_t n, const unsigned long long *offsets, size_t nseg, void *temp,
                              size_t *temp_bytes) {
  typedef SegScanShapes<T> Shapes;
  typedef SgStatus<P> Status;
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  BCX_CHECK(nseg < (size_t(1) << 32), BCX_INVALID_VALUE, "segmented scan: too many segments");
  // Storage for the most tiles any compiled shape makes, so the size does not
  // depend on the tuned shape.  Layout: ticket line | status | tile -> first
  // segment.
  const size_t tiles = div_up(n, size_t(kSegThreads) * Shapes::small);
  const size_t need = 256 + Status::bytes(tiles) + align256(tiles * 4);
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, need, s, &query);
  if (rc || query) return rc;
  char *base = static_cast<char *>(ts.ptr());
  Status st;
  st.bind(base + 256, tiles);
  uint32_t *tile_first_seg = reinterpret_cast<uint32_t *>(base + 256 + Status::bytes(tiles));
  BCX_CUDA(cudaMemsetAsync(base, 0, 256 + Status::zero_bytes(tiles), s));
  T init_v;
  memcpy(&init_v, init, sizeof(T));
  const uint32_t items = param_get(seg_object("segmented_scan", type), "items_per_thread", uint32_t(Shapes::small));
  if (items == uint32_t(Shapes::large))
    return launch_segmented_scan<T, P, Shapes::large>(s, exclusive, init_v, in, out, n, offsets, nseg, base,
                                                      tile_first_seg, st, ds);
  return launch_segmented_scan<T, P, Shapes::small>(s, exclusive, init_v, in, out, n, offsets, nseg, base,
                                                    tile_first_seg, st, ds);
}

template <class T, class P>
bcx_status run_segmented_reduce(cudaStream_t s, bcx_dtype type, const void *in, const unsigned long long *offsets,
                                size_t nseg, const void *init, void *out, void *temp, size_t *temp_bytes) {
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, 256, s, &query);
  if (rc || query) return rc;
  BCX_CUDA(cudaMemsetAsync(ts.ptr(), 0, 256, s));
  T init_v;
  memcpy(&init_v, init, sizeof(T));
  const uint32_t per_sm = param_get(seg_object("segmented_reduce", type), "blocks_per_sm", 8u);
  size_t blocks = size_t(ds->sm_count) * (per_sm ? per_sm : 8u);
  if (blocks > nseg) blocks = nseg;
  KernelScope ks("segmented_reduce", s);
  segmented_reduce_kernel<T, P><<<unsigned(blocks), kSegThreads, 0, s>>>(
      static_cast<const T *>(in), offsets, nseg, P::from_host(init_v), static_cast<T *>(out),
      static_cast<uint32_t *>(ts.ptr()), reinterpret_cast<uintptr_t>(in) % sizeof(T) == 0 ? 1 : 0);
  return launch_status("segmented_reduce");
}

// Host-side conversion of init into the accumulator type.
template <class T, template <class> class OpT>
struct SgPlainH : SgPlain<T, OpT> {
  static typename SgPlain<T, OpT>::Acc from_host(T v) { return typename SgPlain<T, OpT>::Acc(v); }
};
struct SgCompF32H : SgCompF32 {
  static comp_f32 from_host(float v) { return comp_f32{v, 0.f}; }
};

template <class T, class Fn>
bcx_status seg_dispatch_op(int op, int comp, Fn &&fn) {
  switch (op) {
    case BCX_PLUS:
      if constexpr (sizeof(T) == 4 && type_traits<T>::is_float) {
        if (comp) return fn(static_cast<SgCompF32H *>(nullptr));
      }
      return fn(static_cast<SgPlainH<T, op_plus> *>(nullptr));
    case BCX_MULTIPLIES: return fn(static_cast<SgPlainH<T, op_multiplies> *>(nullptr));
    case BCX_MIN: return fn(static_cast<SgPlainH<T, op_min> *>(nullptr));
    case BCX_MAX: return fn(static_cast<SgPlainH<T, op_max> *>(nullptr));
  }
  return BCX_UNSUPPORTED;
}

template <class Fn>
bcx_status seg_dispatch(bcx_dtype t, int op, int comp, Fn &&fn) {
  switch (t) {
    case BCX_INT: return seg_dispatch_op<int32_t>(op, comp, [&](auto *p) { return fn((int32_t *)nullptr, p); });
    case BCX_UINT: return seg_dispatch_op<uint32_t>(op, comp, [&](auto *p) { return fn((uint32_t *)nullptr, p); });
    case BCX_LONG: return seg_dispatch_op<long long>(op, comp, [&](auto *p) { return fn((long long *)nullptr, p); });
    case BCX_ULONG:
      return seg_dispatch_op<unsigned long long>(op, comp, [&](auto *p) { return fn((unsigned long long *)nullptr, p); });
    case BCX_FLOAT: return seg_dispatch_op<float>(op, comp, [&](auto *p) { return fn((float *)nullptr, p); });
    case BCX_DOUBLE: return seg_dispatch_op<double>(op, comp, [&](auto *p) { return fn((double *)nullptr, p); });
    default: break;
  }
  return BCX_UNSUPPORTED;
}

}  // namespace

void segscan_shapes(size_t elem_bytes, uint32_t *small, uint32_t *large) {
  if (elem_bytes == 4) {
    *small = SegScanShapes<int32_t>::small;
    *large = SegScanShapes<int32_t>::large;
  } else {
    *small = SegScanShapes<int64_t>::small;
    *large = SegScanShapes<int64_t>::large;
  }
}

}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_segmented_scan(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive, const void *init,
                              const void *in, void *out, size_t n, const uint64_t *offsets, size_t nseg,
                              int compensated, void *temp, size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (n == 0) {
    if (temp == nullptr && temp_bytes != nullptr) *temp_bytes = 0;
    return BCX_SUCCESS;
  }
  BCX_CHECK(in && out && offsets && nseg > 0, BCX_INVALID_VALUE, "NULL argument or no segments");
  BCX_CHECK(n < (size_t(1) << 40), BCX_INVALID_VALUE, "segmented scan: n too large");
  unsigned char zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const void *init_p = (exclusive && init) ? init : zero;
  const auto *offs = reinterpret_cast<const unsigned long long *>(offsets);
  bcx_status rc = seg_dispatch(type, op, compensated, [&](auto *tp, auto *pp) -> bcx_status {
    typedef std::remove_pointer_t<decltype(tp)> T;
    typedef std::remove_pointer_t<decltype(pp)> P;
    return run_segmented_scan<T, P>((cudaStream_t)stream, type, exclusive, init_p, in, out, n, offs, nseg, temp,
                                    temp_bytes);
  });
  if (rc == BCX_UNSUPPORTED) set_error("segmented scan: dtype %d / functor %d not provided", int(type), int(op));
  return rc;
}

bcx_status bcx_segmented_reduce(bcx_stream stream, bcx_dtype type, bcx_op op, const void *in,
                                const uint64_t *offsets, size_t nseg, const void *init, void *out,
                                int compensated, void *temp, size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (nseg == 0) {
    if (temp == nullptr && temp_bytes != nullptr) *temp_bytes = 0;
    return BCX_SUCCESS;
  }
  BCX_CHECK(in && offsets && out && init, BCX_INVALID_VALUE, "NULL argument");
  const auto *offs = reinterpret_cast<const unsigned long long *>(offsets);
  bcx_status rc = seg_dispatch(type, op, compensated, [&](auto *tp, auto *pp) -> bcx_status {
    typedef std::remove_pointer_t<decltype(tp)> T;
    typedef std::remove_pointer_t<decltype(pp)> P;
    return run_segmented_reduce<T, P>((cudaStream_t)stream, type, in, offs, nseg, init, out, temp, temp_bytes);
  });
  if (rc == BCX_UNSUPPORTED)
    set_error("segmented reduce: dtype %d / functor %d not provided", int(type), int(op));
  return rc;
}

}  // extern "C"
