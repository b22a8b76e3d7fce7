// bcx_reduce_by_key.cu -- reduce_by_key in one pass over HBM.
//
// Reference: reduce_by_key (algorithm/reduce_by_key.hpp,
// algorithm/detail/reduce_by_key.hpp:66-113) -> reduce_by_key_with_scan
// (algorithm/detail/reduce_by_key_with_scan.hpp:432-486): a key-change flag
// kernel plus an inclusive_scan to number the runs (:53-100), per-group
// carry-outs (:105-180), carry-ins (:182-270) and a final Hillis-Steele
// reduction by key (:272-400), then a blocking read of the run count.
//
// GB300 design: one kernel.  The operation is a segmented scan whose element
// is (head?, run count, value) and whose combine (a then b) is
//   (a.count + b.count, a.head | b.head, b.head ? b.value : a.value op b.value).
// Each block takes the next tile from an atomic ticket.  In every chunk a lane
// owns a run of consecutive elements (vector loads, coalesced across the
// warp): it derives head flags from the previous key, folds its run serially,
// and one warp scan per chunk combines the lanes' folds.  Only the head flags
// and the per-chunk prefixes (in shared memory) are kept; warps combine
// through shared memory, the tile with its predecessors by decoupled
// look-back (order-preserving, bounded waits, self-validating status words
// where the value allows), and a second read (from L2), by only the lanes
// whose run holds a run head or a run end, emits the results: run heads write
// the output key, run ends the reduced value, and the block holding the last
// element writes the run count -- nothing is read back to the host.  Key
// equality is the typed == of equal_to<T>.  Float plus with compensated=1
// carries Neumaier (s, c) pairs.
#include <cuda_runtime.h>

#include <type_traits>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"

namespace bcx {
namespace {

constexpr int kRbkThreads = 256;
constexpr int kRbkWarps = kRbkThreads / kWarp;
constexpr uint32_t kHeadBit = 0x80000000u;
constexpr uint32_t kCountMask = 0x7fffffffu;
enum : uint32_t { kRbInvalid = 0, kRbAggregate = 1, kRbPrefix = 2 };

// Value policies.
template <class V, template <class> class OpT>
struct RbPlain {
  typedef typename widen<V>::type Acc;
  typedef OpT<Acc> Op;
  __device__ __forceinline__ static Acc ident() { return Op::identity(); }
  __device__ __forceinline__ static Acc from(V x) { return Acc(x); }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return Op()(a, b); }
  __device__ __forceinline__ static Acc add1(Acc a, V x) { return Op()(a, Acc(x)); }
  __device__ __forceinline__ static V out(Acc a) { return V(a); }
  __device__ __forceinline__ static Acc shfl_up(Acc a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
  __device__ __forceinline__ static Acc shfl_down(Acc a, int d) { return __shfl_down_sync(0xffffffffu, a, d); }
  __device__ __forceinline__ static Acc shfl(Acc a, int s) { return __shfl_sync(0xffffffffu, a, s); }
};
struct RbCompF32 {
  typedef comp_f32 Acc;
  __device__ __forceinline__ static Acc ident() { return comp_f32{0.f, 0.f}; }
  __device__ __forceinline__ static Acc from(float x) { return comp_f32{x, 0.f}; }
  __device__ __forceinline__ static Acc comb(Acc a, Acc b) { return comp_merge(a, b); }
  __device__ __forceinline__ static Acc add1(Acc a, float x) { return comp_add(a, x); }
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

// (head flag | run count, value) triple and its order-preserving combine.
template <class P>
struct Seg {
  uint32_t c;  // kHeadBit | count of heads
  typename P::Acc v;
};
template <class P>
__device__ __forceinline__ Seg<P> seg_comb(const Seg<P> &a, const Seg<P> &b) {
  Seg<P> r;
  r.c = ((a.c & kCountMask) + (b.c & kCountMask)) | ((a.c | b.c) & kHeadBit);
  r.v = (b.c & kHeadBit) ? b.v : P::comb(a.v, b.v);
  return r;
}
template <class P>
__device__ __forceinline__ Seg<P> seg_ident() {
  return Seg<P>{0u, P::ident()};
}

// a then one element x: a head restarts the run with x (and counts a run),
// otherwise x is folded into the running value.
template <class P, class V>
__device__ __forceinline__ void seg_push(Seg<P> &a, bool head, V x) {
  if (head) {
    a.c = ((a.c & kCountMask) + 1u) | kHeadBit;
    a.v = P::from(x);
  } else {
    a.v = P::add1(a.v, x);
  }
}

// Look-back status of one tile, published twice (aggregate, then inclusive
// prefix).  Every word starts as all ones ("unset") and is written once, so a
// relaxed load sees either "unset" or the final value and no fence is needed:
//   kind 1 (4-byte values): run count word and value share one 64-bit word;
//          a count of all ones cannot occur below 2^31 - 1 elements;
//   kind 2 (double, and compensated float carried as the FP64 sum of its
//          pair): a count word plus a 64-bit value word whose all-ones pattern
//          is a NaN GPU arithmetic never produces (computed NaNs are
//          canonical); a poll is ready when both are set;
//   kind 0 (8-byte integers, where every bit pattern is a value): a flag word
//          plus aggregate/inclusive arrays ordered by release/acquire.
template <class P>
struct RbStatusKind {
  typedef typename P::Acc Acc;
  static constexpr int value = sizeof(Acc) == 4                          ? 1
                               : std::is_same<Acc, double>::value        ? 2
                               : std::is_same<Acc, comp_f32>::value      ? 2
                                                                         : 0;
};

template <class P, int KIND = RbStatusKind<P>::value>
struct RbStatus;

template <class P>
struct RbStatus<P, 0> {
  uint32_t *flags;
  Seg<P> *agg;
  Seg<P> *inc;
  static size_t bytes(size_t tiles) { return align256(tiles * 4) + 2 * align256(tiles * sizeof(Seg<P>)); }
  void bind(char *base, size_t tiles) {
    flags = reinterpret_cast<uint32_t *>(base);
    agg = reinterpret_cast<Seg<P> *>(base + align256(tiles * 4));
    inc = reinterpret_cast<Seg<P> *>(base + align256(tiles * 4) + align256(tiles * sizeof(Seg<P>)));
  }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(flags, 0, align256(tiles * 4), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, const Seg<P> &s) {
    if (flag == kRbAggregate) agg[t] = s;
    else inc[t] = s;
    st_release_u32(&flags[t], flag);
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Seg<P> *s) const {
    uint32_t f = ld_acquire_u32(&flags[t]);
    if (f != kRbInvalid) {
      const Seg<P> *src = (f == kRbAggregate) ? &agg[t] : &inc[t];
      const volatile uint32_t *w = reinterpret_cast<const volatile uint32_t *>(src);
      uint32_t tmp[sizeof(Seg<P>) / 4];
#pragma unroll
      for (int i = 0; i < int(sizeof(Seg<P>) / 4); ++i) tmp[i] = w[i];
      memcpy(s, tmp, sizeof(Seg<P>));
    }
    return f;
  }
};

template <class P>
struct RbStatus<P, 1> {
  unsigned long long *agg;
  unsigned long long *inc;
  static size_t bytes(size_t tiles) { return 2 * align256(tiles * 8); }
  void bind(char *base, size_t tiles) {
    agg = reinterpret_cast<unsigned long long *>(base);
    inc = reinterpret_cast<unsigned long long *>(base + align256(tiles * 8));
  }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(agg, 0xff, bytes(tiles), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, const Seg<P> &s) {
    uint32_t vb;
    memcpy(&vb, &s.v, 4);
    const unsigned long long w = (static_cast<unsigned long long>(vb) << 32) | s.c;
    unsigned long long *dst = flag == kRbAggregate ? &agg[t] : &inc[t];
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(dst), "l"(w) : "memory");
  }
  __device__ __forceinline__ static bool unpack(unsigned long long w, Seg<P> *s) {
    if (uint32_t(w) == 0xffffffffu) return false;
    s->c = uint32_t(w);
    const uint32_t vb = uint32_t(w >> 32);
    memcpy(&s->v, &vb, 4);
    return true;
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Seg<P> *s) const {
    const unsigned long long wi = ld_relaxed_u64(&inc[t]);
    const unsigned long long wa = ld_relaxed_u64(&agg[t]);
    if (unpack(wi, s)) return kRbPrefix;
    if (unpack(wa, s)) return kRbAggregate;
    return kRbInvalid;
  }
};

// FP64 view of a value (the compensated pair as its exact-in-double sum).
__device__ __forceinline__ double rb_to_f64(double v) { return v; }
__device__ __forceinline__ double rb_to_f64(comp_f32 v) { return double(v.s) + double(v.c); }
__device__ __forceinline__ void rb_from_f64(double d, double *v) { *v = d; }
__device__ __forceinline__ void rb_from_f64(double d, comp_f32 *v) {
  v->s = float(d);
  v->c = float(d - double(v->s));
}

template <class P>
struct RbStatus<P, 2> {
  uint32_t *agg_c;
  uint32_t *inc_c;
  unsigned long long *agg_v;
  unsigned long long *inc_v;
  static size_t bytes(size_t tiles) { return 2 * align256(tiles * 4) + 2 * align256(tiles * 8); }
  void bind(char *base, size_t tiles) {
    agg_c = reinterpret_cast<uint32_t *>(base);
    inc_c = reinterpret_cast<uint32_t *>(base + align256(tiles * 4));
    agg_v = reinterpret_cast<unsigned long long *>(base + 2 * align256(tiles * 4));
    inc_v = reinterpret_cast<unsigned long long *>(base + 2 * align256(tiles * 4) + align256(tiles * 8));
  }
  cudaError_t clear(size_t tiles, cudaStream_t s) const { return cudaMemsetAsync(agg_c, 0xff, bytes(tiles), s); }
  __device__ __forceinline__ void publish(size_t t, uint32_t flag, const Seg<P> &s) {
    const double d = rb_to_f64(s.v);
    unsigned long long w;
    memcpy(&w, &d, 8);
    uint32_t *dc = flag == kRbAggregate ? &agg_c[t] : &inc_c[t];
    unsigned long long *dv = flag == kRbAggregate ? &agg_v[t] : &inc_v[t];
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(dv), "l"(w) : "memory");
    st_relaxed_u32(dc, s.c);
  }
  __device__ __forceinline__ static bool take(uint32_t c, unsigned long long w, Seg<P> *s) {
    if (c == 0xffffffffu || w == ~0ull) return false;
    double d;
    memcpy(&d, &w, 8);
    s->c = c;
    rb_from_f64(d, &s->v);
    return true;
  }
  __device__ __forceinline__ uint32_t poll(size_t t, Seg<P> *s) const {
    const uint32_t ci = ld_relaxed_u32(&inc_c[t]);
    const unsigned long long wi = ld_relaxed_u64(&inc_v[t]);
    const uint32_t ca = ld_relaxed_u32(&agg_c[t]);
    const unsigned long long wa = ld_relaxed_u64(&agg_v[t]);
    if (take(ci, wi, s)) return kRbPrefix;
    if (take(ca, wa, s)) return kRbAggregate;
    return kRbInvalid;
  }
};

template <class K>
__device__ __forceinline__ bool keys_equal(K a, K b) { return a == b; }

// Tile shape: every lane owns N consecutive elements per chunk (8 elements:
// 32 bytes of 4-byte keys and values, 64 bytes of 8-byte ones; vector loads
// when aligned), CH chunks per thread, EPT elements per thread in all.  Long
// per-lane runs keep most of the work in the serial per-lane fold and the
// warp scans (one per chunk) few; measured on GB300 with compensated float
// values, 16 elements per thread in 4-element runs took 1.77x as long.
//
// Values are loaded VG at a time (keys whole, so the previous lane's last key
// is at hand for the first head flag), which keeps fewer registers live, and
// 4-byte keys and values run 8 blocks per SM.  The workload is latency-bound
// (per-tile loads and look-back), so resident warps matter most: 10,000
// segment-id runs over 9.5e8 int keys with compensated float values on GB300,
// 4 blocks per SM with whole runs 2.97 ms, 6 blocks 2.69 ms, 6 blocks with
// values 8 at a time 2.59 ms (4 at a time 2.70; 8 blocks per SM spill heavily,
// 3.8 ms), 2.52 ms with the lanes' chunk prefixes kept in shared memory,
// 2.48 ms with the chunk loops rolled (fewer spills; runs of ~4 keys 3.01 ->
// 2.65 ms), and 2.31 ms with 8-element lane runs (4 chunks a thread, 32
// registers: 8 blocks per SM; runs of ~4 keys 2.38 ms).  Without its
// look-back that kernel took 1.39 ms: the waits for predecessor tiles are
// what remain, so 4-byte keys and values take 64 elements per thread (tiles
// of 16384, half the look-backs per element): 2.16 ms (runs of ~4 keys
// 2.19 ms).
template <class K, class V>
struct RbkShape {
  static constexpr int W = sizeof(K) > sizeof(V) ? int(sizeof(K)) : int(sizeof(V));
  static constexpr int N = W == 4 ? 8 : 64 / W;
  static constexpr int EPT = W == 4 ? 64 : 32;  // elements per thread
  static constexpr int CH = EPT / N;
  static constexpr int TILE = kRbkThreads * N * CH;
  static constexpr int VG = N / 2;
  static constexpr int BLOCKS_PER_SM = W == 4 ? 8 : 4;
  typedef typename std::conditional<(N * CH > 32), unsigned long long, uint32_t>::type HeadMask;
  static_assert(N * CH <= 64, "head flags of a thread fit one 64-bit mask");
};

template <class T, int N>
struct alignas(sizeof(T) * N) VecN {
  T v[N];
};

// Elements e0 .. e0+N-1 (e0 a multiple of N): one vector load when the array
// is aligned to the vector and the run is in range, else element loads.
template <class T, int N>
__device__ __forceinline__ void load_run(const T *__restrict__ p, size_t e0, size_t n, bool vec, T (&x)[N]) {
  if (vec && e0 + N <= n) {
    const VecN<T, N> w = *reinterpret_cast<const VecN<T, N> *>(p + e0);
#pragma unroll
    for (int m = 0; m < N; ++m) x[m] = w.v[m];
  } else {
#pragma unroll
    for (int m = 0; m < N; ++m) x[m] = (e0 + m < n) ? p[e0 + m] : T(0);
  }
}

// Bytes ahead of a tile whose keys and values are prefetched into L2.  At 8
// blocks per SM of 128 KB tiles about 155 MB of input is in flight, more than
// L2 holds, so a short distance keeps prefetched lines from being evicted
// before their tile reads them.
constexpr size_t kRbkPrefetchBytes = kL2PrefetchBytes;

template <class K, class V, class P>
__global__ void __launch_bounds__(kRbkThreads, RbkShape<K, V>::BLOCKS_PER_SM)
reduce_by_key_kernel(const K *__restrict__ keys, const V *__restrict__ vals, uint32_t n,
                     K *__restrict__ keys_out, V *__restrict__ vals_out,
                     unsigned long long *__restrict__ num_runs, RbStatus<P> st,
                     uint32_t *__restrict__ tile_counter, int single, int vec_k, int vec_v, uint32_t *err) {
  typedef Seg<P> S;
  typedef RbkShape<K, V> Sh;
  constexpr int N = Sh::N;
  constexpr int CH = Sh::CH;
  constexpr int VG = Sh::VG;
  __shared__ S s_warp[kRbkWarps];
  __shared__ S s_prefix;
  __shared__ uint32_t s_tile;
  // Fold of everything before the lane's run in chunk j (within the warp),
  // kept in shared memory across the look-back rather than in registers;
  // only the owning thread reads its entry back.
  __shared__ S s_lane_pre[CH][kRbkThreads];
  const unsigned lane = lane_id(), warp = threadIdx.x / kWarp;
  uint32_t tile = 0;
  if (!single) {
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    tile = s_tile;
    // Ask L2 for the keys and values of the tile kRbkPrefetchBytes ahead, so
    // that tile's first read is served from L2 (short, even load times keep
    // the look-back waits short).
    if (kRbkPrefetchBytes > 0 && threadIdx.x == 0) {
      const size_t ahead =
          (size_t(tile) + kRbkPrefetchBytes / (size_t(Sh::TILE) * (sizeof(K) + sizeof(V)))) * size_t(Sh::TILE);
      if ((reinterpret_cast<uintptr_t>(keys) & 15u) == 0) prefetch_l2_range(keys, ahead, Sh::TILE, n);
      if ((reinterpret_cast<uintptr_t>(vals) & 15u) == 0) prefetch_l2_range(vals, ahead, Sh::TILE, n);
    }
  }
  // Warp w covers CH chunks of 32*N consecutive elements; in chunk j lane l
  // owns elements chunk_base + l*N .. + N-1, so (j, l, m) is input order.
  const size_t warp_base = size_t(tile) * Sh::TILE + size_t(warp) * (CH * kWarp * N);

  // Pass 1 over the tile: head flags (in a register) and per-chunk prefixes
  // (in shared memory).  Only those are kept across the look-back; pass 2
  // reads the keys and values again (they were read microseconds earlier, so
  // from L2) to emit the results.
  typename Sh::HeadMask heads = 0;  // bit j*N+m = element (j, m) starts a run
  S run = seg_ident<P>();
  K carry_key = (warp_base > 0 && warp_base - 1 < n) ? keys[warp_base - 1] : K(0);  // key before chunk j
  // The chunk loops stay rolled: one chunk's registers live at a time keeps
  // the spills of the 32-register (8 blocks per SM) budget small.
#pragma unroll 1
  for (int j = 0; j < CH; ++j) {
    const size_t e0 = warp_base + size_t(j) * kWarp * N + lane * N;
    K k[N];
    load_run<K, N>(keys, e0, n, vec_k != 0, k);
    K prev = __shfl_up_sync(0xffffffffu, k[N - 1], 1);
    if (lane == 0) prev = carry_key;
    carry_key = __shfl_sync(0xffffffffu, k[N - 1], kWarp - 1);
    S a = seg_ident<P>();
#pragma unroll
    for (int g0 = 0; g0 < N; g0 += VG) {
      V v[VG];
      load_run<V, VG>(vals, e0 + g0, n, vec_v != 0, v);
#pragma unroll
      for (int mm = 0; mm < VG; ++mm) {
        const int m = g0 + mm;
        const size_t idx = e0 + m;
        const K p = m > 0 ? k[m - 1] : prev;
        const bool h = idx < n && (idx == 0 || !keys_equal(p, k[m]));
        heads |= typename Sh::HeadMask(h) << (j * N + m);
        if (idx < n) seg_push<P>(a, h, v[mm]);
      }
    }
    S x = a;
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
      S o;
      o.c = __shfl_up_sync(0xffffffffu, x.c, d);
      o.v = P::shfl_up(x.v, d);
      if (int(lane) >= d) x = seg_comb<P>(o, x);
    }
    S ex;
    ex.c = __shfl_up_sync(0xffffffffu, x.c, 1);
    ex.v = P::shfl_up(x.v, 1);
    s_lane_pre[j][threadIdx.x] = lane == 0 ? run : seg_comb<P>(run, ex);
    S tot;
    tot.c = __shfl_sync(0xffffffffu, x.c, kWarp - 1);
    tot.v = P::shfl(x.v, kWarp - 1);
    run = seg_comb<P>(run, tot);
  }
  if (lane == 0) s_warp[warp] = run;
  __syncthreads();
  S warp_excl = seg_ident<P>(), tile_agg = seg_ident<P>();
#pragma unroll
  for (int w = 0; w < kRbkWarps; ++w) {
    if (w == int(warp)) warp_excl = tile_agg;
    tile_agg = seg_comb<P>(tile_agg, s_warp[w]);
  }
  if (single) {
    if (threadIdx.x == 0) s_prefix = seg_ident<P>();
  } else if (warp == 0) {
    S excl = seg_ident<P>();
    if (tile == 0) {
      if (lane == 0) st.publish(0, kRbPrefix, tile_agg);
    } else {
      if (lane == 0) st.publish(tile, kRbAggregate, tile_agg);
      int64_t pred = int64_t(tile) - 1;
      bool gave_up = false;
      while (true) {
        const int64_t t = pred - int64_t(lane);
        S val = seg_ident<P>();
        uint32_t f = kRbPrefix;
        if (t >= 0) {
          uint32_t spins = 0;
          f = st.poll(size_t(t), &val);
          while (f == kRbInvalid) {
            if (++spins > kSpinLimit) {
              gave_up = true;
              f = kRbPrefix;
              val = seg_ident<P>();
              break;
            }
            if (spins > 16) __nanosleep(64);
            f = st.poll(size_t(t), &val);
          }
        }
        const unsigned pmask = __ballot_sync(0xffffffffu, f == kRbPrefix);
        const int first = pmask ? __ffs(pmask) - 1 : kWarp - 1;
        if (int(lane) > first) val = seg_ident<P>();
        // Order-preserving fold: higher lanes are earlier tiles.
#pragma unroll
        for (int d = 1; d < kWarp; d <<= 1) {
          S o;
          o.c = __shfl_down_sync(0xffffffffu, val.c, d);
          o.v = P::shfl_down(val.v, d);
          if (int(lane) + d < kWarp) val = seg_comb<P>(o, val);
        }
        S window;
        window.c = __shfl_sync(0xffffffffu, val.c, 0);
        window.v = P::shfl(val.v, 0);
        excl = seg_comb<P>(window, excl);
        if (pmask) break;
        pred -= kWarp;
      }
      if (__any_sync(0xffffffffu, gave_up) && lane == 0) report_error(err, kErrLookbackTimeout);
      if (lane == 0) st.publish(tile, kRbPrefix, seg_comb<P>(excl, tile_agg));
    }
    if (lane == 0) s_prefix = excl;
  }
  __syncthreads();
  // Pass 2: run heads write their key, run ends their reduced value.
  const S pre = seg_comb<P>(s_prefix, warp_excl);
  const size_t warp_end = warp_base + size_t(CH) * kWarp * N;  // first element after this warp
  const bool after_head = lane == kWarp - 1 && warp_end < n && !keys_equal(keys[warp_end], carry_key);
  // A lane re-reads and re-folds its run of chunk j only if the run holds a
  // run head (its key is written) or a run end (its value is written); with
  // long runs (segment ids as keys) almost every lane skips both.  The fold
  // order is unchanged, so results are identical.
  constexpr uint32_t kRunMask = N >= 32 ? 0xffffffffu : ((1u << N) - 1u);
#pragma unroll 1
  for (int j = 0; j < CH; ++j) {
    const size_t e0 = warp_base + size_t(j) * kWarp * N + lane * N;
    // head flag of the element after this lane's run in chunk j
    const uint32_t h_next_lane = uint32_t(__shfl_down_sync(0xffffffffu, heads >> (j * N), 1)) & 1u;
    const uint32_t h_next_chunk =
        uint32_t(__shfl_sync(0xffffffffu, heads >> (j + 1 < CH ? (j + 1) * N : 0), 0)) & 1u;
    uint32_t next_h = h_next_lane;
    if (lane == kWarp - 1) next_h = j + 1 < CH ? h_next_chunk : uint32_t(after_head);
    const uint32_t hj = uint32_t(heads >> (j * N)) & kRunMask;
    // run ends: the next element is a head, or the element is the last one
    uint32_t ends = (hj >> 1) | (next_h << (N - 1));
    if (e0 >= n) {
      ends = 0;
    } else if (n - e0 <= size_t(N)) {
      ends |= 1u << (n - e0 - 1);
      ends &= n - e0 >= 32 ? 0xffffffffu : ((1u << (n - e0)) - 1u);
    }
    if (((hj & (keys_out ? kRunMask : 0u)) | ends) == 0) continue;
    S acc = seg_comb<P>(pre, s_lane_pre[j][threadIdx.x]);
#pragma unroll
    for (int g0 = 0; g0 < N; g0 += VG) {
      K k[VG];
      V v[VG];
      load_run<K, VG>(keys, e0 + g0, n, vec_k != 0, k);
      load_run<V, VG>(vals, e0 + g0, n, vec_v != 0, v);
#pragma unroll
      for (int mm = 0; mm < VG; ++mm) {
        const int m = g0 + mm;
        const size_t idx = e0 + m;
        const bool h = (hj >> m) & 1u;
        if (idx < n) {
          seg_push<P>(acc, h, v[mm]);
          const uint32_t run_idx = (acc.c & kCountMask) - 1u;
          const bool last = (ends >> m) & 1u;
          if (h && keys_out) keys_out[run_idx] = k[mm];
          if (last) vals_out[run_idx] = P::out(acc.v);
          if (idx + 1 == n) *num_runs = (unsigned long long)(acc.c & kCountMask);
        }
      }
    }
  }
}

template <class K, class V, class P>
bcx_status run_rbk(cudaStream_t s, const void *keys, const void *vals, size_t n, void *keys_out,
                   void *vals_out, uint64_t *num_runs, void *temp, size_t *temp_bytes) {
  typedef Seg<P> S;
  typedef RbkShape<K, V> Sh;
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const size_t tiles = div_up(n, size_t(Sh::TILE));
  const bool single = tiles <= 1;
  typedef RbStatus<P> Status;
  const size_t need = single ? 0 : 256 + Status::bytes(tiles);
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, need, s, &query);
  if (rc || query) return rc;
  Status st{};
  uint32_t *counter = nullptr;
  if (!single) {
    char *base = static_cast<char *>(ts.ptr());
    counter = reinterpret_cast<uint32_t *>(base);
    st.bind(base + 256, tiles);
    BCX_CUDA(cudaMemsetAsync(base, 0, 256, s));
    BCX_CUDA(st.clear(tiles, s));
  }
  const int vec_k = reinterpret_cast<uintptr_t>(keys) % (sizeof(K) * Sh::N) == 0;
  const int vec_v = reinterpret_cast<uintptr_t>(vals) % (sizeof(V) * Sh::N) == 0;
  KernelScope ks("reduce_by_key", s);
  reduce_by_key_kernel<K, V, P><<<unsigned(tiles), kRbkThreads, 0, s>>>(
      static_cast<const K *>(keys), static_cast<const V *>(vals), uint32_t(n), static_cast<K *>(keys_out),
      static_cast<V *>(vals_out), reinterpret_cast<unsigned long long *>(num_runs), st, counter,
      single ? 1 : 0, vec_k, vec_v, ds->err_word);
  return launch_status("reduce_by_key");
}

template <class K, class V>
bcx_status rbk_op(cudaStream_t s, int op, int comp, const void *k, const void *v, size_t n, void *ko,
                  void *vo, uint64_t *nr, void *temp, size_t *tb) {
  switch (op) {
    case BCX_PLUS:
      if constexpr (sizeof(V) == 4 && type_traits<V>::is_float) {
        if (comp) return run_rbk<K, V, RbCompF32>(s, k, v, n, ko, vo, nr, temp, tb);
      }
      return run_rbk<K, V, RbPlain<V, op_plus>>(s, k, v, n, ko, vo, nr, temp, tb);
    case BCX_MULTIPLIES: return run_rbk<K, V, RbPlain<V, op_multiplies>>(s, k, v, n, ko, vo, nr, temp, tb);
    case BCX_MIN: return run_rbk<K, V, RbPlain<V, op_min>>(s, k, v, n, ko, vo, nr, temp, tb);
    case BCX_MAX: return run_rbk<K, V, RbPlain<V, op_max>>(s, k, v, n, ko, vo, nr, temp, tb);
  }
  return BCX_UNSUPPORTED;
}

template <class K>
bcx_status rbk_val(cudaStream_t s, bcx_dtype vt, int op, int comp, const void *k, const void *v, size_t n,
                   void *ko, void *vo, uint64_t *nr, void *temp, size_t *tb) {
  switch (vt) {
    case BCX_INT: return rbk_op<K, int32_t>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    case BCX_UINT: return rbk_op<K, uint32_t>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    case BCX_LONG: return rbk_op<K, long long>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    case BCX_ULONG: return rbk_op<K, unsigned long long>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    case BCX_FLOAT: return rbk_op<K, float>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    case BCX_DOUBLE: return rbk_op<K, double>(s, op, comp, k, v, n, ko, vo, nr, temp, tb);
    default: break;
  }
  return BCX_UNSUPPORTED;
}

}  // namespace
}  // namespace bcx

extern "C" bcx_status bcx_reduce_by_key(bcx_stream stream, bcx_dtype key_type, bcx_dtype value_type,
                                        bcx_op op, const void *keys_in, const void *values_in, size_t n,
                                        void *keys_out, void *values_out, uint64_t *num_runs_dev,
                                        int compensated, void *temp, size_t *temp_bytes) {
  using namespace bcx;
  clear_error();
  BCX_CHECK(dtype_valid(key_type) && dtype_valid(value_type), BCX_INVALID_VALUE, "invalid dtype");
  BCX_CHECK(n < (size_t(1) << 31) - 1, BCX_INVALID_VALUE, "reduce_by_key: n must be below 2^31 - 1");
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) {
    if (temp == nullptr && temp_bytes != nullptr) {
      *temp_bytes = 0;
      return BCX_SUCCESS;
    }
    if (num_runs_dev) BCX_CUDA(cudaMemsetAsync(num_runs_dev, 0, sizeof(uint64_t), s));
    return BCX_SUCCESS;
  }
  BCX_CHECK(keys_in && values_in && values_out && num_runs_dev, BCX_INVALID_VALUE, "NULL argument");
  bcx_status rc = BCX_UNSUPPORTED;
  switch (key_type) {
    case BCX_INT: rc = rbk_val<int32_t>(s, value_type, op, compensated, keys_in, values_in, n, keys_out, values_out, num_runs_dev, temp, temp_bytes); break;
    case BCX_UINT: rc = rbk_val<uint32_t>(s, value_type, op, compensated, keys_in, values_in, n, keys_out, values_out, num_runs_dev, temp, temp_bytes); break;
    case BCX_LONG: rc = rbk_val<long long>(s, value_type, op, compensated, keys_in, values_in, n, keys_out, values_out, num_runs_dev, temp, temp_bytes); break;
    case BCX_ULONG: rc = rbk_val<unsigned long long>(s, value_type, op, compensated, keys_in, values_in, n, keys_out, values_out, num_runs_dev, temp, temp_bytes); break;
    case BCX_FLOAT: rc = rbk_val<float>(s, value_type, op, compensated, keys_in, values_in, n, keys_out, values_out, num_runs_dev, temp, temp_bytes); break;
    default: break;
  }
  if (rc == BCX_UNSUPPORTED)
    set_error("reduce_by_key: key dtype %d / value dtype %d / functor %d not provided", int(key_type),
              int(value_type), int(op));
  return rc;
}
