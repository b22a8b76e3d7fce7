// bcx_radix.cuh -- building blocks of the onesweep radix sort shared by the
// plain sort (bcx_sort.cu) and the segmented sort (bcx_segmented_sort.cu):
// the radix key transform, the per-tile look-back status words and the tile
// routine that ranks, stages and scatters one tile for one 8-bit digit.
#pragma once

#include <cuda_runtime.h>

#include "bcx_common.cuh"

namespace bcx {
namespace radix {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr int kHistThreads = 256;

// Status word of one (tile, digit): 2-bit flag above a 30-bit count.
constexpr uint32_t kStFlagShift = 30;
constexpr uint32_t kStValueMask = (1u << kStFlagShift) - 1;
constexpr uint32_t kStAggregate = 1u << kStFlagShift;
constexpr uint32_t kStPrefix = 2u << kStFlagShift;
constexpr size_t kMaxSortN = size_t(1) << 30;

enum KeyKind : int { kKeyUnsigned = 0, kKeySigned = 1, kKeyFloat = 2 };


// The radix() transform as four masks chosen on the host, so kernels apply it
// without branches: key = ((x ^ a) + b) ^ ((f & -(x >> sign)) | c).
//   ascending unsigned a=0  b=0 f=0  c=0        descending unsigned a=~0 b=0 f=0  c=0
//   ascending signed   a=0  b=0 f=0  c=sign     descending signed   a=~0 b=1 f=0  c=sign
//   ascending float    a=0  b=0 f=~0 c=sign     descending float    a=~0 b=1 f=~0 c=sign
// (~x + 1 is -x; the float mask is taken from x, as the reference does.)
template <class U>
struct KeyXform {
  U a, b, f, c;
};
template <class U>
KeyXform<U> make_xform(int kind, int desc) {
  const U sign = U(U(1) << (sizeof(U) * 8 - 1));
  KeyXform<U> x;
  x.a = desc ? U(~U(0)) : U(0);
  x.b = (desc && kind != kKeyUnsigned) ? U(1) : U(0);
  x.f = kind == kKeyFloat ? U(~U(0)) : U(0);
  x.c = kind == kKeyUnsigned ? U(0) : sign;
  return x;
}
template <class U>
__device__ __forceinline__ U apply_xform(U x, const KeyXform<U> &t) {
  constexpr int kSign = int(sizeof(U) * 8 - 1);
  return U(U(U(x ^ t.a) + t.b) ^ U((t.f & U(U(0) - U(x >> kSign))) | t.c));
}

template <int VB> struct value_type_of;
template <> struct value_type_of<0> { typedef uint8_t type; };
template <> struct value_type_of<1> { typedef uint8_t type; };
template <> struct value_type_of<2> { typedef uint16_t type; };
template <> struct value_type_of<4> { typedef uint32_t type; };
template <> struct value_type_of<8> { typedef unsigned long long type; };
template <> struct value_type_of<16> { typedef uint4 type; };

template <class U> struct items_per_thread { static constexpr int value = 16; };
template <> struct items_per_thread<unsigned long long> { static constexpr int value = 12; };

// Device-side control block written by the prep kernel.
struct SortControl {
  uint32_t skip[8];     // pass p moves nothing (all keys share its digit)
  uint32_t src_alt[8];  // pass p reads the temporary buffers
  uint32_t final_alt;   // the sorted data ended in the temporary buffers
  uint32_t pad[47];
};
static_assert(sizeof(SortControl) == 256, "control block is 256 bytes");

// One onesweep tile.
//
// Order of work inside a tile is chosen so that a tile's inclusive digit
// prefixes become visible as early as possible (that is what bounds how far
// successors must look back): load, count digits with shared-memory atomics,
// publish the counts, look back (each thread one digit, kLookbackWindow
// predecessor words in flight at a time), publish the inclusive prefix, and
// only then rank keys stably and scatter them.
constexpr int kLookbackWindow = 4;


// Exclusive prefix of digit `d` over the tiles first_tile .. tile-1 (the
// tiles of the same sort, or of the same segment).  first_tile publishes its
// inclusive prefix without looking back, so the walk always ends there.
__device__ __forceinline__ uint32_t onesweep_lookback(const uint32_t *__restrict__ status, uint32_t tile,
                                                      uint32_t first_tile, unsigned d, bool *gave_up) {
  uint32_t excl = 0;
  const int64_t floor_t = int64_t(first_tile);
  int64_t t = int64_t(tile) - 1;
  while (t >= floor_t) {
    uint32_t w[kLookbackWindow];
#pragma unroll
    for (int j = 0; j < kLookbackWindow; ++j)
      w[j] = (t - j >= floor_t) ? ld_relaxed_u32(status + size_t(t - j) * kRadix + d) : kStPrefix;
    bool done = false;
#pragma unroll
    for (int j = 0; j < kLookbackWindow; ++j) {
      if (done) break;
      uint32_t x = w[j];
      uint32_t spins = 0;
      while ((x >> kStFlagShift) == 0) {
        if (++spins > kSpinLimit) {
          *gave_up = true;
          return excl;
        }
        __nanosleep(spins < 32 ? 16 : 128);
        x = ld_relaxed_u32(status + size_t(t - j) * kRadix + d);
      }
      excl += x & kStValueMask;
      done = (x >> kStFlagShift) == 2u;
    }
    if (done) break;
    t -= kLookbackWindow;
  }
  return excl;
}

// Shared-memory footprint of one onesweep block: per-warp digit counters,
// keys and values in load order, the load index and digit of every staged
// position in digit order.
template <class U, int VB>
struct OnesweepSmem {
  typedef typename value_type_of<VB>::type VT;
  static constexpr int IPT = items_per_thread<U>::value;
  static constexpr int TILE = kSortThreads * IPT;
  static constexpr size_t kCounters = size_t(kSortWarps) * kRadix * 4;
  static constexpr size_t kKeys = kCounters;
  static constexpr size_t kVals = kKeys + size_t(TILE) * sizeof(U);
  static constexpr size_t kPerm = kVals + (VB ? size_t(TILE) * sizeof(VT) : 0);
  static constexpr size_t kDigit = kPerm + size_t(TILE) * 2;
  static constexpr size_t kBytes = kDigit + size_t(TILE);
};

// Sorts one tile of `count` elements starting at `base` by the digit at
// `shift` into dst: element of digit d goes to digit_start[d] + (elements of
// digit d in tiles first_tile .. tile-1) + (its stable rank in this tile).
// Status row `tile` of `status` is this tile's look-back word per digit.
// Called by every thread of a kSortThreads block after a barrier.
template <class U, int VB>
__device__ __forceinline__ void onesweep_tile(const U *__restrict__ src_k, U *__restrict__ dst_k,
                                              const typename value_type_of<VB>::type *__restrict__ src_v,
                                              typename value_type_of<VB>::type *__restrict__ dst_v,
                                              uint32_t base, uint32_t count, uint32_t tile, uint32_t first_tile,
                                              const uint32_t *__restrict__ digit_start, uint32_t dst_limit,
                                              int shift, const KeyXform<U> &xf, uint32_t *__restrict__ status,
                                              uint32_t *err) {
  typedef OnesweepSmem<U, VB> L;
  typedef typename L::VT VT;
  constexpr int IPT = L::IPT;
  constexpr int TILE = L::TILE;
  static_assert(kSortThreads == kRadix, "one thread per digit");
  static_assert(TILE <= 65536, "16-bit load indices");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t *wcnt = reinterpret_cast<uint32_t *>(smem_raw);  // [kSortWarps][kRadix]
  U *s_keys = reinterpret_cast<U *>(smem_raw + L::kKeys);    // load order
  VT *s_vals = reinterpret_cast<VT *>(smem_raw + L::kVals);  // load order
  uint16_t *s_perm = reinterpret_cast<uint16_t *>(smem_raw + L::kPerm);  // digit order -> load index
  uint8_t *s_digit = smem_raw + L::kDigit;                                  // digit order -> digit
  __shared__ uint32_t s_hist[kRadix];
  __shared__ uint32_t s_local_start[kRadix];
  __shared__ uint32_t s_adj[kRadix];  // global base - local start, per digit
  __shared__ uint32_t s_warp_sum[kSortWarps];

  const unsigned tid = threadIdx.x, lane = lane_id(), warp = tid / kWarp;
  for (int i = lane; i < kRadix; i += kWarp) wcnt[warp * kRadix + i] = 0;
  s_hist[tid] = 0;
  __syncthreads();
  const uint32_t tile_base = base;
  const uint32_t warp_first = warp * (kWarp * IPT);  // tile-local index of this warp's first item

  // Load warp-striped (item i of lane l is tile element warp_first + i*32 + l,
  // so (i, l) order is input order), stage in shared memory in that order,
  // and count digits.
  uint32_t dr[IPT];  // digit | rank-within-warp << 8 | invalid << 31
  const bool full = count == uint32_t(TILE);
  if (full) {
    U key[IPT];
#pragma unroll
    for (int i = 0; i < IPT; ++i) key[i] = src_k[tile_base + warp_first + i * kWarp + lane];
    if (VB) {
      VT val[VB ? IPT : 1];
#pragma unroll
      for (int i = 0; i < IPT; ++i) val[i] = src_v[tile_base + warp_first + i * kWarp + lane];
#pragma unroll
      for (int i = 0; i < IPT; ++i) s_vals[warp_first + i * kWarp + lane] = val[i];
    }
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      s_keys[warp_first + i * kWarp + lane] = key[i];
      dr[i] = uint32_t(apply_xform<U>(key[i], xf) >> shift) & (kRadix - 1);
      atomicAdd(&s_hist[dr[i]], 1u);
    }
  } else {
    U key[IPT];
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const uint32_t idx = tile_base + warp_first + i * kWarp + lane;
      key[i] = idx < tile_base + count ? src_k[idx] : U(0);
    }
    if (VB) {
      VT val[VB ? IPT : 1];
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const uint32_t idx = tile_base + warp_first + i * kWarp + lane;
        if (idx < tile_base + count) val[i] = src_v[idx];
      }
#pragma unroll
      for (int i = 0; i < IPT; ++i) s_vals[warp_first + i * kWarp + lane] = val[i];
    }
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const uint32_t li = warp_first + i * kWarp + lane;
      s_keys[li] = key[i];
      if (li < count) {
        dr[i] = uint32_t(apply_xform<U>(key[i], xf) >> shift) & (kRadix - 1);
        atomicAdd(&s_hist[dr[i]], 1u);
      } else {
        dr[i] = 0x80000000u;
      }
    }
  }
  __syncthreads();

  // Thread `tid` owns digit `tid`: publish, local start, look-back.
  const uint32_t tile_cnt = s_hist[tid];
  uint32_t *my_status = status + size_t(tile) * kRadix + tid;
  st_relaxed_u32(my_status, (tile == first_tile ? kStPrefix : kStAggregate) | tile_cnt);
  uint32_t incl = tile_cnt;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (int(lane) >= o) incl += t;
  }
  if (lane == kWarp - 1) s_warp_sum[warp] = incl;
  uint32_t excl = 0;
  if (tile > first_tile) {
    bool gave_up = false;
    excl = onesweep_lookback(status, tile, first_tile, tid, &gave_up);
    if (gave_up) report_error(err, kErrLookbackTimeout);
    st_relaxed_u32(my_status, kStPrefix | ((excl + tile_cnt) & kStValueMask));
  }
  __syncthreads();
  {
    uint32_t before = 0;
    for (unsigned j = 0; j < warp; ++j) before += s_warp_sum[j];
    const uint32_t local_start = before + incl - tile_cnt;
    s_local_start[tid] = local_start;
    s_adj[tid] = digit_start[tid] + excl - local_start;
  }

  // Stable rank within the warp: per item, the lanes holding the same digit
  // are found with eight ballots (one per digit bit); the lowest such lane
  // advances the warp's counter for that digit and every lane adds the count
  // of same-digit lanes below it.
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const bool valid = !(dr[i] & 0x80000000u);
    const uint32_t d = dr[i] & 0xffu;
    unsigned grp = full ? 0xffffffffu : __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b) {
      const bool bit = (d >> b) & 1u;
      const unsigned v = __ballot_sync(0xffffffffu, bit);
      grp &= bit ? v : ~v;
    }
    const int leader = __ffs(grp) - 1;
    uint32_t old = 0;
    if (valid && int(lane) == leader) {
      old = wcnt[warp * kRadix + d];
      wcnt[warp * kRadix + d] = old + __popc(grp);
    }
    old = __shfl_sync(0xffffffffu, old, valid ? leader : int(lane));
    if (valid) dr[i] = d | ((old + __popc(grp & lt)) << 8);
    __syncwarp();
  }
  __syncthreads();
  // Exclusive prefix of each digit's count across warps.
  {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = wcnt[w * kRadix + tid];
      wcnt[w * kRadix + tid] = run;
      run += c;
    }
  }
  __syncthreads();

  // Digit-order position of every item: record its load index and digit.
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    if (!(dr[i] & 0x80000000u)) {
      const uint32_t d = dr[i] & 0xffu;
      const uint32_t pos = s_local_start[d] + wcnt[warp * kRadix + d] + (dr[i] >> 8);
      s_perm[pos] = uint16_t(warp_first + i * kWarp + lane);
      s_digit[pos] = uint8_t(d);
    }
  }
  __syncthreads();

  // Write out: consecutive threads take consecutive digit-order positions, so
  // each digit's run is written to consecutive addresses.
  const uint32_t tile_valid = count;
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const uint32_t idx = k * kSortThreads + tid;
    if (full || idx < tile_valid) {
      const uint32_t li = s_perm[idx];
      const uint32_t dst = s_adj[s_digit[idx]] + idx;
      // Always in range unless a look-back wait gave up (then the error word
      // is set and the output is garbage, but no write leaves the buffer).
      if (dst < dst_limit) {
        dst_k[dst] = s_keys[li];
        if (VB) dst_v[dst] = s_vals[li];
      }
    }
  }
}


}  // namespace radix
}  // namespace bcx
