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
// Onesweep blocks resident per SM the register budget is sized for (64
// registers a thread at 256 threads; 53 KB of shared memory a block with
// 16-bit counters and uint32 values).  One pass over 2^28 uint32 pairs on
// GB300: 3 blocks 1.262 ms, 4 blocks 1.236 ms (values copied asynchronously).
constexpr int kSortBlocksPerSm = 4;
constexpr int kHistThreads = 256;

// Status word of one (tile, digit) during one digit pass: a tag in the high
// 32 bits and a count in the low 32 bits.  Tag 2p+1 (tag_aggregate(p)) means
// "this tile's count of the digit"; tag 2p+2 means "inclusive prefix of the
// digit over the tiles first_tile .. this tile".  A word with a smaller tag
// (zero from the memset, or a word left by an earlier pass of the same sort)
// is not yet published, so one zeroed status array serves every pass.
__host__ __device__ constexpr uint32_t tag_aggregate(int pass) { return 2u * uint32_t(pass) + 1u; }
// Sorts take n below 2^32: element indices, digit counts and prefixes are
// 32-bit (the reference's counters are uint, radix_sort.hpp:338-345).
constexpr size_t kMaxSortN = (size_t(1) << 32) - 1;

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

// Keys per thread of a onesweep tile.  Measured on GB300, one pass over 2^28
// uint32 pairs: 12 -> 1.64 ms, 16 -> 1.40, 20 -> 1.33, 24 -> 1.30, 28 -> 1.40,
// 32 -> 1.31 (ballot ranking, 3-4 blocks per SM).
template <class U> struct items_per_thread { static constexpr int value = 24; };
template <> struct items_per_thread<unsigned long long> { static constexpr int value = 12; };

// Device-side control block written by the prep kernel.
struct SortControl {
  uint32_t skip[8];     // pass p moves nothing (all keys share its digit)
  uint32_t src_alt[8];  // pass p reads the temporary buffers
  uint32_t final_alt;   // the sorted data ended in the temporary buffers
  uint32_t pad[47];
};
static_assert(sizeof(SortControl) == 256, "control block is 256 bytes");

// Predecessor status words read per look-back step.
constexpr int kLookbackWindow = 4;
// A tile asks L2 for the keys and values of the tile this many tickets ahead
// (about a third of the blocks resident at once).  One pass over 2^28 uint32
// pairs on GB300: none 1.302 ms, 152 tiles 1.271, 456 1.277, 912 1.316.
constexpr int kOnesweepPrefetchTiles = 152;

// Exclusive prefix of digit `d` over the tiles first_tile .. tile-1 (the
// tiles of the same sort, or of the same segment) in pass `pass`.  first_tile
// publishes its inclusive prefix without looking back, so the walk always ends
// there.  Every wait is bounded; on expiry *gave_up is set.
template <int W = kLookbackWindow>
__device__ __forceinline__ uint32_t onesweep_lookback(const unsigned long long *__restrict__ status, uint32_t tile,
                                                      uint32_t first_tile, unsigned d, uint32_t tag_agg,
                                                      bool *gave_up, uint32_t limit = kSpinLimit) {
  uint32_t excl = 0;
  const int64_t floor_t = int64_t(first_tile);
  int64_t t = int64_t(tile) - 1;
  const unsigned long long kDone = (unsigned long long)(tag_agg + 1u) << 32;
  while (t >= floor_t) {
    unsigned long long w[W];
#pragma unroll
    for (int j = 0; j < W; ++j)
      w[j] = (t - j >= floor_t) ? ld_relaxed_u64(status + size_t(t - j) * kRadix + d) : kDone;
    bool done = false;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      if (done) break;
      unsigned long long x = w[j];
      uint32_t spins = 0;
      while (uint32_t(x >> 32) < tag_agg) {
        if (++spins > limit) {
          *gave_up = true;
          return excl;
        }
        __nanosleep(spins < 32 ? 16 : 128);
        x = ld_relaxed_u64(status + size_t(t - j) * kRadix + d);
      }
      excl += uint32_t(x);
      done = uint32_t(x >> 32) != tag_agg;
    }
    if (done) break;
    t -= W;
  }
  return excl;
}

// Shared-memory footprint of one onesweep block: per-warp digit counters
// (later the tile-local start of each warp's run of each digit), then the
// tile's keys and values staged in digit order.
// Counter width in bytes: a tile holds at most 65536 keys, so 16-bit counters
// suffice (and leave room for a fourth block per SM).
constexpr int kCounterBytes = 2;
template <int CB> struct counter_type;
template <> struct counter_type<2> { typedef uint16_t type; };
template <> struct counter_type<4> { typedef uint32_t type; };

template <class U, int VB, int IPT_ = items_per_thread<U>::value, int CB = kCounterBytes>
struct OnesweepSmem {
  typedef typename value_type_of<VB>::type VT;
  typedef typename counter_type<CB>::type CT;
  static constexpr int IPT = IPT_;
  static constexpr int TILE = kSortThreads * IPT;
  static constexpr size_t kCounters = size_t(kSortWarps) * kRadix * CB;
  static constexpr size_t kKeys = kCounters;
  static constexpr size_t kVals = kKeys + ((size_t(TILE) * sizeof(U) + 15) & ~size_t(15));
  static constexpr size_t kBytes = kVals + (VB ? size_t(TILE) * sizeof(VT) : 0);
};

// How a warp finds, for each item, the lanes holding the same digit:
// kRankMatch issues one match instruction per item just before using it;
// kRankMatchAhead issues the matches of all items first so their latencies
// overlap; kRankBallot builds the mask from one ballot per digit bit.
enum RankMethod : int { kRankMatch = 0, kRankMatchAhead = 1, kRankBallot = 2 };
// The match instruction waits on a long-latency unit and each item's counter
// update depends on the previous one, so warps stall on it; the ballots are
// plain ALU work.  One pass over 2^28 uint32 pairs on GB300 (16 keys per
// thread): kRankMatch 2.10 ms, kRankMatchAhead 2.23 ms, kRankBallot 1.40 ms.
// With 24 keys per thread, computing the ballots of 4 or 8 items ahead of
// their counter updates gave the same time (1.233-1.235 ms against 1.236),
// and counter updates by shared-memory atomics from each digit's lowest lane
// were slower (1.27 ms): the ballots are limited by issue throughput, not by
// the counter chain.
constexpr int kRankDefault = kRankBallot;

// How values reach their digit-order slots in shared memory: kValsRegs loads
// them into registers before the look-back and stores them after it;
// kValsAsync copies each value from global memory straight to its slot with
// cp.async (4-, 8- and 16-byte values), holding no registers across the walk.
// One pass over 2^28 uint32 pairs on GB300 at 3 blocks per SM: registers
// 1.262 ms, asynchronous 1.299 ms; at 4 blocks per SM (which the register
// variant cannot reach without spilling its 24 values) asynchronous 1.236 ms.
enum ValueStaging : int { kValsRegs = 0, kValsAsync = 1 };
constexpr int kValsDefault = kValsAsync;

// Lanes of this warp whose digit equals d (d < kRadix for valid lanes;
// `valid_mask` holds the valid lanes).
template <int RANK>
__device__ __forceinline__ unsigned digit_peers(uint32_t d, unsigned valid_mask) {
  if (RANK == kRankBallot) {
    unsigned peers = valid_mask;
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b) {
      const bool bit = (d >> b) & 1u;
      const unsigned v = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? v : ~v;
    }
    return peers;
  } else {
    return __match_any_sync(0xffffffffu, d);
  }
}

// Digit of a key at `shift`; PLAIN keys (unsigned, ascending) skip the
// transform.
template <class U, bool PLAIN>
__device__ __forceinline__ uint32_t key_digit(U x, const KeyXform<U> &xf, int shift) {
  const U k = PLAIN ? x : apply_xform<U>(x, xf);
  return uint32_t(k >> shift) & (kRadix - 1);
}

// One onesweep tile (FULL: count == TILE, no bounds checks).
//
// Order of work: load the keys warp-striped (item i of lane l is element
// warp_first + 32 i + l, so (i, l) order is input order), rank every key
// within its warp against per-warp digit counters (stable: a key's rank
// counts the equal digits before it in input order), publish the tile's digit
// counts, stage keys in shared memory in digit order while the values are
// copied to their digit-order slots, and only then look back over
// predecessor tiles: by then the predecessors, which started earlier, have
// mostly published their inclusive prefixes, so the walk is short.  The whole
// tile is then written out in digit order, each digit's run to consecutive
// addresses.
template <class U, int VB, bool PLAIN, bool FULL, int IPT_, int RANK, int LBW, int PF = 0, int CB = kCounterBytes,
          int VS = kValsDefault>
__device__ __forceinline__ void onesweep_tile_impl(const U *__restrict__ src_k, U *__restrict__ dst_k,
                                                   const typename value_type_of<VB>::type *__restrict__ src_v,
                                                   typename value_type_of<VB>::type *__restrict__ dst_v,
                                                   uint32_t base, uint32_t count, uint32_t tile,
                                                   uint32_t first_tile, const uint32_t *__restrict__ digit_start,
                                                   uint32_t dst_limit, int pass, int shift, const KeyXform<U> &xf,
                                                   unsigned long long *__restrict__ status, uint32_t *err) {
  typedef OnesweepSmem<U, VB, IPT_, CB> L;
  typedef typename L::VT VT;
  typedef typename L::CT CT;
  constexpr int IPT = L::IPT;
  static_assert(kSortThreads == kRadix, "one thread per digit");
  static_assert(L::TILE <= 65536, "16-bit tile positions");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT *wcnt = reinterpret_cast<CT *>(smem_raw);               // [kSortWarps][kRadix]
  U *s_keys = reinterpret_cast<U *>(smem_raw + L::kKeys);    // digit order
  VT *s_vals = reinterpret_cast<VT *>(smem_raw + L::kVals);  // digit order
  __shared__ uint32_t s_gofs[kRadix];  // output index of a digit's run minus its tile-local start
  __shared__ uint32_t s_warp_sum[kSortWarps];

  const unsigned tid = threadIdx.x, lane = lane_id(), warp = tid / kWarp;
  if (PF > 0 && tid == 0) {
    // Ask L2 for the tile PF tickets ahead (processed about one resident wave
    // later), keys and values, clipped to this sort's elements.
    const uint64_t fb = uint64_t(base) + uint64_t(PF) * L::TILE;
    if (fb < dst_limit) {
      const uint32_t m = uint32_t((uint64_t(dst_limit) - fb) < uint64_t(L::TILE) ? (uint64_t(dst_limit) - fb)
                                                                              : uint64_t(L::TILE));
      const uint32_t kb = uint32_t(m * sizeof(U)) & ~15u;
      const char *kp = reinterpret_cast<const char *>(src_k + fb);
      if ((reinterpret_cast<uintptr_t>(kp) & 15u) == 0 && kb) bulk_prefetch_l2(kp, kb);
      if (VB) {
        const uint32_t vbytes = uint32_t(m * sizeof(VT)) & ~15u;
        const char *vp = reinterpret_cast<const char *>(src_v + fb);
        if ((reinterpret_cast<uintptr_t>(vp) & 15u) == 0 && vbytes) bulk_prefetch_l2(vp, vbytes);
      }
    }
  }
  const uint32_t dstart = digit_start[tid];
  CT *my_cnt = wcnt + warp * kRadix;
#pragma unroll
  for (int j = 0; j < kRadix * CB / 4 / kWarp; ++j) reinterpret_cast<uint32_t *>(my_cnt)[j * kWarp + lane] = 0;
  const uint32_t warp_first = warp * (kWarp * IPT);
  const U *wk = src_k + base + warp_first + lane;
  U key[IPT];
#pragma unroll
  for (int i = 0; i < IPT; ++i)
    if (FULL || warp_first + i * kWarp + lane < count) key[i] = wk[i * kWarp];
  __syncwarp();

  // Rank within the warp: 16-bit field i of pos[] (two per register) is the
  // rank of item i among the equal digits of this warp, later its position in
  // the tile.
  uint32_t pos[(IPT + 1) / 2];
  const unsigned lt = lanemask_lt();
  unsigned ahead[RANK == kRankMatchAhead ? IPT : 1];
  if (RANK == kRankMatchAhead) {
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const bool valid = FULL || warp_first + i * kWarp + lane < count;
      ahead[i] = __match_any_sync(0xffffffffu, valid ? key_digit<U, PLAIN>(key[i], xf, shift) : uint32_t(kRadix));
    }
  }
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const bool valid = FULL || warp_first + i * kWarp + lane < count;
    const uint32_t d = valid ? key_digit<U, PLAIN>(key[i], xf, shift) : uint32_t(kRadix);
    unsigned peers;
    if (RANK == kRankMatchAhead) {
      peers = ahead[i];
    } else {
      const unsigned vmask = FULL ? 0xffffffffu : __ballot_sync(0xffffffffu, valid);
      peers = digit_peers<RANK>(d, vmask);
    }
    const uint32_t below = __popc(peers & lt);
    uint32_t prior = 0;
    if (valid) prior = my_cnt[d];
    __syncwarp();
    if (valid && below == 0) my_cnt[d] = CT(prior + __popc(peers));
    __syncwarp();
    if (i & 1) pos[i / 2] |= (prior + below) << 16;
    else pos[i / 2] = prior + below;
  }
  __syncthreads();

  // Thread `tid` owns digit `tid`: the tile total (published for the
  // successors), the tile-local start of the digit, and the start of each
  // warp's run of it.
  uint32_t tile_cnt = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) tile_cnt += wcnt[w * kRadix + tid];
  const uint32_t tag = tag_aggregate(pass);
  unsigned long long *my_status = status + size_t(tile) * kRadix + tid;
  st_relaxed_u64(my_status, ((unsigned long long)(tile == first_tile ? tag + 1u : tag) << 32) | tile_cnt);
  uint32_t incl = tile_cnt;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (int(lane) >= o) incl += t;
  }
  if (lane == kWarp - 1) s_warp_sum[warp] = incl;
  __syncthreads();
  uint32_t local_start = incl - tile_cnt;
  for (unsigned j = 0; j < warp; ++j) local_start += s_warp_sum[j];
  {
    uint32_t run = local_start;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = wcnt[w * kRadix + tid];
      wcnt[w * kRadix + tid] = CT(run);
      run += c;
    }
  }
  __syncthreads();

  // Stage keys in digit order.  Values are copied asynchronously to their
  // slots as each position is known (their latency overlaps the walk, and
  // they hold no registers); or, for 1- and 2-byte values and the register
  // variant, values of up to 4 bytes are loaded before the look-back and
  // staged after it, and wider ones are staged first, in groups, to bound the
  // registers they hold.
  const VT *wv = src_v + base + warp_first + lane;
  constexpr bool kAsync = VB && VS == kValsAsync && sizeof(VT) >= 4;
  constexpr bool kEarly = !kAsync && sizeof(VT) <= 4;
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    if (FULL || warp_first + i * kWarp + lane < count) {
      const uint32_t d = key_digit<U, PLAIN>(key[i], xf, shift);
      const uint32_t half = (i & 1) ? 16 : 0;
      const uint32_t p = my_cnt[d] + ((pos[i / 2] >> half) & 0xffffu);
      s_keys[p] = key[i];
      if constexpr (kAsync)
        cp_async_smem<sizeof(VT)>(s_vals + p, wv + i * kWarp);
      else
        pos[i / 2] = (pos[i / 2] & (0xffff0000u >> half)) | (p << half);
    }
  }
  VT val[(VB && kEarly) ? IPT : 1];
  if (VB && kEarly) {
#pragma unroll
    for (int i = 0; i < IPT; ++i)
      if (FULL || warp_first + i * kWarp + lane < count) val[i] = wv[i * kWarp];
  }
  if (VB && !kEarly && !kAsync) {
    constexpr int G = 4;
#pragma unroll
    for (int g = 0; g < IPT; g += G) {
      VT v[G];
#pragma unroll
      for (int j = 0; j < G; ++j)
        if (g + j < IPT && (FULL || warp_first + (g + j) * kWarp + lane < count)) v[j] = wv[(g + j) * kWarp];
#pragma unroll
      for (int j = 0; j < G; ++j) {
        const int i = g + j;
        if (i < IPT && (FULL || warp_first + i * kWarp + lane < count))
          s_vals[(pos[i / 2] >> ((i & 1) ? 16 : 0)) & 0xffffu] = v[j];
      }
    }
  }

  // Look back for the digit's count in the predecessor tiles.
  uint32_t excl = 0;
  if (tile > first_tile) {
    bool gave_up = false;
    excl = onesweep_lookback<LBW>(status, tile, first_tile, tid, tag, &gave_up);
    if (gave_up) report_error(err, kErrLookbackTimeout);
    st_relaxed_u64(my_status, ((unsigned long long)(tag + 1u) << 32) | (excl + tile_cnt));
  }
  s_gofs[tid] = dstart + excl - local_start;
  if (VB && kEarly) {
#pragma unroll
    for (int i = 0; i < IPT; ++i)
      if (FULL || warp_first + i * kWarp + lane < count)
        s_vals[(pos[i / 2] >> ((i & 1) ? 16 : 0)) & 0xffffu] = val[i];
  }
  if (kAsync) cp_async_wait_all();
  __syncthreads();

  // Write out: consecutive threads take consecutive digit-order positions.
  // Every index is in range unless a look-back wait gave up (then the error
  // word is set and the output is garbage, but no write leaves the buffer).
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const uint32_t p = k * kSortThreads + tid;
    if (FULL || p < count) {
      const U x = s_keys[p];
      const uint32_t g = s_gofs[key_digit<U, PLAIN>(x, xf, shift)] + p;
      if (g < dst_limit) {
        dst_k[g] = x;
        if (VB) dst_v[g] = s_vals[p];
      }
    }
  }
}

// Sorts one tile of `count` elements starting at `base` by the digit at
// `shift` into dst: element of digit d goes to digit_start[d] + (elements of
// digit d in tiles first_tile .. tile-1) + (its stable rank in this tile).
// Row `tile` of `status` holds this tile's look-back word per digit.
// Called by every thread of a kSortThreads block; the dynamic shared memory is
// OnesweepSmem<U, VB>::kBytes.
// The partial last tile takes a separate, out-of-line copy of the routine so
// that its bounds checks do not raise the register pressure of the full-tile
// path.
template <class U, int VB, bool PLAIN, int IPT, int RANK, int LBW, int CB, int VS>
__device__ __noinline__ void onesweep_partial_tile(const U *__restrict__ src_k, U *__restrict__ dst_k,
                                                   const typename value_type_of<VB>::type *__restrict__ src_v,
                                                   typename value_type_of<VB>::type *__restrict__ dst_v,
                                                   uint32_t base, uint32_t count, uint32_t tile,
                                                   uint32_t first_tile, const uint32_t *__restrict__ digit_start,
                                                   uint32_t dst_limit, int pass, int shift, const KeyXform<U> xf,
                                                   unsigned long long *__restrict__ status, uint32_t *err) {
  onesweep_tile_impl<U, VB, PLAIN, false, IPT, RANK, LBW, 0, CB, VS>(src_k, dst_k, src_v, dst_v, base, count, tile,
                                                                     first_tile, digit_start, dst_limit, pass, shift,
                                                                     xf, status, err);
}

template <class U, int VB, bool PLAIN, int IPT = items_per_thread<U>::value, int RANK = kRankDefault,
          int LBW = kLookbackWindow, int PF = kOnesweepPrefetchTiles, int CB = kCounterBytes, int VS = kValsDefault>
__device__ __forceinline__ void onesweep_tile(const U *__restrict__ src_k, U *__restrict__ dst_k,
                                              const typename value_type_of<VB>::type *__restrict__ src_v,
                                              typename value_type_of<VB>::type *__restrict__ dst_v,
                                              uint32_t base, uint32_t count, uint32_t tile, uint32_t first_tile,
                                              const uint32_t *__restrict__ digit_start, uint32_t dst_limit,
                                              int pass, int shift, const KeyXform<U> &xf,
                                              unsigned long long *__restrict__ status, uint32_t *err) {
  if (count == uint32_t(OnesweepSmem<U, VB, IPT, CB>::TILE))
    onesweep_tile_impl<U, VB, PLAIN, true, IPT, RANK, LBW, PF, CB, VS>(src_k, dst_k, src_v, dst_v, base, count, tile,
                                                                       first_tile, digit_start, dst_limit, pass,
                                                                       shift, xf, status, err);
  else
    onesweep_partial_tile<U, VB, PLAIN, IPT, RANK, LBW, CB, VS>(src_k, dst_k, src_v, dst_v, base, count, tile,
                                                                first_tile, digit_start, dst_limit, pass, shift, xf,
                                                                status, err);
}


}  // namespace radix
}  // namespace bcx
