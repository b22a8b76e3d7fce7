// bcx_segmented_sort.cu -- segmented sort / sort_by_key as one stream of
// kernels (graph-capturable: nothing is read back to the host).
//
// The reference has no segmented sort: a caller sorts each segment with its
// own sort_by_key call (sort_by_key.hpp:33-163 -> radix_sort.hpp:253-426,
// ~6 launches per 4-bit pass).  Here segments are CSR offsets (device
// memory, nseg + 1 uint64, offsets[0] == 0, offsets[nseg] == n) and every
// segment is sorted stably and independently, in the reference's radix order
// (the same key transform as the plain sort).
//
// Small segments (up to a few thousand pairs) are sorted by one block each,
// entirely in shared memory: load once, one stable 8-bit LSD pass per digit
// between two shared-memory buffers (passes whose digit is the same for the
// whole segment are skipped), store once.
//
// Large segments are cut into tiles that never cross a segment boundary and
// sorted with the onesweep tile routine of the plain sort: a device-side plan
// numbers the tiles, one kernel builds every large segment's digit
// histograms, one turns them into per-segment digit start offsets, and one
// kernel per digit pass moves the tiles, each tile looking back only over the
// tiles of its own segment.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"
#include "bcx_radix.cuh"

namespace bcx {
namespace {

using namespace radix;

constexpr int kPlanThreads = 1024;

// Largest segment the shared-memory path sorts: about 96 KB of double
// buffered keys and values, at most 4096 pairs.  The path is compiled for
// tiles of 1024, 2048 and 4096 pairs up to that limit; the tile in use (and
// with it the size below which a segment is sorted in shared memory) is the
// tunable "small_tile", the grid the tunable "small_blocks_per_sm".
template <class U, int VB>
struct SmallCap {
  typedef typename value_type_of<VB>::type VT;
  static constexpr size_t kPair = sizeof(U) + (VB ? sizeof(VT) : 0);
  static constexpr int raw = int((96 * 1024) / (2 * kPair));
  static constexpr int value = raw >= 4096 ? 4096 : (raw >= 2048 ? 2048 : 1024);
};
constexpr uint32_t kMinSmallTile = 1024;

template <class U, int VB, int CAP>
struct SmallTile {
  static constexpr int IPT = CAP / kSortThreads;
  static constexpr size_t kBytes = size_t(kSortWarps) * kRadix * 4 + 2 * size_t(CAP) * SmallCap<U, VB>::kPair;
};

// ---- plan ------------------------------------------------------------------
// tile_first[s]: first large tile of segment s (exclusive scan of tile counts,
// tile_first[nseg] = total tiles); large_ord[s]: ordinal of s among the large
// segments; seg_of_large[k]: segment of the k-th large segment;
// totals[0] = large tiles, totals[1] = large segments.
__global__ void __launch_bounds__(kPlanThreads)
segsort_plan_kernel(const unsigned long long *__restrict__ offsets, uint32_t nseg, uint32_t small_cap,
                    uint32_t tile, uint32_t *__restrict__ tile_first, uint32_t *__restrict__ large_ord,
                    uint32_t *__restrict__ seg_of_large, uint32_t *__restrict__ totals) {
  __shared__ uint32_t warp_t[kPlanThreads / kWarp], warp_l[kPlanThreads / kWarp];
  __shared__ uint32_t carry_t, carry_l;
  const unsigned lane = lane_id(), warp = threadIdx.x / kWarp;
  if (threadIdx.x == 0) carry_t = carry_l = 0;
  __syncthreads();
  for (uint32_t b = 0; b < nseg; b += kPlanThreads) {
    const uint32_t s = b + threadIdx.x;
    uint32_t t = 0, l = 0;
    if (s < nseg) {
      const unsigned long long len = offsets[s + 1] - offsets[s];
      if (len > small_cap) {
        l = 1;
        t = uint32_t((len + tile - 1) / tile);
      }
    }
    uint32_t it = t, il = l;
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
      const uint32_t ot = __shfl_up_sync(0xffffffffu, it, d), ol = __shfl_up_sync(0xffffffffu, il, d);
      if (int(lane) >= d) {
        it += ot;
        il += ol;
      }
    }
    if (lane == kWarp - 1) {
      warp_t[warp] = it;
      warp_l[warp] = il;
    }
    __syncthreads();
    uint32_t bt = carry_t, bl = carry_l;
    for (unsigned w = 0; w < warp; ++w) {
      bt += warp_t[w];
      bl += warp_l[w];
    }
    if (s < nseg) {
      tile_first[s] = bt + it - t;
      large_ord[s] = bl + il - l;
      if (l) seg_of_large[bl + il - l] = s;
    }
    __syncthreads();
    if (threadIdx.x == kPlanThreads - 1) {
      carry_t = bt + it;
      carry_l = bl + il;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tile_first[nseg] = carry_t;
    totals[0] = carry_t;
    totals[1] = carry_l;
  }
}

// Segment holding large tile t: the last s with tile_first[s] <= t among the
// segments that own tiles.
__device__ __forceinline__ uint32_t segment_of_tile(const uint32_t *__restrict__ tile_first, uint32_t nseg,
                                                    uint32_t t) {
  uint32_t lo = 0, hi = nseg;  // find last s with tile_first[s] <= t and tile_first[s+1] > t
  while (lo + 1 < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (tile_first[mid] <= t) lo = mid;
    else hi = mid;
  }
  // skip segments without tiles that share the same tile_first
  while (lo + 1 < nseg && tile_first[lo + 1] <= t) ++lo;
  return lo;
}

struct LargeTile {
  uint32_t seg, ord, base, count, first_tile;
};

// Large tile t of segment seg: its elements and look-back floor.
__device__ __forceinline__ LargeTile tile_of_segment(const unsigned long long *__restrict__ offsets,
                                                     const uint32_t *__restrict__ tile_first,
                                                     const uint32_t *__restrict__ large_ord, uint32_t seg,
                                                     uint32_t t, uint32_t tile) {
  LargeTile r;
  r.seg = seg;
  r.ord = large_ord[r.seg];
  r.first_tile = tile_first[r.seg];
  const unsigned long long b = offsets[r.seg], e = offsets[r.seg + 1];
  r.base = uint32_t(b + (unsigned long long)(t - r.first_tile) * tile);
  const unsigned long long left = e - r.base;
  r.count = uint32_t(left < tile ? left : tile);
  return r;
}

// ---- large segments: histograms and digit starts --------------------------
template <class U, int PASSES>
__global__ void __launch_bounds__(kHistThreads)
segsort_hist_kernel(const U *__restrict__ keys, const unsigned long long *__restrict__ offsets, uint32_t nseg,
                    const uint32_t *__restrict__ tile_first, const uint32_t *__restrict__ large_ord,
                    const uint32_t *__restrict__ totals, uint32_t tile, const KeyXform<U> xf,
                    uint32_t *__restrict__ seg_hist, uint32_t *__restrict__ tile_seg) {
  __shared__ uint32_t sh[PASSES][kRadix];
  __shared__ uint32_t s_seg;
  const uint32_t t = blockIdx.x;
  if (t >= totals[0]) return;
  for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistThreads) (&sh[0][0])[i] = 0;
  // The segment of this tile is searched once here and recorded for the
  // digit passes.
  if (threadIdx.x == 0) {
    s_seg = segment_of_tile(tile_first, nseg, t);
    tile_seg[t] = s_seg;
  }
  __syncthreads();
  const LargeTile lt = tile_of_segment(offsets, tile_first, large_ord, s_seg, t, tile);
  for (uint32_t i = threadIdx.x; i < lt.count; i += kHistThreads) {
    const U k = apply_xform<U>(keys[lt.base + i], xf);
#pragma unroll
    for (int p = 0; p < PASSES; ++p) atomicAdd(&sh[p][uint32_t(k >> (p * kRadixBits)) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  uint32_t *dst = seg_hist + size_t(lt.ord) * PASSES * kRadix;
  for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistThreads) {
    const uint32_t c = (&sh[0][0])[i];
    if (c) atomicAdd(&dst[i], c);
  }
}

// Per large segment and pass: exclusive scan of the 256 digit counts, plus the
// segment's first element, in place.
template <int PASSES>
__global__ void __launch_bounds__(kRadix)
segsort_starts_kernel(const unsigned long long *__restrict__ offsets, const uint32_t *__restrict__ seg_of_large,
                      const uint32_t *__restrict__ totals, uint32_t *__restrict__ seg_hist) {
  __shared__ uint32_t warp_sum[kRadix / kWarp];
  const uint32_t k = blockIdx.x;
  if (k >= totals[1]) return;
  const uint32_t seg_begin = uint32_t(offsets[seg_of_large[k]]);
  const unsigned d = threadIdx.x, lane = lane_id(), w = d / kWarp;
  for (int p = 0; p < PASSES; ++p) {
    uint32_t *h = seg_hist + (size_t(k) * PASSES + p) * kRadix;
    const uint32_t c = h[d];
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (int(lane) >= o) incl += t;
    }
    if (lane == kWarp - 1) warp_sum[w] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (unsigned j = 0; j < w; ++j) before += warp_sum[j];
    h[d] = seg_begin + before + incl - c;
    __syncthreads();
  }
}

template <class U, int VB, bool PLAIN>
__global__ void __launch_bounds__(kSortThreads, kSortBlocksPerSm)
segsort_onesweep_kernel(U *__restrict__ keys_main, U *__restrict__ keys_alt,
                        typename value_type_of<VB>::type *__restrict__ vals_main,
                        typename value_type_of<VB>::type *__restrict__ vals_alt, uint32_t n,
                        const unsigned long long *__restrict__ offsets, uint32_t nseg,
                        const uint32_t *__restrict__ tile_first, const uint32_t *__restrict__ large_ord,
                        const uint32_t *__restrict__ totals, int pass, int passes, const KeyXform<U> xf,
                        const uint32_t *__restrict__ digit_start, unsigned long long *__restrict__ status,
                        uint32_t *__restrict__ tile_counter, const uint32_t *__restrict__ tile_seg, uint32_t *err) {
  constexpr uint32_t TILE = OnesweepSmem<U, VB>::TILE;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const uint32_t t = s_tile;
  if (t >= totals[0]) return;
  const LargeTile lt = tile_of_segment(offsets, tile_first, large_ord, tile_seg[t], t, TILE);
  const bool from_alt = (pass & 1) != 0;
  onesweep_tile<U, VB, PLAIN>(from_alt ? keys_alt : keys_main, from_alt ? keys_main : keys_alt,
                              from_alt ? vals_alt : vals_main, from_alt ? vals_main : vals_alt, lt.base, lt.count, t,
                              lt.first_tile, digit_start + (size_t(lt.ord) * passes + pass) * kRadix, n, pass,
                              pass * kRadixBits, xf, status, err);
}

// Odd pass counts leave large segments in the temporary buffers.
template <class U, int VB>
__global__ void segsort_copyback_kernel(U *__restrict__ keys_main, const U *__restrict__ keys_alt,
                                        typename value_type_of<VB>::type *__restrict__ vals_main,
                                        const typename value_type_of<VB>::type *__restrict__ vals_alt,
                                        const unsigned long long *__restrict__ offsets, uint32_t nseg,
                                        const uint32_t *__restrict__ tile_first,
                                        const uint32_t *__restrict__ large_ord,
                                        const uint32_t *__restrict__ totals, const uint32_t *__restrict__ tile_seg) {
  constexpr uint32_t TILE = OnesweepSmem<U, VB>::TILE;
  const uint32_t t = blockIdx.x;
  if (t >= totals[0]) return;
  const LargeTile lt = tile_of_segment(offsets, tile_first, large_ord, tile_seg[t], t, TILE);
  for (uint32_t i = threadIdx.x; i < lt.count; i += blockDim.x) {
    keys_main[lt.base + i] = keys_alt[lt.base + i];
    if (VB) vals_main[lt.base + i] = vals_alt[lt.base + i];
  }
}

// ---- small segments: whole-segment sort in shared memory -------------------
template <class U, int VB, int CAP>
__global__ void __launch_bounds__(kSortThreads)
segsort_small_kernel(U *__restrict__ keys, typename value_type_of<VB>::type *__restrict__ vals,
                     const unsigned long long *__restrict__ offsets, uint32_t nseg, int passes,
                     const KeyXform<U> xf, uint32_t *__restrict__ seg_counter) {
  typedef typename value_type_of<VB>::type VT;
  constexpr int IPT = SmallTile<U, VB, CAP>::IPT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t *wcnt = reinterpret_cast<uint32_t *>(smem_raw);
  U *kbuf = reinterpret_cast<U *>(smem_raw + size_t(kSortWarps) * kRadix * 4);  // [2][CAP]
  VT *vbuf = reinterpret_cast<VT *>(smem_raw + size_t(kSortWarps) * kRadix * 4 + 2 * size_t(CAP) * sizeof(U));
  __shared__ uint32_t s_start[kRadix];
  __shared__ uint32_t s_warp_sum[kSortWarps];
  __shared__ uint32_t s_seg;
  __shared__ int s_skip;
  const unsigned tid = threadIdx.x, lane = lane_id(), warp = tid / kWarp;
  const unsigned lt_mask = lanemask_lt();
  while (true) {
    if (tid == 0) s_seg = atomicAdd(seg_counter, 1u);
    __syncthreads();
    const uint32_t seg = s_seg;
    if (seg >= nseg) break;
    const unsigned long long b = offsets[seg];
    const uint32_t m = uint32_t(offsets[seg + 1] - b);
    if (m < 2 || m > uint32_t(CAP)) {
      __syncthreads();
      continue;
    }
    int cur = 0;
    for (uint32_t i = tid; i < m; i += kSortThreads) {
      kbuf[i] = keys[b + i];
      if (VB) vbuf[i] = vals[b + i];
    }
    for (int p = 0; p < passes; ++p) {
      U *ka = kbuf + size_t(cur) * CAP;
      U *kb = kbuf + size_t(cur ^ 1) * CAP;
      VT *va = vbuf + size_t(cur) * CAP;
      VT *vb = vbuf + size_t(cur ^ 1) * CAP;
      for (int i = lane; i < kRadix; i += kWarp) wcnt[warp * kRadix + i] = 0;
      __syncthreads();
      uint32_t dr[IPT];
      const uint32_t warp_first = warp * (kWarp * IPT);
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const uint32_t e = warp_first + i * kWarp + lane;
        const bool valid = e < m;
        const uint32_t d = valid ? (uint32_t(apply_xform<U>(ka[e], xf) >> (p * kRadixBits)) & (kRadix - 1)) : 0u;
        unsigned grp = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int bit = 0; bit < kRadixBits; ++bit) {
          const bool on = (d >> bit) & 1u;
          const unsigned v = __ballot_sync(0xffffffffu, on);
          grp &= on ? v : ~v;
        }
        const int leader = __ffs(grp) - 1;
        uint32_t old = 0;
        if (valid && int(lane) == leader) {
          old = wcnt[warp * kRadix + d];
          wcnt[warp * kRadix + d] = old + __popc(grp);
        }
        old = __shfl_sync(0xffffffffu, old, valid ? leader : int(lane));
        dr[i] = valid ? (d | ((old + __popc(grp & lt_mask)) << 8)) : 0x80000000u;
        __syncwarp();
      }
      __syncthreads();
      // thread tid owns digit tid: prefix over warps, then over digits
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = wcnt[w * kRadix + tid];
        wcnt[w * kRadix + tid] = run;
        run += c;
      }
      uint32_t incl = run;
#pragma unroll
      for (int o = 1; o < kWarp; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (int(lane) >= o) incl += t;
      }
      if (lane == kWarp - 1) s_warp_sum[warp] = incl;
      if (tid == 0) s_skip = 0;
      __syncthreads();
      uint32_t before = 0;
      for (unsigned j = 0; j < warp; ++j) before += s_warp_sum[j];
      s_start[tid] = before + incl - run;
      if (run == m) s_skip = 1;  // one digit holds the whole segment: identity pass
      __syncthreads();
      if (!s_skip) {
#pragma unroll
        for (int i = 0; i < IPT; ++i) {
          if (!(dr[i] & 0x80000000u)) {
            const uint32_t d = dr[i] & 0xffu;
            const uint32_t pos = s_start[d] + wcnt[warp * kRadix + d] + (dr[i] >> 8);
            const uint32_t e = warp_first + i * kWarp + lane;
            kb[pos] = ka[e];
            if (VB) vb[pos] = va[e];
          }
        }
        cur ^= 1;
      }
      __syncthreads();
    }
    const U *kf = kbuf + size_t(cur) * CAP;
    const VT *vf = vbuf + size_t(cur) * CAP;
    for (uint32_t i = tid; i < m; i += kSortThreads) {
      keys[b + i] = kf[i];
      if (VB) vals[b + i] = vf[i];
    }
    __syncthreads();
  }
}

// ---- host ------------------------------------------------------------------
struct SegLayout {
  size_t alt_keys, alt_vals, tile_first, large_ord, seg_of_large, tile_seg, totals, counters, seg_hist, status, total;
  size_t zero_begin, zero_bytes;
  uint32_t max_tiles, max_large;
};

template <class U, int VB>
SegLayout seg_layout(size_t n, size_t nseg) {
  typedef typename value_type_of<VB>::type VT;
  constexpr int PASSES = int(sizeof(U));
  constexpr uint32_t TILE = OnesweepSmem<U, VB>::TILE;
  SegLayout L;
  // sized for the smallest small tile (the most large segments), so the
  // size does not depend on the tuned tile
  L.max_large = uint32_t(std::min<size_t>(nseg, n / (kMinSmallTile + 1) + 1));
  L.max_tiles = uint32_t(n / TILE + L.max_large + 1);
  size_t off = 0;
  L.alt_keys = off;
  off += align256(n * sizeof(U));
  L.alt_vals = off;
  off += VB ? align256(n * sizeof(VT)) : 0;
  L.tile_first = off;
  off += align256((nseg + 1) * 4);
  L.large_ord = off;
  off += align256(nseg * 4);
  L.seg_of_large = off;
  off += align256(nseg * 4);
  L.tile_seg = off;
  off += align256(size_t(L.max_tiles) * 4);
  L.totals = off;
  off += 256;
  L.counters = off;  // small-segment ticket + one ticket per pass
  off += 256;
  L.seg_hist = off;
  off += align256(size_t(L.max_large) * PASSES * kRadix * 4);
  L.status = off;  // one array for every pass (status words carry the pass)
  off += align256(size_t(L.max_tiles) * kRadix * 8);
  L.total = off;
  L.zero_begin = L.counters;
  L.zero_bytes = off - L.counters;
  return L;
}

template <class U, int VB, int CAP>
bcx_status launch_small(cudaStream_t s, U *k_main, typename value_type_of<VB>::type *v_main,
                        const unsigned long long *offsets, size_t nseg, const KeyXform<U> &xf, uint32_t *counter,
                        uint32_t per_sm, const DeviceState *ds) {
  if constexpr (CAP > SmallCap<U, VB>::value) {
    return BCX_UNSUPPORTED;
  } else {
    constexpr size_t smem = SmallTile<U, VB, CAP>::kBytes;
    static std::atomic<uint64_t> optin{0};
    BCX_CUDA(smem_optin(reinterpret_cast<const void *>(segsort_small_kernel<U, VB, CAP>), int(smem), &optin));
    static int resident = 0;  // blocks per SM at this shared-memory size (same GPU model on every device)
    if (!resident) {
      int r = 0;
      BCX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, segsort_small_kernel<U, VB, CAP>, kSortThreads,
                                                             smem));
      resident = r > 0 ? r : 1;
    }
    size_t blocks = size_t(ds->sm_count) * (per_sm ? per_sm : uint32_t(resident));
    if (blocks > nseg) blocks = nseg;
    KernelScope ks("segsort_small", s);
    segsort_small_kernel<U, VB, CAP><<<unsigned(blocks), kSortThreads, smem, s>>>(
        k_main, v_main, offsets, uint32_t(nseg), int(sizeof(U)), xf, counter);
    return launch_status("segsort_small");
  }
}

template <class U, int VB, bool PLAIN>
bcx_status seg_onesweep_passes(cudaStream_t s, const SegLayout &L, U *k_main, U *k_alt,
                               typename value_type_of<VB>::type *v_main, typename value_type_of<VB>::type *v_alt,
                               size_t n, const unsigned long long *offsets, size_t nseg, const uint32_t *tile_first,
                               const uint32_t *large_ord, const uint32_t *totals, const KeyXform<U> &xf,
                               const uint32_t *seg_hist, unsigned long long *status, uint32_t *counters,
                               const uint32_t *tile_seg, uint32_t *err) {
  constexpr int PASSES = int(sizeof(U));
  constexpr size_t smem = OnesweepSmem<U, VB>::kBytes;
  static std::atomic<uint64_t> optin{0};
  BCX_CUDA(smem_optin(reinterpret_cast<const void *>(segsort_onesweep_kernel<U, VB, PLAIN>), int(smem), &optin));
  for (int p = 0; p < PASSES; ++p) {
    KernelScope ks("segsort_onesweep", s);
    segsort_onesweep_kernel<U, VB, PLAIN><<<L.max_tiles, kSortThreads, smem, s>>>(
        k_main, k_alt, v_main, v_alt, uint32_t(n), offsets, uint32_t(nseg), tile_first, large_ord, totals, p, PASSES,
        xf, seg_hist, status, counters + 1 + p, tile_seg, err);
    bcx_status rc = launch_status("segsort_onesweep");
    if (rc) return rc;
  }
  return BCX_SUCCESS;
}

template <class U, int VB>
bcx_status segsort_t(cudaStream_t s, void *keys, void *values, size_t n, const unsigned long long *offsets,
                     size_t nseg, int kind, int desc, void *temp, size_t *temp_bytes) {
  typedef typename value_type_of<VB>::type VT;
  constexpr int PASSES = int(sizeof(U));
  constexpr uint32_t TILE = OnesweepSmem<U, VB>::TILE;
  BCX_CHECK(n < (size_t(1) << 31), BCX_INVALID_VALUE, "segmented sort: n must be below 2^31");
  BCX_CHECK(nseg < (size_t(1) << 31), BCX_INVALID_VALUE, "segmented sort: too many segments");
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const SegLayout L = seg_layout<U, VB>(n, nseg);
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, L.total, s, &query);
  if (rc || query) return rc;
  char *base = static_cast<char *>(ts.ptr());
  U *k_main = static_cast<U *>(keys);
  U *k_alt = reinterpret_cast<U *>(base + L.alt_keys);
  VT *v_main = static_cast<VT *>(values);
  VT *v_alt = VB ? reinterpret_cast<VT *>(base + L.alt_vals) : nullptr;
  uint32_t *tile_first = reinterpret_cast<uint32_t *>(base + L.tile_first);
  uint32_t *large_ord = reinterpret_cast<uint32_t *>(base + L.large_ord);
  uint32_t *seg_of_large = reinterpret_cast<uint32_t *>(base + L.seg_of_large);
  uint32_t *tile_seg = reinterpret_cast<uint32_t *>(base + L.tile_seg);
  uint32_t *totals = reinterpret_cast<uint32_t *>(base + L.totals);
  uint32_t *counters = reinterpret_cast<uint32_t *>(base + L.counters);
  uint32_t *seg_hist = reinterpret_cast<uint32_t *>(base + L.seg_hist);
  unsigned long long *status = reinterpret_cast<unsigned long long *>(base + L.status);
  const KeyXform<U> xf = make_xform<U>(kind, desc);
  const std::string obj = "segmented_sort_k" + std::to_string(8 * sizeof(U)) + "_v" + std::to_string(VB);
  uint32_t cap = param_get(obj, "small_tile", uint32_t(SmallCap<U, VB>::value));
  cap = cap >= 4096 ? 4096u : (cap >= 2048 ? 2048u : kMinSmallTile);
  if (cap > uint32_t(SmallCap<U, VB>::value)) cap = uint32_t(SmallCap<U, VB>::value);
  const uint32_t per_sm = param_get(obj, "small_blocks_per_sm", 0u);
  BCX_CUDA(cudaMemsetAsync(base + L.zero_begin, 0, L.zero_bytes, s));
  {
    KernelScope ks("segsort_plan", s);
    segsort_plan_kernel<<<1, kPlanThreads, 0, s>>>(offsets, uint32_t(nseg), cap, TILE, tile_first, large_ord,
                                                   seg_of_large, totals);
    rc = launch_status("segsort_plan");
    if (rc) return rc;
  }
  if (cap == 4096) rc = launch_small<U, VB, 4096>(s, k_main, v_main, offsets, nseg, xf, counters, per_sm, ds);
  else if (cap == 2048) rc = launch_small<U, VB, 2048>(s, k_main, v_main, offsets, nseg, xf, counters, per_sm, ds);
  else rc = launch_small<U, VB, 1024>(s, k_main, v_main, offsets, nseg, xf, counters, per_sm, ds);
  if (rc) return rc;
  {
    KernelScope ks("segsort_hist", s);
    segsort_hist_kernel<U, PASSES><<<L.max_tiles, kHistThreads, 0, s>>>(
        k_main, offsets, uint32_t(nseg), tile_first, large_ord, totals, TILE, xf, seg_hist, tile_seg);
    rc = launch_status("segsort_hist");
    if (rc) return rc;
  }
  {
    KernelScope ks("segsort_starts", s);
    segsort_starts_kernel<PASSES><<<L.max_large, kRadix, 0, s>>>(offsets, seg_of_large, totals, seg_hist);
    rc = launch_status("segsort_starts");
    if (rc) return rc;
  }
  const bool plain = kind == kKeyUnsigned && !desc;
  rc = plain ? seg_onesweep_passes<U, VB, true>(s, L, k_main, k_alt, v_main, v_alt, n, offsets, nseg, tile_first,
                                                large_ord, totals, xf, seg_hist, status, counters, tile_seg,
                                                ds->err_word)
             : seg_onesweep_passes<U, VB, false>(s, L, k_main, k_alt, v_main, v_alt, n, offsets, nseg, tile_first,
                                                 large_ord, totals, xf, seg_hist, status, counters, tile_seg,
                                                 ds->err_word);
  if (rc) return rc;
  if (PASSES & 1) {
    KernelScope ks("segsort_copyback", s);
    segsort_copyback_kernel<U, VB><<<L.max_tiles, 256, 0, s>>>(k_main, k_alt, v_main, v_alt, offsets,
                                                               uint32_t(nseg), tile_first, large_ord, totals,
                                                               tile_seg);
    rc = launch_status("segsort_copyback");
  }
  return rc;
}

template <class U>
bcx_status segsort_vb(cudaStream_t s, size_t vb, void *k, void *v, size_t n, const unsigned long long *offs,
                      size_t nseg, int kind, int desc, void *temp, size_t *tb) {
  switch (vb) {
    case 0: return segsort_t<U, 0>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
    case 1: return segsort_t<U, 1>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
    case 2: return segsort_t<U, 2>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
    case 4: return segsort_t<U, 4>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
    case 8: return segsort_t<U, 8>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
    case 16: return segsort_t<U, 16>(s, k, v, n, offs, nseg, kind, desc, temp, tb);
  }
  set_error("segmented sort: value size %zu not in {1,2,4,8,16}", vb);
  return BCX_INVALID_VALUE;
}

}  // namespace

uint32_t segsort_small_tile_limit(size_t key_bytes, size_t value_bytes) {
  const size_t pair = key_bytes + value_bytes;
  const size_t raw = (96 * 1024) / (2 * pair);
  return raw >= 4096 ? 4096u : (raw >= 2048 ? 2048u : 1024u);
}

}  // namespace bcx

using namespace bcx;

extern "C" bcx_status bcx_segmented_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes,
                                               void *keys, void *values, size_t n, const uint64_t *offsets,
                                               size_t nseg, int descending, void *temp, size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(key_type), BCX_INVALID_VALUE, "invalid key dtype %d", int(key_type));
  if (n == 0 || nseg == 0) {
    if (temp == nullptr && temp_bytes != nullptr) *temp_bytes = 0;
    return BCX_SUCCESS;
  }
  BCX_CHECK(keys && offsets, BCX_INVALID_VALUE, "NULL argument");
  BCX_CHECK(value_bytes == 0 || values, BCX_INVALID_VALUE, "values is NULL");
  const int kind = (key_type == BCX_FLOAT || key_type == BCX_DOUBLE)
                       ? 2
                       : ((key_type == BCX_CHAR || key_type == BCX_SHORT || key_type == BCX_INT || key_type == BCX_LONG)
                              ? 1
                              : 0);
  const auto *offs = reinterpret_cast<const unsigned long long *>(offsets);
  cudaStream_t s = (cudaStream_t)stream;
  const int desc = descending ? 1 : 0;
  switch (dtype_size(key_type)) {
    case 1: return segsort_vb<uint8_t>(s, value_bytes, keys, values, n, offs, nseg, kind, desc, temp, temp_bytes);
    case 2: return segsort_vb<uint16_t>(s, value_bytes, keys, values, n, offs, nseg, kind, desc, temp, temp_bytes);
    case 4: return segsort_vb<uint32_t>(s, value_bytes, keys, values, n, offs, nseg, kind, desc, temp, temp_bytes);
    case 8:
      return segsort_vb<unsigned long long>(s, value_bytes, keys, values, n, offs, nseg, kind, desc, temp,
                                            temp_bytes);
  }
  return BCX_INVALID_VALUE;
}
