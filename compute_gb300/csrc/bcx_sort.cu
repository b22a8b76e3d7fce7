// bcx_sort.cu -- sort / sort_by_key: onesweep LSD radix sort with 8-bit digits.
//
// Reference: detail::radix_sort_impl (algorithm/detail/radix_sort.hpp:253-426)
// runs sizeof(T)*8/4 passes of 4-bit digits; each pass launches a count kernel
// (per-group 16-bin histogram), an exclusive_scan of the block histograms,
// a single work-item scan of the digit totals and a scatter kernel whose
// work-items rank themselves with an O(block) serial loop (:235-239), ping-
// ponging between the input and a temporary (:421-424).  Small inputs go to a
// single work-item insertion sort (sort.hpp:34-80, insertion_sort.hpp:26-159).
//
// GB300 design (onesweep):
//   1. one histogram kernel reads the keys once and builds the 256-bin digit
//      histogram of EVERY pass in shared memory (warp-uniform digits are
//      added once per warp instead of once per lane);
//   2. a one-block prep kernel turns them into per-pass digit start offsets,
//      marks passes whose digit is the same for all keys (an identity
//      permutation: skipped, which keeps the result bit-identical), and
//      decides which buffer each pass reads and writes;
//   3. one kernel per 8-bit digit: each block takes the next tile from an
//      atomic ticket, loads its keys warp-striped and fully coalesced, ranks
//      them within each warp against per-warp digit counters in shared memory
//      (the lanes holding the same digit are found with one ballot per digit
//      bit; stable: ranks follow input order), publishes its 256 digit counts,
//      stages the keys in shared memory in digit order, issues the value
//      loads, then looks back over predecessor tiles per digit for the global
//      offset (decoupled look-back, 64-bit status words tagged with the pass,
//      bounded waits), stages the values and writes the tile out as runs of
//      consecutive addresses;
//   4. if an odd number of passes ran, one copy kernel moves the result back.
// Every launch is asynchronous on the caller's stream; nothing reads back to
// the host, so the whole sort can be captured in a CUDA graph.
//
// The digit of a key is taken from the reference's radix() transform
// (bcx_common.cuh radix_key), so the order of equal-under-transform keys, of
// -0.0/+0.0 and of NaNs is the reference's.
#include <cuda_runtime.h>

#include <string.h>

#include "bcx.h"
#include "bcx_common.cuh"
#include "bcx_internal.h"
#include "bcx_radix.cuh"

namespace bcx {
namespace {

using namespace radix;

// ---------------------------------------------------------------------------
// 1. Histogram of every digit position, one read of the keys.  Keys stream in
// as 16-byte vectors; when the 32 lanes' vectors all hold one key (all-equal
// and heavily skewed distributions), lane 0 adds 32 x N once per digit
// position instead of 32 x N shared-memory atomics on one address.  PLAIN keys
// (unsigned, ascending) skip the key transform.
template <class U, int PASSES>
__device__ __forceinline__ void hist_add(uint32_t (*sh)[kRadix], U k, uint32_t c) {
#pragma unroll
  for (int p = 0; p < PASSES; ++p) atomicAdd(&sh[p][uint32_t(k >> (p * kRadixBits)) & (kRadix - 1)], c);
}

template <class U, int PASSES, bool PLAIN>
__device__ __forceinline__ U hist_key(U x, const KeyXform<U> &xf) {
  return PLAIN ? x : apply_xform<U>(x, xf);
}

template <class U, int PASSES, bool PLAIN>
__global__ void __launch_bounds__(kHistThreads)
radix_histogram_kernel(const U *__restrict__ keys, size_t n, size_t head, size_t nvec, const KeyXform<U> xf,
                       uint32_t *__restrict__ hist) {
  constexpr int N = 16 / sizeof(U);
  __shared__ uint32_t sh[PASSES][kRadix];
  for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistThreads) (&sh[0][0])[i] = 0;
  __syncthreads();
  const unsigned lane = lane_id();
  const size_t warp_id = (size_t(blockIdx.x) * kHistThreads + threadIdx.x) / kWarp;
  const size_t nwarps = size_t(gridDim.x) * kHistThreads / kWarp;
  // Unaligned head and the tail: the first warp, 32 scalars at a time.
  if (warp_id == 0) {
    const size_t tail = head + nvec * N;
    for (size_t b = 0; b < head; b += kWarp)
      if (b + lane < head) hist_add<U, PASSES>(sh, hist_key<U, PASSES, PLAIN>(keys[b + lane], xf), 1u);
    for (size_t b = tail; b < n; b += kWarp)
      if (b + lane < n) hist_add<U, PASSES>(sh, hist_key<U, PASSES, PLAIN>(keys[b + lane], xf), 1u);
  }
  const vec16<U> *vk = reinterpret_cast<const vec16<U> *>(keys + head);
  for (size_t vb = warp_id * kWarp; vb < nvec; vb += nwarps * kWarp) {
    const size_t v = vb + lane;
    const bool valid = v < nvec;
    vec16<U> r;
    if (valid) r = ld_stream16(vk + v);
    bool same = valid;
#pragma unroll
    for (int j = 1; j < N; ++j) same = same && r.v[j] == r.v[0];
    const U k0 = __shfl_sync(0xffffffffu, r.v[0], 0);
    if (__all_sync(0xffffffffu, same && r.v[0] == k0)) {
      if (lane == 0) hist_add<U, PASSES>(sh, hist_key<U, PASSES, PLAIN>(k0, xf), uint32_t(kWarp * N));
    } else if (valid) {
#pragma unroll
      for (int j = 0; j < N; ++j) hist_add<U, PASSES>(sh, hist_key<U, PASSES, PLAIN>(r.v[j], xf), 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistThreads) {
    const uint32_t c = (&sh[0][0])[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

// The same counts with one column of counters per lane: lane l adds to
// column l of each (pass, digit) row, so the 32 lanes of an atomic always hit
// 32 different banks whatever their digits (with one shared row per digit,
// random digits put about 3.5 lanes on the busiest bank and the atomics
// serialise on it).  One block of kHistLaneThreads per SM holds
// PASSES * kRadix * 32 counters (128 KB for 32-bit keys); the columns are
// summed at the end, each warp reading a rotated order so the sums are
// conflict-free too.  Each lane keeps kHistLaneUnroll 16-byte loads in
// flight.  sort_by_key of 2^28 uniform uint32 pairs on GB300: 5.36 ms with
// the shared rows, 5.11 ms with lane columns (the count at the read
// bandwidth); Zipf(1.1) keys 5.14 -> 4.99 ms.  Keys of up to 4 bytes take this
// kernel (tunable "radix_sort"/"histogram_lanes", 0 = shared rows); 64-bit
// keys, whose 8 passes would need 256 KB, keep the shared rows.
constexpr int kHistLaneThreads = 1024;
constexpr int kHistLaneUnroll = 4;
template <int PASSES>
constexpr size_t hist_lane_smem() {
  return size_t(PASSES) * kRadix * kWarp * sizeof(uint32_t);
}

template <class U, int PASSES>
__device__ __forceinline__ void hist_lane_add(uint32_t *col, U k, uint32_t c) {
#pragma unroll
  for (int p = 0; p < PASSES; ++p)
    atomicAdd(col + (p * kRadix + (uint32_t(k >> (p * kRadixBits)) & (kRadix - 1))) * kWarp, c);
}

template <class U, int PASSES, bool PLAIN>
__global__ void __launch_bounds__(kHistLaneThreads, 1)
radix_histogram_lanes_kernel(const U *__restrict__ keys, size_t n, size_t head, size_t nvec, const KeyXform<U> xf,
                             uint32_t *__restrict__ hist) {
  constexpr int N = 16 / sizeof(U);
  extern __shared__ __align__(16) uint32_t shl[];  // [PASSES][kRadix][kWarp]
  for (int i = threadIdx.x; i < PASSES * kRadix * kWarp; i += kHistLaneThreads) shl[i] = 0;
  __syncthreads();
  const unsigned lane = lane_id();
  uint32_t *col = shl + lane;
  const size_t warp_id = (size_t(blockIdx.x) * kHistLaneThreads + threadIdx.x) / kWarp;
  const size_t nwarps = size_t(gridDim.x) * kHistLaneThreads / kWarp;
  if (warp_id == 0) {
    const size_t tail = head + nvec * N;
    for (size_t b = 0; b < head; b += kWarp)
      if (b + lane < head) hist_lane_add<U, PASSES>(col, hist_key<U, PASSES, PLAIN>(keys[b + lane], xf), 1u);
    for (size_t b = tail; b < n; b += kWarp)
      if (b + lane < n) hist_lane_add<U, PASSES>(col, hist_key<U, PASSES, PLAIN>(keys[b + lane], xf), 1u);
  }
  const vec16<U> *vk = reinterpret_cast<const vec16<U> *>(keys + head);
  constexpr size_t kStep = size_t(kWarp) * kHistLaneUnroll;
  for (size_t vb = warp_id * kStep; vb < nvec; vb += nwarps * kStep) {
    vec16<U> r[kHistLaneUnroll];
#pragma unroll
    for (int u = 0; u < kHistLaneUnroll; ++u)
      if (vb + u * kWarp + lane < nvec) r[u] = ld_stream16(vk + vb + u * kWarp + lane);
#pragma unroll
    for (int u = 0; u < kHistLaneUnroll; ++u)
      if (vb + u * kWarp + lane < nvec) {
#pragma unroll
        for (int j = 0; j < N; ++j) hist_lane_add<U, PASSES>(col, hist_key<U, PASSES, PLAIN>(r[u].v[j], xf), 1u);
      }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < PASSES * kRadix; i += kHistLaneThreads) {
    uint32_t c = 0;
#pragma unroll 8
    for (int j = 0; j < kWarp; ++j) c += shl[i * kWarp + ((j + i) & (kWarp - 1))];
    if (c) atomicAdd(&hist[i], c);
  }
}

// 2. Digit start offsets per pass, pass skipping and buffer schedule.
__global__ void __launch_bounds__(kRadix)
radix_prep_kernel(uint32_t *__restrict__ hist, int passes, uint32_t n,
                  SortControl *__restrict__ ctrl) {
  __shared__ uint32_t warp_sum[kRadix / kWarp];
  __shared__ uint32_t skip[8];
  const unsigned d = threadIdx.x, lane = lane_id(), w = d / kWarp;
  for (int p = 0; p < passes; ++p) {
    const uint32_t c = hist[p * kRadix + d];
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (int(lane) >= o) incl += t;
    }
    if (lane == kWarp - 1) warp_sum[w] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (unsigned j = 0; j < w; ++j) before += warp_sum[j];
    const int all_one = __syncthreads_or(c == n);
    hist[p * kRadix + d] = before + incl - c;  // exclusive start of digit d
    if (d == 0) skip[p] = all_one ? 1u : 0u;
    __syncthreads();
  }
  if (d == 0) {
    uint32_t alt = 0;
    for (int p = 0; p < 8; ++p) {
      const uint32_t sk = p < passes ? skip[p] : 1u;
      ctrl->skip[p] = sk;
      ctrl->src_alt[p] = alt;
      if (!sk) alt ^= 1u;
    }
    ctrl->final_alt = alt;
  }
}

// 3. One onesweep pass over digit `pass` (tiles taken from an atomic ticket,
// so a tile only ever waits on tiles already running).
template <class U, int VB, bool PLAIN>
__global__ void __launch_bounds__(kSortThreads, kSortBlocksPerSm)
radix_onesweep_kernel(U *__restrict__ keys_main, U *__restrict__ keys_alt,
                      typename value_type_of<VB>::type *__restrict__ vals_main,
                      typename value_type_of<VB>::type *__restrict__ vals_alt, uint32_t n,
                      int pass, const KeyXform<U> xf, const uint32_t *__restrict__ digit_start,
                      unsigned long long *__restrict__ status, uint32_t *__restrict__ tile_counter,
                      const SortControl *__restrict__ ctrl, uint32_t *err) {
  constexpr uint32_t TILE = OnesweepSmem<U, VB>::TILE;
  __shared__ uint32_t s_tile;
  if (ctrl->skip[pass]) return;
  const bool from_alt = ctrl->src_alt[pass] != 0;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * TILE;
  const uint32_t count = (n - base) < TILE ? (n - base) : TILE;
  onesweep_tile<U, VB, PLAIN>(from_alt ? keys_alt : keys_main, from_alt ? keys_main : keys_alt,
                              from_alt ? vals_alt : vals_main, from_alt ? vals_main : vals_alt, base, count, tile,
                              0u, digit_start + pass * kRadix, n, pass, pass * kRadixBits, xf, status, err);
}

// 4. Copy the result back when it ended in the temporary buffers.
template <class U, int VB>
__global__ void radix_copyback_kernel(U *__restrict__ keys_main, const U *__restrict__ keys_alt,
                                      typename value_type_of<VB>::type *__restrict__ vals_main,
                                      const typename value_type_of<VB>::type *__restrict__ vals_alt,
                                      size_t n, const SortControl *__restrict__ ctrl) {
  if (!ctrl->final_alt) return;
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    keys_main[i] = keys_alt[i];
    if (VB) vals_main[i] = vals_alt[i];
  }
}

// Serial insertion sort by one thread with the functor's comparison on the
// typed keys (insertion_sort.hpp:26-159): value moves left while
// compare(value, previous) holds.
template <class T, int VB>
__global__ void insertion_sort_kernel(T *__restrict__ keys, typename value_type_of<VB>::type *__restrict__ vals,
                                      int n, int desc) {
  typedef typename value_type_of<VB>::type VT;
  T k[32];
  VT v[VB ? 32 : 1];
  for (int i = 0; i < n; ++i) {
    k[i] = keys[i];
    if (VB) v[i] = vals[i];
  }
  for (int i = 1; i < n; ++i) {
    const T key = k[i];
    VT value;
    if (VB) value = v[i];
    int pos = i;
    while (pos > 0 && (desc ? (key > k[pos - 1]) : (key < k[pos - 1]))) {
      k[pos] = k[pos - 1];
      if (VB) v[pos] = v[pos - 1];
      --pos;
    }
    k[pos] = key;
    if (VB) v[pos] = value;
  }
  for (int i = 0; i < n; ++i) {
    keys[i] = k[i];
    if (VB) vals[i] = v[i];
  }
}

// ---------------------------------------------------------------------------
struct SortLayout {
  size_t alt_keys = 0, alt_vals = 0, hist = 0, ctrl = 0, counters = 0, status = 0, total = 0;
  size_t zero_begin = 0, zero_bytes = 0;
  uint32_t tiles = 0;
};

template <class U>
SortLayout sort_layout(size_t n, size_t vb, int passes) {
  constexpr int IPT = items_per_thread<U>::value;
  SortLayout L;
  L.tiles = uint32_t(div_up(n, size_t(kSortThreads) * IPT));
  size_t off = 0;
  L.alt_keys = off;
  off += align256(n * sizeof(U));
  L.alt_vals = off;
  off += align256(n * vb);
  L.hist = off;
  off += align256(size_t(passes) * kRadix * 4);
  L.ctrl = off;
  off += 256;
  L.counters = off;
  off += 256;
  L.status = off;  // one array for every pass (status words carry the pass)
  off += align256(size_t(L.tiles) * kRadix * 8);
  L.total = off;
  L.zero_begin = L.hist;
  L.zero_bytes = off - L.hist;
  return L;
}

template <class U, int VB, bool PLAIN>
bcx_status onesweep_passes(cudaStream_t s, const SortLayout &L, U *k_main, U *k_alt,
                           typename value_type_of<VB>::type *v_main, typename value_type_of<VB>::type *v_alt,
                           size_t n, const KeyXform<U> &xf, const uint32_t *hist, unsigned long long *status,
                           uint32_t *counters, const SortControl *ctrl, uint32_t *err) {
  const size_t smem = OnesweepSmem<U, VB>::kBytes;
  static std::atomic<uint64_t> optin{0};
  BCX_CUDA(smem_optin(reinterpret_cast<const void *>(radix_onesweep_kernel<U, VB, PLAIN>), int(smem), &optin));
  for (int p = 0; p < int(sizeof(U)); ++p) {
    KernelScope ks("radix_onesweep", s);
    radix_onesweep_kernel<U, VB, PLAIN><<<L.tiles, kSortThreads, smem, s>>>(
        k_main, k_alt, v_main, v_alt, uint32_t(n), p, xf, hist, status, counters + p, ctrl, err);
    bcx_status rc = launch_status("radix_onesweep");
    if (rc) return rc;
  }
  return BCX_SUCCESS;
}

template <class U, int VB>
bcx_status radix_sort_t(cudaStream_t s, void *keys, void *values, size_t n, int kind, int desc,
                        void *temp, size_t *temp_bytes) {
  typedef typename value_type_of<VB>::type VT;
  constexpr int PASSES = int(sizeof(U));
  BCX_CHECK(n <= kMaxSortN, BCX_INVALID_VALUE, "radix sort: n must be below 2^32 (got %zu)", n);
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const SortLayout L = sort_layout<U>(n, VB, PASSES);
  if (n < 2 && !(temp == nullptr && temp_bytes != nullptr)) return BCX_SUCCESS;
  TempStorage ts;
  bool query = false;
  rc = ts.acquire(temp, temp_bytes, L.total, s, &query);
  if (rc || query) return rc;
  char *base = static_cast<char *>(ts.ptr());
  U *k_main = static_cast<U *>(keys);
  U *k_alt = reinterpret_cast<U *>(base + L.alt_keys);
  VT *v_main = static_cast<VT *>(values);
  VT *v_alt = VB ? reinterpret_cast<VT *>(base + L.alt_vals) : nullptr;
  uint32_t *hist = reinterpret_cast<uint32_t *>(base + L.hist);
  SortControl *ctrl = reinterpret_cast<SortControl *>(base + L.ctrl);
  uint32_t *counters = reinterpret_cast<uint32_t *>(base + L.counters);
  unsigned long long *status = reinterpret_cast<unsigned long long *>(base + L.status);
  BCX_CUDA(cudaMemsetAsync(base + L.zero_begin, 0, L.zero_bytes, s));
  const KeyXform<U> xf = make_xform<U>(kind, desc);
  {
    KernelScope ks("radix_histogram", s);
    constexpr int N = 16 / sizeof(U);
    const uintptr_t a = reinterpret_cast<uintptr_t>(keys);
    size_t head = (a % sizeof(U)) ? n : ((16u - (a & 15u)) & 15u) / sizeof(U);
    if (head > n) head = n;
    const size_t nvec = (n - head) / N;
    bool lanes = false;
    if constexpr (PASSES <= 4) {
      if (param_get("radix_sort", "histogram_lanes", 1u) != 0) {
        lanes = true;
        constexpr size_t smem = hist_lane_smem<PASSES>();
        static std::atomic<uint64_t> optin_plain{0}, optin_xf{0};
        BCX_CUDA(smem_optin(reinterpret_cast<const void *>(radix_histogram_lanes_kernel<U, PASSES, true>),
                            int(smem), &optin_plain));
        BCX_CUDA(smem_optin(reinterpret_cast<const void *>(radix_histogram_lanes_kernel<U, PASSES, false>),
                            int(smem), &optin_xf));
        size_t blocks = div_up(nvec, size_t(kHistLaneThreads) * kHistLaneUnroll);
        if (blocks > size_t(ds->sm_count)) blocks = size_t(ds->sm_count);
        if (blocks < 1) blocks = 1;
        if (kind == kKeyUnsigned && !desc)
          radix_histogram_lanes_kernel<U, PASSES, true><<<unsigned(blocks), kHistLaneThreads, smem, s>>>(
              k_main, n, head, nvec, xf, hist);
        else
          radix_histogram_lanes_kernel<U, PASSES, false><<<unsigned(blocks), kHistLaneThreads, smem, s>>>(
              k_main, n, head, nvec, xf, hist);
      }
    }
    if (!lanes) {
      size_t blocks = div_up(nvec, size_t(kHistThreads) * 4);
      size_t cap = size_t(ds->sm_count) * 8;
      if (blocks > cap) blocks = cap;
      if (blocks < 1) blocks = 1;
      if (kind == kKeyUnsigned && !desc)
        radix_histogram_kernel<U, PASSES, true><<<unsigned(blocks), kHistThreads, 0, s>>>(k_main, n, head, nvec, xf,
                                                                                          hist);
      else
        radix_histogram_kernel<U, PASSES, false><<<unsigned(blocks), kHistThreads, 0, s>>>(k_main, n, head, nvec,
                                                                                           xf, hist);
    }
    rc = launch_status("radix_histogram");
    if (rc) return rc;
  }
  {
    KernelScope ks("radix_prep", s);
    radix_prep_kernel<<<1, kRadix, 0, s>>>(hist, PASSES, uint32_t(n), ctrl);
    rc = launch_status("radix_prep");
    if (rc) return rc;
  }
  const bool plain = kind == kKeyUnsigned && !desc;
  rc = plain ? onesweep_passes<U, VB, true>(s, L, k_main, k_alt, v_main, v_alt, n, xf, hist, status, counters, ctrl,
                                            ds->err_word)
             : onesweep_passes<U, VB, false>(s, L, k_main, k_alt, v_main, v_alt, n, xf, hist, status, counters, ctrl,
                                             ds->err_word);
  if (rc) return rc;
  KernelScope ks("radix_copyback", s);
  size_t blocks = div_up(n, 256);
  size_t cap = size_t(ds->sm_count) * 8;
  if (blocks > cap) blocks = cap;
  radix_copyback_kernel<U, VB><<<unsigned(blocks), 256, 0, s>>>(k_main, k_alt, v_main, v_alt, n, ctrl);
  return launch_status("radix_copyback");
}

template <class T, int VB>
bcx_status insertion_t(cudaStream_t s, void *keys, void *values, size_t n, int desc) {
  typedef typename value_type_of<VB>::type VT;
  KernelScope ks("insertion_sort", s);
  insertion_sort_kernel<T, VB><<<1, 1, 0, s>>>(static_cast<T *>(keys), static_cast<VT *>(values), int(n), desc);
  return launch_status("insertion_sort");
}

int key_kind(bcx_dtype t) {
  if (t == BCX_FLOAT || t == BCX_DOUBLE) return kKeyFloat;
  if (t == BCX_CHAR || t == BCX_SHORT || t == BCX_INT || t == BCX_LONG) return kKeySigned;
  return kKeyUnsigned;
}

template <class U>
bcx_status radix_by_vb(cudaStream_t s, size_t vb, void *k, void *v, size_t n, int kind, int desc,
                       void *temp, size_t *tb) {
  switch (vb) {
    case 0: return radix_sort_t<U, 0>(s, k, v, n, kind, desc, temp, tb);
    case 1: return radix_sort_t<U, 1>(s, k, v, n, kind, desc, temp, tb);
    case 2: return radix_sort_t<U, 2>(s, k, v, n, kind, desc, temp, tb);
    case 4: return radix_sort_t<U, 4>(s, k, v, n, kind, desc, temp, tb);
    case 8: return radix_sort_t<U, 8>(s, k, v, n, kind, desc, temp, tb);
    case 16: return radix_sort_t<U, 16>(s, k, v, n, kind, desc, temp, tb);
  }
  set_error("radix sort: value size %zu not in {1,2,4,8,16}", vb);
  return BCX_INVALID_VALUE;
}

bcx_status radix_entry(cudaStream_t s, bcx_dtype kt, size_t vb, void *keys, void *values, size_t n,
                       int desc, void *temp, size_t *tb) {
  BCX_CHECK(dtype_valid(kt), BCX_INVALID_VALUE, "invalid key dtype %d", int(kt));
  BCX_CHECK(n == 0 || keys != nullptr, BCX_INVALID_VALUE, "keys is NULL");
  BCX_CHECK(vb == 0 || n == 0 || values != nullptr, BCX_INVALID_VALUE, "values is NULL");
  const int kind = key_kind(kt);
  desc = desc ? 1 : 0;
  switch (dtype_size(kt)) {
    case 1: return radix_by_vb<uint8_t>(s, vb, keys, values, n, kind, desc, temp, tb);
    case 2: return radix_by_vb<uint16_t>(s, vb, keys, values, n, kind, desc, temp, tb);
    case 4: return radix_by_vb<uint32_t>(s, vb, keys, values, n, kind, desc, temp, tb);
    case 8: return radix_by_vb<unsigned long long>(s, vb, keys, values, n, kind, desc, temp, tb);
  }
  return BCX_INVALID_VALUE;
}

template <class T>
bcx_status insertion_by_vb(cudaStream_t s, size_t vb, void *k, void *v, size_t n, int desc) {
  switch (vb) {
    case 0: return insertion_t<T, 0>(s, k, v, n, desc);
    case 1: return insertion_t<T, 1>(s, k, v, n, desc);
    case 2: return insertion_t<T, 2>(s, k, v, n, desc);
    case 4: return insertion_t<T, 4>(s, k, v, n, desc);
    case 8: return insertion_t<T, 8>(s, k, v, n, desc);
    case 16: return insertion_t<T, 16>(s, k, v, n, desc);
  }
  set_error("sort: value size %zu not in {1,2,4,8,16}", vb);
  return BCX_INVALID_VALUE;
}

bcx_status insertion_entry(cudaStream_t s, bcx_dtype kt, size_t vb, void *k, void *v, size_t n, int desc) {
  switch (kt) {
    case BCX_CHAR: return insertion_by_vb<int8_t>(s, vb, k, v, n, desc);
    case BCX_UCHAR: return insertion_by_vb<uint8_t>(s, vb, k, v, n, desc);
    case BCX_SHORT: return insertion_by_vb<int16_t>(s, vb, k, v, n, desc);
    case BCX_USHORT: return insertion_by_vb<uint16_t>(s, vb, k, v, n, desc);
    case BCX_INT: return insertion_by_vb<int32_t>(s, vb, k, v, n, desc);
    case BCX_UINT: return insertion_by_vb<uint32_t>(s, vb, k, v, n, desc);
    case BCX_LONG: return insertion_by_vb<long long>(s, vb, k, v, n, desc);
    case BCX_ULONG: return insertion_by_vb<unsigned long long>(s, vb, k, v, n, desc);
    case BCX_FLOAT: return insertion_by_vb<float>(s, vb, k, v, n, desc);
    case BCX_DOUBLE: return insertion_by_vb<double>(s, vb, k, v, n, desc);
  }
  return BCX_INVALID_VALUE;
}

}  // namespace
}  // namespace bcx

using namespace bcx;

extern "C" {

bcx_status bcx_radix_sort_keys(bcx_stream stream, bcx_dtype key_type, void *keys, size_t n,
                               int descending, void *temp, size_t *temp_bytes) {
  clear_error();
  return radix_entry((cudaStream_t)stream, key_type, 0, keys, nullptr, n, descending, temp, temp_bytes);
}

bcx_status bcx_radix_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes, void *keys,
                                void *values, size_t n, int descending, void *temp,
                                size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(value_bytes != 0, BCX_INVALID_VALUE, "value_bytes is 0");
  return radix_entry((cudaStream_t)stream, key_type, value_bytes, keys, values, n, descending, temp,
                     temp_bytes);
}

bcx_status bcx_sort_keys(bcx_stream stream, bcx_dtype key_type, void *keys, size_t n, int descending,
                         void *temp, size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(key_type), BCX_INVALID_VALUE, "invalid key dtype %d", int(key_type));
  if (n <= 32) {
    if (temp == nullptr && temp_bytes != nullptr) {
      *temp_bytes = 0;
      return BCX_SUCCESS;
    }
    if (n < 2) return BCX_SUCCESS;
    return insertion_entry((cudaStream_t)stream, key_type, 0, keys, nullptr, n, descending ? 1 : 0);
  }
  return radix_entry((cudaStream_t)stream, key_type, 0, keys, nullptr, n, descending, temp, temp_bytes);
}

bcx_status bcx_sort_pairs(bcx_stream stream, bcx_dtype key_type, size_t value_bytes, void *keys,
                          void *values, size_t n, int descending, void *temp, size_t *temp_bytes) {
  clear_error();
  BCX_CHECK(dtype_valid(key_type), BCX_INVALID_VALUE, "invalid key dtype %d", int(key_type));
  BCX_CHECK(value_bytes != 0, BCX_INVALID_VALUE, "value_bytes is 0");
  if (n < 32) {
    if (temp == nullptr && temp_bytes != nullptr) {
      *temp_bytes = 0;
      return BCX_SUCCESS;
    }
    if (n < 2) return BCX_SUCCESS;
    return insertion_entry((cudaStream_t)stream, key_type, value_bytes, keys, values, n, descending ? 1 : 0);
  }
  return radix_entry((cudaStream_t)stream, key_type, value_bytes, keys, values, n, descending, temp,
                     temp_bytes);
}

bcx_status bcx_sort_pairs_host(bcx_stream stream, bcx_dtype key_type, size_t value_bytes,
                               void *host_keys, void *host_values, size_t n, int descending) {
  clear_error();
  BCX_CHECK(dtype_valid(key_type), BCX_INVALID_VALUE, "invalid key dtype %d", int(key_type));
  if (n == 0) return BCX_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  const size_t kb = n * dtype_size(key_type), vb = n * value_bytes;
  void *dk = nullptr, *dv = nullptr;
  BCX_CUDA(cudaMallocAsync(&dk, kb, s));
  if (vb) {
    cudaError_t e = cudaMallocAsync(&dv, vb, s);
    if (e != cudaSuccess) {
      cudaFreeAsync(dk, s);
      return cuda_status(e, "cudaMallocAsync(values)");
    }
  }
  // Each direction's copies are split over the caller's stream and the
  // library's second stream (keys on one, values on the other; keys-only
  // sorts split the keys in halves), so two copy engines share the link.
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
  cudaStream_t s2 = ds->aux_stream;
  char *hk = static_cast<char *>(host_keys), *hv = static_cast<char *>(host_values);
  char *dkc = static_cast<char *>(dk), *dvc = static_cast<char *>(dv);
  const size_t khalf = vb ? kb : (kb / 2) & ~size_t(255);
  auto split_copy = [&](cudaMemcpyKind kind) -> cudaError_t {
    cudaError_t r = cudaEventRecord(fork, s);
    if (r == cudaSuccess) r = cudaStreamWaitEvent(s2, fork, 0);
    const bool h2d = kind == cudaMemcpyHostToDevice;
    if (r == cudaSuccess)
      r = h2d ? cudaMemcpyAsync(dkc, hk, khalf, kind, s) : cudaMemcpyAsync(hk, dkc, khalf, kind, s);
    if (r == cudaSuccess && kb > khalf)
      r = h2d ? cudaMemcpyAsync(dkc + khalf, hk + khalf, kb - khalf, kind, s2)
              : cudaMemcpyAsync(hk + khalf, dkc + khalf, kb - khalf, kind, s2);
    if (r == cudaSuccess && vb) r = h2d ? cudaMemcpyAsync(dvc, hv, vb, kind, s2) : cudaMemcpyAsync(hv, dvc, vb, kind, s2);
    if (r == cudaSuccess) r = cudaEventRecord(join, s2);
    if (r == cudaSuccess) r = cudaStreamWaitEvent(s, join, 0);
    return r;
  };
  if (e == cudaSuccess) e = split_copy(cudaMemcpyHostToDevice);
  if (e != cudaSuccess) rc = cuda_status(e, "copy to device");
  if (!rc) {
    rc = vb ? bcx_sort_pairs(stream, key_type, value_bytes, dk, dv, n, descending, nullptr, nullptr)
            : bcx_sort_keys(stream, key_type, dk, n, descending, nullptr, nullptr);
  }
  if (!rc) {
    e = split_copy(cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_status(e, "copy to host");
  }
  cudaFreeAsync(dk, s);
  if (dv) cudaFreeAsync(dv, s);
  e = cudaStreamSynchronize(s);
  if (!rc && e != cudaSuccess) rc = cuda_status(e, "cudaStreamSynchronize");
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  return rc;
}

}  // extern "C"
