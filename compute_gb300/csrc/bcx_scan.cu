// bcx_scan.cu -- the exclusive_scan / inclusive_scan entry points: bcx_scan,
// which hands each element type to its group's translation unit
// (bcx_scan_small/word/wide/float.cu), and bcx_scan_noalloc.  The kernels and
// their design are in bcx_scan.cuh.
#include "bcx_scan.cuh"

extern "C" bcx_status bcx_scan(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive,
                               const void *init, const void *in, void *out, size_t n,
                               int compensated, void *temp, size_t *temp_bytes) {
  using namespace bcx;
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (n == 0) {
    if (temp == nullptr && temp_bytes != nullptr) *temp_bytes = 0;
    return BCX_SUCCESS;
  }
  BCX_CHECK(in != nullptr && out != nullptr, BCX_INVALID_VALUE, "NULL input or output");
  unsigned char zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const void *init_p = (exclusive && init) ? init : zero;
  cudaStream_t s = (cudaStream_t)stream;
  bcx_status rc = BCX_UNSUPPORTED;
  switch (type) {
    case BCX_CHAR:
    case BCX_UCHAR:
    case BCX_SHORT:
    case BCX_USHORT: rc = scan_small_ints(s, type, op, exclusive, init_p, in, out, n, temp, temp_bytes); break;
    case BCX_INT:
    case BCX_UINT: rc = scan_word_ints(s, type, op, exclusive, init_p, in, out, n, temp, temp_bytes); break;
    case BCX_LONG:
    case BCX_ULONG: rc = scan_wide_ints(s, type, op, exclusive, init_p, in, out, n, temp, temp_bytes); break;
    case BCX_FLOAT:
    case BCX_DOUBLE:
      rc = scan_floats(s, type, op, exclusive, init_p, in, out, n, compensated, temp, temp_bytes);
      break;
  }
  if (rc == BCX_UNSUPPORTED) set_error("scan: functor %d not provided for dtype %d", int(op), int(type));
  return rc;
}

// ---------------------------------------------------------------------------
// Scan that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they need a
// scan: a host application that owns every device allocation through its own
// pool and forbids libraries from calling cudaMalloc, or a latency-critical
// path where cudaMalloc/cudaFree (which may synchronize the device) is not
// acceptable.  bcx_scan_noalloc serves them: its look-back scratch (the tile
// ticket and the per-tile status words) and its error word live in one fixed
// array compiled into this library, so the call needs only the caller's input
// and output.  It also leaves the library's per-device state alone (that state
// allocates an error word and a stream and configures the default memory
// pool the first time any other entry point runs on a device).
//
// The array is kNoAllocScratchBytes (5 MiB + 4 KiB) on every GPU that loads
// the library and stays allocated until the process exits.  Its size covers
// the per-call limits below with any input alignment; larger n is rejected.
// All calls share it: each call clears the part it uses on its own stream
// before the scan kernel runs, so back-to-back calls are fine, but calls whose
// work overlaps on the GPU (different streams, or different host threads)
// race on the array and must be serialized by the caller.
namespace bcx {
namespace {

// Layout: [0, 128) tile ticket, cleared by every call; [128, 132) error word
// (a bounded wait that expired), kept until bcx_device_error_check reads and
// clears it; tile status words from byte 256.
constexpr size_t kNoAllocHeader = 256;
constexpr size_t kNoAllocErrOffset = 128;
// Per-call limits, by the carry between tiles: 2^30 elements of 1-, 2- and
// 4-byte types (4-byte carries); 2^28 of 8-byte types and compensated float
// (8-byte carries); 2^27 of compensated double (16-byte carries).
constexpr size_t kNoAllocMax4 = size_t(1) << 30;
constexpr size_t kNoAllocMax8 = size_t(1) << 28;
constexpr size_t kNoAllocMax16 = size_t(1) << 27;
constexpr size_t kNoAllocScratchBytes = (size_t(5) << 20) + 4096;
constexpr int kNoAllocThreads = 128;
constexpr int kNoAllocVectorsPerThread = 4;
static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.  In host code
// the array's name only stands in for the symbol, so the address is looked up
// once per device (with that device current) and cached.
static std::mutex g_noalloc_mu;
static std::map<int, void *> g_noalloc_ptr;

bcx_status noalloc_scratch(void **out) {
  int dev = 0;
  BCX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  auto it = g_noalloc_ptr.find(dev);
  if (it != g_noalloc_ptr.end()) {
    *out = it->second;
    return BCX_SUCCESS;
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(scan scratch)");
  g_noalloc_ptr[dev] = p;
  *out = p;
  return BCX_SUCCESS;
}

template <class T, class P>
bcx_status run_scan_noalloc_t(cudaStream_t s, int exclusive, const void *init, const void *in, void *out,
                              size_t n) {
  typedef typename P::Carry Carry;
  typedef TileStatus<Carry> Status;
  constexpr int N = 16 / sizeof(T);
  // Fixed tile shape, so the size limit of the fixed scratch array does not
  // move when the allocating scan is retuned.
  constexpr int V = kNoAllocVectorsPerThread;
  constexpr size_t tile_elems = size_t(kNoAllocThreads) * V * N;
  constexpr size_t max_n = sizeof(Carry) == 4 ? kNoAllocMax4 : (sizeof(Carry) == 8 ? kNoAllocMax8 : kNoAllocMax16);
  // Worst case: max_n elements behind an unaligned head (one extra tile).
  static_assert(kNoAllocHeader + Status::bytes((max_n + tile_elems - 1) / tile_elems + 1) <= kNoAllocScratchBytes,
                "no-alloc scratch array too small for its documented limit");
  if (n > max_n) {
    set_error("bcx_scan_noalloc: n = %zu is above its limit of %zu elements for this type and functor "
              "(the fixed scratch array is %zu bytes; use bcx_scan for more)",
              n, max_n, kNoAllocScratchBytes);
    return BCX_INVALID_BUFFER_SIZE;
  }
  void *scratch = nullptr;
  bcx_status rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  char *base = static_cast<char *>(scratch);
  uint32_t *err = reinterpret_cast<uint32_t *>(base + kNoAllocErrOffset);
  const uintptr_t ain = reinterpret_cast<uintptr_t>(in), aout = reinterpret_cast<uintptr_t>(out);
  const bool elem_aligned = (ain % sizeof(T) == 0) && (aout % sizeof(T) == 0);
  const bool vec_ok = elem_aligned && ((ain & 15u) == (aout & 15u));
  const size_t head_pad = vec_ok ? (ain & 15u) / sizeof(T) : 0;
  const size_t tiles = div_up(n + head_pad, tile_elems);
  const Carry init_carry = P::host_carry(init);
  const T *pin = static_cast<const T *>(in);
  T *pout = static_cast<T *>(out);
  if (tiles <= 1) {
    Status st{};
    KernelScope ks("scan_single", s);
    scan_tile_kernel<T, P, kNoAllocThreads, V, true, Status><<<1, kNoAllocThreads, 0, s>>>(
        pin, pout, n, head_pad, vec_ok ? 1 : 0, exclusive, init_carry, st, nullptr, err);
    return launch_status("scan_single");
  }
  uint32_t *counter = reinterpret_cast<uint32_t *>(base);
  Status st;
  st.bind(base + kNoAllocHeader, tiles);
  // The array keeps the previous call's ticket and status words: clear them.
  BCX_CUDA(cudaMemsetAsync(base, 0, kNoAllocErrOffset, s));
  BCX_CUDA(st.clear(tiles, s));
  KernelScope ks("scan_lookback", s);
  scan_tile_kernel<T, P, kNoAllocThreads, V, false, Status><<<unsigned(tiles), kNoAllocThreads, 0, s>>>(
      pin, pout, n, head_pad, vec_ok ? 1 : 0, exclusive, init_carry, st, counter, err);
  return launch_status("scan_lookback");
}

template <class T>
bcx_status noalloc_int(cudaStream_t s, int op, int ex, const void *init, const void *in, void *out,
                       size_t n) {
  switch (op) {
    case BCX_PLUS: return run_scan_noalloc_t<T, ScanPlain<T, op_plus>>(s, ex, init, in, out, n);
    case BCX_MULTIPLIES: return run_scan_noalloc_t<T, ScanPlain<T, op_multiplies>>(s, ex, init, in, out, n);
    case BCX_MIN: return run_scan_noalloc_t<T, ScanPlain<T, op_min>>(s, ex, init, in, out, n);
    case BCX_MAX: return run_scan_noalloc_t<T, ScanPlain<T, op_max>>(s, ex, init, in, out, n);
    case BCX_BIT_AND: return run_scan_noalloc_t<T, ScanPlain<T, op_bit_and>>(s, ex, init, in, out, n);
    case BCX_BIT_OR: return run_scan_noalloc_t<T, ScanPlain<T, op_bit_or>>(s, ex, init, in, out, n);
    case BCX_BIT_XOR: return run_scan_noalloc_t<T, ScanPlain<T, op_bit_xor>>(s, ex, init, in, out, n);
  }
  return BCX_UNSUPPORTED;
}

template <class T>
bcx_status noalloc_float(cudaStream_t s, int op, int ex, const void *init, const void *in, void *out,
                         size_t n, int comp) {
  switch (op) {
    case BCX_PLUS:
      if (comp) {
        if (sizeof(T) == 4) return run_scan_noalloc_t<float, ScanCompF32>(s, ex, init, in, out, n);
        return run_scan_noalloc_t<double, ScanCompF64>(s, ex, init, in, out, n);
      }
      return run_scan_noalloc_t<T, ScanPlain<T, op_plus>>(s, ex, init, in, out, n);
    case BCX_MULTIPLIES: return run_scan_noalloc_t<T, ScanPlain<T, op_multiplies>>(s, ex, init, in, out, n);
    case BCX_MIN: return run_scan_noalloc_t<T, ScanPlain<T, op_min>>(s, ex, init, in, out, n);
    case BCX_MAX: return run_scan_noalloc_t<T, ScanPlain<T, op_max>>(s, ex, init, in, out, n);
  }
  return BCX_UNSUPPORTED;
}

}  // namespace

bcx_status noalloc_take_error(uint32_t *word) {
  *word = 0;
  int dev = 0;
  BCX_CUDA(cudaGetDevice(&dev));
  void *p = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    auto it = g_noalloc_ptr.find(dev);
    if (it == g_noalloc_ptr.end()) return BCX_SUCCESS;  // never used on this device
    p = it->second;
  }
  char *err = static_cast<char *>(p) + kNoAllocErrOffset;
  BCX_CUDA(cudaMemcpy(word, err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (*word) BCX_CUDA(cudaMemset(err, 0, sizeof(uint32_t)));
  return BCX_SUCCESS;
}

}  // namespace bcx

extern "C" bcx_status bcx_scan_noalloc(bcx_stream stream, bcx_dtype type, bcx_op op, int exclusive,
                                       const void *init, const void *in, void *out, size_t n,
                                       int compensated) {
  using namespace bcx;
  clear_error();
  BCX_CHECK(dtype_valid(type), BCX_INVALID_VALUE, "invalid dtype %d", int(type));
  if (n == 0) return BCX_SUCCESS;
  BCX_CHECK(in != nullptr && out != nullptr, BCX_INVALID_VALUE, "NULL input or output");
  unsigned char zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const void *init_p = (exclusive && init) ? init : zero;
  cudaStream_t s = (cudaStream_t)stream;
  bcx_status rc = BCX_UNSUPPORTED;
  switch (type) {
    case BCX_CHAR: rc = noalloc_int<int8_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_UCHAR: rc = noalloc_int<uint8_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_SHORT: rc = noalloc_int<int16_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_USHORT: rc = noalloc_int<uint16_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_INT: rc = noalloc_int<int32_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_UINT: rc = noalloc_int<uint32_t>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_LONG: rc = noalloc_int<long long>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_ULONG: rc = noalloc_int<unsigned long long>(s, op, exclusive, init_p, in, out, n); break;
    case BCX_FLOAT: rc = noalloc_float<float>(s, op, exclusive, init_p, in, out, n, compensated); break;
    case BCX_DOUBLE: rc = noalloc_float<double>(s, op, exclusive, init_p, in, out, n, compensated); break;
  }
  if (rc == BCX_UNSUPPORTED) set_error("scan: functor %d not provided for dtype %d", int(op), int(type));
  return rc;
}
