// bcx_debug.cu -- test hook for failure detection: runs each kind of bounded
// device-side wait the library's kernels use (the onesweep digit look-back,
// the scan tile look-back, the bulk-copy mbarrier wait) against a status word
// or barrier that nothing ever publishes, with a small poll limit, so a test
// can check that the wait gives up, the kernel returns, and
// bcx_device_error_check reports BCX_DEVICE_TIMEOUT with the context intact.
// Nothing here faults, traps or waits without a bound.
#include <cuda_runtime.h>

#include "bcx.h"
#include "bcx_internal.h"
#include "bcx_radix.cuh"
#include "bcx_scan.cuh"

namespace bcx {
namespace {

// Tile 1 of a sort looks back at tile 0, whose status words stay zero.
__global__ void expire_onesweep_wait(const unsigned long long *status, uint32_t limit, uint32_t *err) {
  bool gave_up = false;
  (void)radix::onesweep_lookback<>(status, 1u, 0u, threadIdx.x, radix::tag_aggregate(0), &gave_up, limit);
  if (gave_up) report_error(err, kErrLookbackTimeout);
}

// Warp 0 of scan tile 1 looks back at tile 0, whose status word stays zero.
__global__ void expire_scan_wait(unsigned long long *words, uint32_t limit, uint32_t *err) {
  typedef ScanPlain<int32_t, op_plus> P;
  TileStatus<typename P::Carry> st;
  st.words = words;
  if (threadIdx.x < kWarp) (void)lookback<P>(st, 1, typename P::Carry(5), err, limit);
}

// A block waits for phase 0 of an mbarrier that nothing arrives on.
__global__ void expire_copy_wait(uint32_t limit, uint32_t *err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, limit)) report_error(err, kErrCopyTimeout);
}

}  // namespace
}  // namespace bcx

using namespace bcx;

extern "C" bcx_status bcx_debug_expire_wait(bcx_stream stream, int which, unsigned polls) {
  clear_error();
  BCX_CHECK(which >= 0 && which <= 2, BCX_INVALID_VALUE, "which must be 0, 1 or 2 (got %d)", which);
  BCX_CHECK(polls >= 1 && polls <= (1u << 20), BCX_INVALID_VALUE, "polls must be in [1, 2^20]");
  DeviceState *ds = nullptr;
  bcx_status rc = current_device_state(&ds);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = size_t(2) * radix::kRadix * sizeof(unsigned long long);
  void *status = nullptr;
  BCX_CUDA(cudaMallocAsync(&status, bytes, s));
  BCX_CUDA(cudaMemsetAsync(status, 0, bytes, s));
  auto *words = static_cast<unsigned long long *>(status);
  if (which == 0) expire_onesweep_wait<<<1, radix::kRadix, 0, s>>>(words, polls, ds->err_word);
  else if (which == 1) expire_scan_wait<<<1, kWarp, 0, s>>>(words, polls, ds->err_word);
  else expire_copy_wait<<<1, kWarp, 0, s>>>(polls, ds->err_word);
  rc = launch_status("bcx_debug_expire_wait");
  cudaFreeAsync(status, s);
  return rc;
}
