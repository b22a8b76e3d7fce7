// bcx_scan_wide.cu -- the allocating scan for 8-byte integers (the kernels
// and their design are in bcx_scan.cuh).
#include "bcx_scan.cuh"

namespace bcx {

bcx_status scan_wide_ints(cudaStream_t s, bcx_dtype type, int op, int ex, const void *init, const void *in,
                          void *out, size_t n, void *temp, size_t *tb) {
  switch (type) {
    case BCX_LONG: return dispatch_int<long long>(s, op, ex, init, in, out, n, temp, tb);
    case BCX_ULONG: return dispatch_int<unsigned long long>(s, op, ex, init, in, out, n, temp, tb);
    default: return BCX_UNSUPPORTED;
  }
}

}  // namespace bcx
