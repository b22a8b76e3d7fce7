// bcx_scan_small.cu -- the allocating scan for 1- and 2-byte integers (the
// kernels and their design are in bcx_scan.cuh).
#include "bcx_scan.cuh"

namespace bcx {

bcx_status scan_small_ints(cudaStream_t s, bcx_dtype type, int op, int ex, const void *init, const void *in,
                           void *out, size_t n, void *temp, size_t *tb) {
  switch (type) {
    case BCX_CHAR: return dispatch_int<int8_t>(s, op, ex, init, in, out, n, temp, tb);
    case BCX_UCHAR: return dispatch_int<uint8_t>(s, op, ex, init, in, out, n, temp, tb);
    case BCX_SHORT: return dispatch_int<int16_t>(s, op, ex, init, in, out, n, temp, tb);
    case BCX_USHORT: return dispatch_int<uint16_t>(s, op, ex, init, in, out, n, temp, tb);
    default: return BCX_UNSUPPORTED;
  }
}

}  // namespace bcx
