// bcx_scan_word.cu -- the allocating scan for 4-byte integers (the kernels
// and their design are in bcx_scan.cuh).
#include "bcx_scan.cuh"

namespace bcx {

bcx_status scan_word_ints(cudaStream_t s, bcx_dtype type, int op, int ex, const void *init, const void *in,
                          void *out, size_t n, void *temp, size_t *tb) {
  switch (type) {
    case BCX_INT: return dispatch_int<int32_t>(s, op, ex, init, in, out, n, temp, tb);
    case BCX_UINT: return dispatch_int<uint32_t>(s, op, ex, init, in, out, n, temp, tb);
    default: return BCX_UNSUPPORTED;
  }
}

}  // namespace bcx
