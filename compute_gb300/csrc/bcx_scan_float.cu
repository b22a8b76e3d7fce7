// bcx_scan_float.cu -- the allocating scan for float and double, plain and
// compensated (the kernels and their design are in bcx_scan.cuh).
#include "bcx_scan.cuh"

namespace bcx {

bcx_status scan_floats(cudaStream_t s, bcx_dtype type, int op, int ex, const void *init, const void *in,
                       void *out, size_t n, int comp, void *temp, size_t *tb) {
  switch (type) {
    case BCX_FLOAT: return dispatch_float<float>(s, op, ex, init, in, out, n, comp, temp, tb);
    case BCX_DOUBLE: return dispatch_float<double>(s, op, ex, init, in, out, n, comp, temp, tb);
    default: return BCX_UNSUPPORTED;
  }
}

}  // namespace bcx
