// Prints the CUDA source the drop-in headers generate for user functors
// (fold and scan kernels) for a few element types, each preceded by a
// "//@@ <kernel name>" line, so a test can compile every one with NVRTC
// without a GPU.
#include <cstdio>
#include <string>

#include <boost/compute/detail/jit.hpp>
#include <boost/compute/function.hpp>
#include <boost/compute/lambda.hpp>
#include <boost/compute/iterator/zip_iterator.hpp>
#include <boost/compute/types/tuple.hpp>

using namespace boost::compute::detail;

static void emit(const char *name, const std::string &src) {
  std::printf("//@@ %s\n%s\n", name, src.c_str());
}

int main() {
  // plain scalar functors
  emit("bcx_jit_scan", jit_scan_source("", "_1 + _2", "int", 4));
  emit("bcx_jit_scan", jit_scan_source("", "_1 * _2", "long long", 8));
  emit("bcx_jit_scan", jit_scan_source("", "max(_1, _2)", "float", 4));
  emit("bcx_jit_scan", jit_scan_source("", "_1 + _2", "double", 8));
  emit("bcx_jit_scan", jit_scan_source("", "(unsigned char)(_1 ^ _2)", "unsigned char", 1));
  // a user function and a 16-byte struct (non-commutative: keeps the later)
  emit("bcx_jit_scan", jit_scan_source("__device__ int add_four(int a, int b) { return a + b + 4; }\n",
                                       "add_four(_1, _2)", "int", 4));
  emit("bcx_jit_scan", jit_scan_source("struct P { float x; float y; int z; int w; };\n",
                                       "P{_1.x + _2.x, _2.y, _1.z + _2.z, _2.w}", "P", 16));
  // the staged scan (bulk-copied tiles) for every element size that divides 16
  auto staged = [](const std::string &defs, const char *op, const char *t, size_t ts) {
    emit("bcx_jit_scan_staged", jit_scan_source(defs, op, t, ts, 0, true, -1, -1, 1, -1,
                                                jit_scan_staged_tile_bytes(ts)));
  };
  staged("", "_1 + _2", "int", 4);
  staged("", "_1 * _2", "long long", 8);
  staged("", "max(_1, _2)", "float", 4);
  staged("", "_1 + _2", "double", 8);
  staged("", "(unsigned char)(_1 ^ _2)", "unsigned char", 1);
  staged("", "(short)(_1 + _2)", "short", 2);
  staged("struct P { float x; float y; int z; int w; };\n", "P{_1.x + _2.x, _2.y, _1.z + _2.z, _2.w}", "P", 16);
  emit("bcx_jit_fold", jit_fold_source("", "_1 + _2", "int", 4, "return a[i];", "int", nullptr));
  emit("bcx_jit_fold", jit_fold_source("", "_1 + _2", "float", 4, "return a[i] * b[i];", "float", "float"));
  emit("bcx_jit_fold", jit_fold_source("struct BcxArg { float v; unsigned long long i; };\n",
                                       "_2.v < _1.v ? _2 : _1", "BcxArg", 16,
                                       "BcxArg r; r.v = a[i]; r.i = i; return r;", "float", nullptr));
  emit("bcx_jit_fold", jit_fold_source("", "_1 + _2", "unsigned long long", 8,
                                       "const auto _1 = a[i]; return (T)((_1 > 3) ? 1ull : 0ull);", "int",
                                       nullptr));
  // zipped ranges: the gather kernel, a transform of the tuple through get<N>
  // and through a user function taking the tuple, count_if on a tuple field
  typedef std::tuple<char, int, float> T3;
  emit("bcx_jit_zip_gather", zip_gather_source<char, int, float>());
  emit("bcx_jit_transform", jit_transform_source(type_definition<T3>::get(), "bcx_get<1>(_1)", cuda_type_name<T3>::get(),
                                                 "", "int", sizeof(T3), 0, 4, false));
  typedef std::tuple<float, float, float> F3;
  emit("bcx_jit_transform",
       jit_transform_source(type_definition<F3>::get() +
                                "__device__ __forceinline__ float fma3(std::tuple<float, float, float> t) "
                                "{ return boost_tuple_get(t, 0) * boost_tuple_get(t, 1) + boost_tuple_get(t, 2); }\n",
                            "fma3(_1)", cuda_type_name<F3>::get(), "", "float", sizeof(F3), 0, 4, false));
  typedef std::tuple<int, int> I2;
  emit("bcx_jit_fold", jit_fold_source(type_definition<I2>::get(), "_1 + _2", "unsigned long long", 8,
                                       "const auto _1 = a[i]; return (T)((bcx_get<0>(_1) < 5) ? 1ull : 0ull);",
                                       cuda_type_name<I2>::get(), nullptr));
  // get<N> on a vector type; accumulate with an init of another type
  emit("bcx_jit_transform", jit_transform_source("", "bcx_get<2>(_1)", "float4", "", "float", 16, 0, 4, false));
  emit("bcx_jit_serial_fold", jit_serial_fold_source("", "(_1 + _2)", "int", "float"));
  emit("bcx_jit_serial_fold", jit_serial_fold_source("", "(_2 < _1 ? _2 : _1)", "long long", "unsigned char"));
  // user functions written the way callers write them, through the drop-in
  // macro: a qualified vector type in the signature, a non-commutative body
  namespace compute = boost::compute;
  BOOST_COMPUTE_FUNCTION(compute::int4_, matmul, (compute::int4_ a, compute::int4_ b), {
    const unsigned a0 = a.x, a1 = a.y, a2 = a.z, a3 = a.w, b0 = b.x, b1 = b.y, b2 = b.z, b3 = b.w;
    return make_int4((int)(a0 * b0 + a1 * b2), (int)(a0 * b1 + a1 * b3), (int)(a2 * b0 + a3 * b2),
                     (int)(a2 * b1 + a3 * b3));
  });
  emit("bcx_jit_scan", jit_scan_source(matmul.defs(), matmul.print(), "int4", 16));
  staged(matmul.defs(), matmul.print().c_str(), "int4", 16);
  emit("bcx_jit_fold", jit_fold_source(matmul.defs(), matmul.print(), "int4", 16, "return a[i];", "int4", nullptr));
  BOOST_COMPUTE_FUNCTION(int, times, (int x, int y), { return x * y; });
  emit("bcx_jit_scan", jit_scan_source(times.defs(), times.print(), "int", 4));
  staged(times.defs(), times.print().c_str(), "int", 4);
  using compute::_1;
  using compute::_2;
  const float alpha = 2.5f;
  auto saxpy = alpha * _1 + _2;
  emit("bcx_jit_transform", jit_transform_source(saxpy.defs(), saxpy.print(), "float", "float", "float", 4, 4, 4, true));
  return 0;
}
