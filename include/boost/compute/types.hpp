// boost/compute/types.hpp -- scalar and vector element types of the drop-in
// layer (the reference's types/fundamental.hpp: char_ ... double_, int2_,
// float4_ ...), and their mapping to bcx_dtype.
#ifndef BOOST_COMPUTE_TYPES_HPP
#define BOOST_COMPUTE_TYPES_HPP

#include <cstdint>
#include <ostream>

#include <bcx.h>

namespace boost {
namespace compute {

typedef int8_t char_;
typedef uint8_t uchar_;
typedef int16_t short_;
typedef uint16_t ushort_;
typedef int32_t int_;
typedef uint32_t uint_;
typedef int64_t long_;
typedef uint64_t ulong_;
typedef float float_;
typedef double double_;

// Fixed-size vector types, laid out like the OpenCL/CUDA vector types.
template <class T, int N>
struct vector_type {
  T s[N];
  vector_type() : s() {}
  explicit vector_type(T v) {
    for (int i = 0; i < N; ++i) s[i] = v;
  }
  vector_type(T a, T b) : s{a, b} { static_assert(N == 2, "two components"); }
  vector_type(T a, T b, T c, T d) : s{a, b, c, d} { static_assert(N == 4, "four components"); }
  T &operator[](int i) { return s[i]; }
  const T &operator[](int i) const { return s[i]; }
  bool operator==(const vector_type &o) const {
    for (int i = 0; i < N; ++i)
      if (!(s[i] == o.s[i])) return false;
    return true;
  }
  bool operator!=(const vector_type &o) const { return !(*this == o); }
};
template <class T, int N>
std::ostream &operator<<(std::ostream &os, const vector_type<T, N> &v) {
  os << "(";
  for (int i = 0; i < N; ++i) os << (i ? ", " : "") << v.s[i];
  return os << ")";
}
typedef vector_type<int_, 2> int2_;
typedef vector_type<int_, 4> int4_;
typedef vector_type<uint_, 2> uint2_;
typedef vector_type<float_, 2> float2_;
typedef vector_type<float_, 4> float4_;

namespace detail {
template <class T> struct bcx_type_of { static const int value = -1; };
#define BOOST_COMPUTE_BCX_TYPE(T, V) template <> struct bcx_type_of<T> { static const int value = V; };
BOOST_COMPUTE_BCX_TYPE(char_, BCX_CHAR)
BOOST_COMPUTE_BCX_TYPE(char, BCX_CHAR)
BOOST_COMPUTE_BCX_TYPE(uchar_, BCX_UCHAR)
BOOST_COMPUTE_BCX_TYPE(short_, BCX_SHORT)
BOOST_COMPUTE_BCX_TYPE(ushort_, BCX_USHORT)
BOOST_COMPUTE_BCX_TYPE(int_, BCX_INT)
BOOST_COMPUTE_BCX_TYPE(uint_, BCX_UINT)
BOOST_COMPUTE_BCX_TYPE(long_, BCX_LONG)
BOOST_COMPUTE_BCX_TYPE(ulong_, BCX_ULONG)
BOOST_COMPUTE_BCX_TYPE(float_, BCX_FLOAT)
BOOST_COMPUTE_BCX_TYPE(double_, BCX_DOUBLE)
#undef BOOST_COMPUTE_BCX_TYPE

// CUDA C++ spelling of an element type, for generated kernel source.
template <class T> struct cuda_type_name;
#define BOOST_COMPUTE_TYPE_NAME(T, S) template <> struct cuda_type_name<T> { static const char *get() { return S; } };
BOOST_COMPUTE_TYPE_NAME(char_, "signed char")
BOOST_COMPUTE_TYPE_NAME(char, "char")
BOOST_COMPUTE_TYPE_NAME(uchar_, "unsigned char")
BOOST_COMPUTE_TYPE_NAME(short_, "short")
BOOST_COMPUTE_TYPE_NAME(ushort_, "unsigned short")
BOOST_COMPUTE_TYPE_NAME(int_, "int")
BOOST_COMPUTE_TYPE_NAME(uint_, "unsigned int")
BOOST_COMPUTE_TYPE_NAME(long_, "long long")
BOOST_COMPUTE_TYPE_NAME(ulong_, "unsigned long long")
BOOST_COMPUTE_TYPE_NAME(float_, "float")
BOOST_COMPUTE_TYPE_NAME(double_, "double")
BOOST_COMPUTE_TYPE_NAME(int2_, "int2")
BOOST_COMPUTE_TYPE_NAME(int4_, "int4")
BOOST_COMPUTE_TYPE_NAME(uint2_, "uint2")
BOOST_COMPUTE_TYPE_NAME(float2_, "float2")
BOOST_COMPUTE_TYPE_NAME(float4_, "float4")
#undef BOOST_COMPUTE_TYPE_NAME
}  // namespace detail

}  // namespace compute
}  // namespace boost

#endif
