// boost/compute/functional.hpp -- built-in function objects
// (the reference's functional/operator.hpp:57-92, functional/integer.hpp,
// functional/math.hpp).  Each carries the bcx functor id the algorithms pass
// to libbcx, the host evaluation used by host-side fallbacks of tiny helper
// algorithms, and its CUDA spelling for generated kernels.
#ifndef BOOST_COMPUTE_FUNCTIONAL_HPP
#define BOOST_COMPUTE_FUNCTIONAL_HPP

#include <cmath>

#include <bcx.h>

namespace boost {
namespace compute {

#define BOOST_COMPUTE_BINARY_FUNCTOR(NAME, OPID, EXPR, SRC)                     \
  template <class T>                                                            \
  struct NAME {                                                                 \
    typedef T result_type;                                                      \
    static const int bcx_op = OPID;                                             \
    T operator()(const T &a, const T &b) const { return EXPR; }                 \
    static const char *source() { return SRC; }                                 \
  };
BOOST_COMPUTE_BINARY_FUNCTOR(plus, BCX_PLUS, T(a + b), "(a + b)")
BOOST_COMPUTE_BINARY_FUNCTOR(minus, BCX_MINUS, T(a - b), "(a - b)")
BOOST_COMPUTE_BINARY_FUNCTOR(multiplies, BCX_MULTIPLIES, T(a * b), "(a * b)")
BOOST_COMPUTE_BINARY_FUNCTOR(divides, BCX_DIVIDES, T(a / b), "(a / b)")
BOOST_COMPUTE_BINARY_FUNCTOR(modulus, BCX_MODULUS, T(a % b), "(a % b)")
BOOST_COMPUTE_BINARY_FUNCTOR(min, BCX_MIN, (b < a ? b : a), "(b < a ? b : a)")
BOOST_COMPUTE_BINARY_FUNCTOR(max, BCX_MAX, (b > a ? b : a), "(b > a ? b : a)")
BOOST_COMPUTE_BINARY_FUNCTOR(bit_and, BCX_BIT_AND, T(a & b), "(a & b)")
BOOST_COMPUTE_BINARY_FUNCTOR(bit_or, BCX_BIT_OR, T(a | b), "(a | b)")
BOOST_COMPUTE_BINARY_FUNCTOR(bit_xor, BCX_BIT_XOR, T(a ^ b), "(a ^ b)")
#undef BOOST_COMPUTE_BINARY_FUNCTOR

#define BOOST_COMPUTE_COMPARE_FUNCTOR(NAME, EXPR, SRC)                          \
  template <class T>                                                            \
  struct NAME {                                                                 \
    typedef bool result_type;                                                   \
    bool operator()(const T &a, const T &b) const { return EXPR; }              \
    static const char *source() { return SRC; }                                 \
  };
BOOST_COMPUTE_COMPARE_FUNCTOR(less, a < b, "(a < b)")
BOOST_COMPUTE_COMPARE_FUNCTOR(greater, a > b, "(a > b)")
BOOST_COMPUTE_COMPARE_FUNCTOR(equal_to, a == b, "(a == b)")
BOOST_COMPUTE_COMPARE_FUNCTOR(not_equal_to, a != b, "(a != b)")
BOOST_COMPUTE_COMPARE_FUNCTOR(less_equal, a <= b, "(a <= b)")
BOOST_COMPUTE_COMPARE_FUNCTOR(greater_equal, a >= b, "(a >= b)")
#undef BOOST_COMPUTE_COMPARE_FUNCTOR

#define BOOST_COMPUTE_UNARY_FUNCTOR(NAME, OPID, EXPR, SRC)                      \
  template <class T>                                                            \
  struct NAME {                                                                 \
    typedef T result_type;                                                      \
    static const int bcx_unary_op = OPID;                                       \
    T operator()(const T &x) const { return EXPR; }                             \
    static const char *source() { return SRC; }                                 \
  };
BOOST_COMPUTE_UNARY_FUNCTOR(identity, BCX_IDENTITY, x, "(x)")
BOOST_COMPUTE_UNARY_FUNCTOR(negate, BCX_NEGATE, T(-x), "(-x)")
BOOST_COMPUTE_UNARY_FUNCTOR(abs, BCX_ABS, (x < T(0) ? T(-x) : x), "(x < 0 ? -x : x)")
BOOST_COMPUTE_UNARY_FUNCTOR(sqrt, BCX_SQRT, T(std::sqrt(x)), "sqrt(x)")
BOOST_COMPUTE_UNARY_FUNCTOR(logical_not, BCX_LOGICAL_NOT, T(!x), "(!x)")
#undef BOOST_COMPUTE_UNARY_FUNCTOR

namespace detail {
template <class F> struct is_builtin_binary { static const bool value = false; };
#define BOOST_COMPUTE_IS_BUILTIN(F) template <class T> struct is_builtin_binary<F<T> > { static const bool value = true; };
BOOST_COMPUTE_IS_BUILTIN(plus)
BOOST_COMPUTE_IS_BUILTIN(minus)
BOOST_COMPUTE_IS_BUILTIN(multiplies)
BOOST_COMPUTE_IS_BUILTIN(divides)
BOOST_COMPUTE_IS_BUILTIN(modulus)
BOOST_COMPUTE_IS_BUILTIN(min)
BOOST_COMPUTE_IS_BUILTIN(max)
BOOST_COMPUTE_IS_BUILTIN(bit_and)
BOOST_COMPUTE_IS_BUILTIN(bit_or)
BOOST_COMPUTE_IS_BUILTIN(bit_xor)
#undef BOOST_COMPUTE_IS_BUILTIN
template <class F> struct is_builtin_unary { static const bool value = false; };
template <class T> struct is_builtin_unary<identity<T> > { static const bool value = true; };
template <class T> struct is_builtin_unary<negate<T> > { static const bool value = true; };
template <class T> struct is_builtin_unary<abs<T> > { static const bool value = true; };
template <class T> struct is_builtin_unary<sqrt<T> > { static const bool value = true; };
template <class T> struct is_builtin_unary<logical_not<T> > { static const bool value = true; };
// Comparisons, spelled with a and b like the binary functors.
template <class F> struct is_builtin_compare { static const bool value = false; };
template <class T> struct is_builtin_compare<less<T> > { static const bool value = true; };
template <class T> struct is_builtin_compare<greater<T> > { static const bool value = true; };
template <class T> struct is_builtin_compare<equal_to<T> > { static const bool value = true; };
template <class T> struct is_builtin_compare<not_equal_to<T> > { static const bool value = true; };
template <class T> struct is_builtin_compare<less_equal<T> > { static const bool value = true; };
template <class T> struct is_builtin_compare<greater_equal<T> > { static const bool value = true; };
}  // namespace detail

}  // namespace compute
}  // namespace boost

#endif
