// boost/compute/lambda.hpp -- placeholder expressions (_1, _2, _3).
//
// Reference: lambda/ (Boost.Proto) turns expressions such as alpha * _1 + _2
// into OpenCL C text (lambda/context.hpp:60-240).  Here a small expression
// template does the same for CUDA C++: every node knows how to print itself,
// host values are printed as exact literals (float bits, not decimal text),
// and the algorithms hand the text to the generated-kernel path
// (detail/jit.hpp).
#ifndef BOOST_COMPUTE_LAMBDA_HPP
#define BOOST_COMPUTE_LAMBDA_HPP

#include <cstddef>
#include <string>
#include <type_traits>

#include <boost/compute/detail/jit.hpp>

namespace boost {
namespace compute {
namespace lambda {

// Base of every lambda node: print(args) returns the CUDA expression.
template <class Derived>
struct expr_base {
  const Derived &self() const { return static_cast<const Derived &>(*this); }
};

template <int N>
struct placeholder : expr_base<placeholder<N> > {
  std::string print() const { return "_" + std::to_string(N + 1); }
  std::string defs() const { return ""; }
};

template <class T>
struct value_node : expr_base<value_node<T> > {
  T v;
  explicit value_node(T x) : v(x) {}
  std::string print() const { return detail::literal(v); }
  std::string defs() const { return ""; }
};

template <class L, class R>
struct binary_node : expr_base<binary_node<L, R> > {
  L l;
  R r;
  const char *op;
  binary_node(const L &a, const R &b, const char *o) : l(a), r(b), op(o) {}
  std::string print() const { return "(" + l.print() + " " + op + " " + r.print() + ")"; }
  std::string defs() const { return l.defs() + r.defs(); }
};

template <class A>
struct unary_node : expr_base<unary_node<A> > {
  A a;
  const char *op;
  unary_node(const A &x, const char *o) : a(x), op(o) {}
  std::string print() const { return std::string("(") + op + a.print() + ")"; }
  std::string defs() const { return a.defs(); }
};

template <class... A>
struct call_node;
template <class A>
struct call_node<A> : expr_base<call_node<A> > {
  const char *fn;
  A a;
  call_node(const char *f, const A &x) : fn(f), a(x) {}
  std::string print() const { return std::string(fn) + "(" + a.print() + ")"; }
  std::string defs() const { return a.defs(); }
};
template <class A, class B>
struct call_node<A, B> : expr_base<call_node<A, B> > {
  const char *fn;
  A a;
  B b;
  call_node(const char *f, const A &x, const B &y) : fn(f), a(x), b(y) {}
  std::string print() const { return std::string(fn) + "(" + a.print() + ", " + b.print() + ")"; }
  std::string defs() const { return a.defs() + b.defs(); }
};
template <class A, class B, class C>
struct call_node<A, B, C> : expr_base<call_node<A, B, C> > {
  const char *fn;
  A a;
  B b;
  C c;
  call_node(const char *f, const A &x, const B &y, const C &z) : fn(f), a(x), b(y), c(z) {}
  std::string print() const { return std::string(fn) + "(" + a.print() + ", " + b.print() + ", " + c.print() + ")"; }
  std::string defs() const { return a.defs() + b.defs() + c.defs(); }
};

template <class T> struct is_node : std::is_base_of<expr_base<T>, T> {};

// Wrap host values as literal nodes, leave nodes alone.
template <class T, bool = is_node<T>::value>
struct as_node {
  typedef T type;
  static const T &wrap(const T &t) { return t; }
};
template <class T>
struct as_node<T, false> {
  typedef value_node<T> type;
  static value_node<T> wrap(const T &t) { return value_node<T>(t); }
};

#define BOOST_COMPUTE_LAMBDA_BINARY(OP, TEXT)                                                          \
  template <class L, class R, class = typename std::enable_if<is_node<L>::value || is_node<R>::value>::type> \
  binary_node<typename as_node<L>::type, typename as_node<R>::type> operator OP(const L &l, const R &r) { \
    return binary_node<typename as_node<L>::type, typename as_node<R>::type>(as_node<L>::wrap(l),        \
                                                                             as_node<R>::wrap(r), TEXT); \
  }
BOOST_COMPUTE_LAMBDA_BINARY(+, "+")
BOOST_COMPUTE_LAMBDA_BINARY(-, "-")
BOOST_COMPUTE_LAMBDA_BINARY(*, "*")
BOOST_COMPUTE_LAMBDA_BINARY(/, "/")
BOOST_COMPUTE_LAMBDA_BINARY(%, "%")
BOOST_COMPUTE_LAMBDA_BINARY(<, "<")
BOOST_COMPUTE_LAMBDA_BINARY(>, ">")
BOOST_COMPUTE_LAMBDA_BINARY(<=, "<=")
BOOST_COMPUTE_LAMBDA_BINARY(>=, ">=")
BOOST_COMPUTE_LAMBDA_BINARY(==, "==")
BOOST_COMPUTE_LAMBDA_BINARY(!=, "!=")
BOOST_COMPUTE_LAMBDA_BINARY(&&, "&&")
BOOST_COMPUTE_LAMBDA_BINARY(||, "||")
BOOST_COMPUTE_LAMBDA_BINARY(&, "&")
BOOST_COMPUTE_LAMBDA_BINARY(|, "|")
BOOST_COMPUTE_LAMBDA_BINARY(^, "^")
#undef BOOST_COMPUTE_LAMBDA_BINARY

template <class A, class = typename std::enable_if<is_node<A>::value>::type>
unary_node<A> operator-(const A &a) { return unary_node<A>(a, "-"); }
template <class A, class = typename std::enable_if<is_node<A>::value>::type>
unary_node<A> operator!(const A &a) { return unary_node<A>(a, "!"); }

// get<N>(expr): element N of a tuple, component N of a vector type
// (lambda/get.hpp of the reference).
template <std::size_t N, class A>
struct get_node : expr_base<get_node<N, A> > {
  A a;
  explicit get_node(const A &a_) : a(a_) {}
  std::string print() const { return "bcx_get<" + std::to_string(N) + ">(" + a.print() + ")"; }
  std::string defs() const { return a.defs(); }
};
template <std::size_t N, class A, class = typename std::enable_if<is_node<A>::value>::type>
get_node<N, A> get(const A &a) {
  return get_node<N, A>(a);
}

#define BOOST_COMPUTE_LAMBDA_FN1(NAME, TEXT)                                    \
  template <class A, class = typename std::enable_if<is_node<A>::value>::type>  \
  call_node<A> NAME(const A &a) { return call_node<A>(TEXT, a); }
BOOST_COMPUTE_LAMBDA_FN1(sqrt, "sqrt")
BOOST_COMPUTE_LAMBDA_FN1(fabs, "fabs")
BOOST_COMPUTE_LAMBDA_FN1(abs, "abs")
BOOST_COMPUTE_LAMBDA_FN1(exp, "exp")
BOOST_COMPUTE_LAMBDA_FN1(log, "log")
BOOST_COMPUTE_LAMBDA_FN1(sin, "sin")
BOOST_COMPUTE_LAMBDA_FN1(cos, "cos")
BOOST_COMPUTE_LAMBDA_FN1(floor, "floor")
BOOST_COMPUTE_LAMBDA_FN1(ceil, "ceil")
BOOST_COMPUTE_LAMBDA_FN1(popcount, "popcount")
#undef BOOST_COMPUTE_LAMBDA_FN1

#define BOOST_COMPUTE_LAMBDA_FN2(NAME, TEXT)                                                             \
  template <class A, class B, class = typename std::enable_if<is_node<A>::value || is_node<B>::value>::type> \
  call_node<typename as_node<A>::type, typename as_node<B>::type> NAME(const A &a, const B &b) {          \
    return call_node<typename as_node<A>::type, typename as_node<B>::type>(TEXT, as_node<A>::wrap(a),     \
                                                                           as_node<B>::wrap(b));        \
  }
BOOST_COMPUTE_LAMBDA_FN2(pown, "pown")
BOOST_COMPUTE_LAMBDA_FN2(pow, "pow")
BOOST_COMPUTE_LAMBDA_FN2(min, "min")
BOOST_COMPUTE_LAMBDA_FN2(max, "max")
#undef BOOST_COMPUTE_LAMBDA_FN2

template <class A, class B, class C,
          class = typename std::enable_if<is_node<A>::value || is_node<B>::value || is_node<C>::value>::type>
call_node<typename as_node<A>::type, typename as_node<B>::type, typename as_node<C>::type>
clamp(const A &a, const B &b, const C &c) {
  return call_node<typename as_node<A>::type, typename as_node<B>::type, typename as_node<C>::type>(
      "clamp", as_node<A>::wrap(a), as_node<B>::wrap(b), as_node<C>::wrap(c));
}
template <class A, class B, class C,
          class = typename std::enable_if<is_node<A>::value || is_node<B>::value || is_node<C>::value>::type>
call_node<typename as_node<A>::type, typename as_node<B>::type, typename as_node<C>::type>
fma(const A &a, const B &b, const C &c) {
  return call_node<typename as_node<A>::type, typename as_node<B>::type, typename as_node<C>::type>(
      "fma", as_node<A>::wrap(a), as_node<B>::wrap(b), as_node<C>::wrap(c));
}

static const placeholder<0> _1 = placeholder<0>();
static const placeholder<1> _2 = placeholder<1>();
static const placeholder<2> _3 = placeholder<2>();

}  // namespace lambda

using lambda::_1;
using lambda::_2;
using lambda::_3;

}  // namespace compute
}  // namespace boost

#endif
