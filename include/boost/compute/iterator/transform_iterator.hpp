// boost/compute/iterator/transform_iterator.hpp -- f(*it) on the fly
// (the reference's iterator/transform_iterator.hpp:85-213).  Algorithms that
// read one evaluate it through one generated transform kernel into a
// temporary, then run their normal device path.
#ifndef BOOST_COMPUTE_ITERATOR_TRANSFORM_ITERATOR_HPP
#define BOOST_COMPUTE_ITERATOR_TRANSFORM_ITERATOR_HPP

#include <iterator>
#include <type_traits>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/function.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/lambda.hpp>

namespace boost {
namespace compute {
namespace detail {

template <class F, class A, class = void>
struct functor_result { typedef A type; };  // lambda expressions keep the input type
template <class F, class A>
struct functor_result<F, A, typename std::enable_if<!std::is_same<typename F::result_type, void>::value>::type> {
  typedef typename F::result_type type;
};

template <class F>
struct is_jit_functor {
  static const bool value = lambda::is_node<F>::value || is_user_function<F>::value;
};

// Kernel-side spelling of a unary built-in functor applied to _1.
template <class F>
inline std::string builtin_unary_expr() {
  std::string s = F::source();
  std::string out;
  for (char c : s) {
    if (c == 'x') out += "_1";
    else out += c;
  }
  return out;
}

}  // namespace detail

template <class InputIterator, class UnaryFunction>
class transform_iterator {
 public:
  typedef typename std::iterator_traits<InputIterator>::value_type input_type;
  typedef typename detail::functor_result<UnaryFunction, input_type>::type value_type;
  typedef std::random_access_iterator_tag iterator_category;
  typedef std::ptrdiff_t difference_type;
  typedef value_type *pointer;
  typedef value_type reference;
  transform_iterator(InputIterator it, UnaryFunction f) : m_it(it), m_f(f) {}
  InputIterator base() const { return m_it; }
  const UnaryFunction &functor() const { return m_f; }
  transform_iterator operator+(difference_type d) const { return transform_iterator(m_it + d, m_f); }
  difference_type operator-(const transform_iterator &o) const { return m_it - o.m_it; }
  bool operator==(const transform_iterator &o) const { return m_it == o.m_it; }
  bool operator!=(const transform_iterator &o) const { return m_it != o.m_it; }

 private:
  InputIterator m_it;
  UnaryFunction m_f;
};

template <class InputIterator, class UnaryFunction>
inline transform_iterator<InputIterator, UnaryFunction> make_transform_iterator(InputIterator it, UnaryFunction f) {
  return transform_iterator<InputIterator, UnaryFunction>(it, f);
}

namespace detail {

// A transform_iterator range as a device array: one generated kernel.
template <class InputIterator, class F>
struct device_range<transform_iterator<InputIterator, F> > {
  typedef transform_iterator<InputIterator, F> It;
  typedef typename It::input_type A;
  typedef typename It::value_type T;
  device_range(It first, It last, command_queue &queue) : base(first.base(), last.base(), queue) {
    n = base.n;
    tmp = vector<T>(n, queue.get_context());
    std::string defs, expr;
    expr_of(first.functor(), &defs, &expr);
    jit_transform(defs, expr, cuda_type_name<A>::get(), "", cuda_type_name<T>::get(), sizeof(A), 0, sizeof(T),
                  base.ptr, nullptr, tmp.data(), n, queue);
    queue.finish();
    ptr = tmp.data();
  }
  template <class G>
  static typename std::enable_if<is_jit_functor<G>::value>::type expr_of(const G &g, std::string *d, std::string *e) {
    *d = g.defs();
    *e = g.print();
  }
  template <class G>
  static typename std::enable_if<!is_jit_functor<G>::value>::type expr_of(const G &, std::string *d, std::string *e) {
    *d = "";
    *e = builtin_unary_expr<G>();
  }
  device_range<InputIterator> base;
  const T *ptr;
  size_t n;
  vector<T> tmp;
};

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
