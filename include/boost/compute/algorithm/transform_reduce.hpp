// boost/compute/algorithm/transform_reduce.hpp
//
// Reference: transform_reduce(first, last, result, f, op) reduces a
// transform_iterator (transform_reduce.hpp:39-60); the binary form zips two
// inputs and unpacks them into f (:62-95).  Here both forms are ONE generated
// reduce kernel whose element read applies f, so the transformed values are
// never written to memory.  f and op may be built-in functors, lambda
// expressions or BOOST_COMPUTE_FUNCTIONs; op must be associative (it may be
// non-commutative: elements are folded in index order).  An empty range writes
// nothing, as reduce() does.
#ifndef BOOST_COMPUTE_ALGORITHM_TRANSFORM_REDUCE_HPP
#define BOOST_COMPUTE_ALGORITHM_TRANSFORM_REDUCE_HPP

#include <iterator>
#include <string>
#include <type_traits>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/detail/jit.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>

namespace boost {
namespace compute {
namespace detail {

// Kernel-side spelling of a functor applied to _1 (and _2), with any
// definitions it needs.
template <class G>
inline typename std::enable_if<is_jit_functor<G>::value>::type functor_expr(const G &g, std::string *d,
                                                                             std::string *e) {
  *d = g.defs();
  *e = g.print();
}
template <class G>
inline typename std::enable_if<!is_jit_functor<G>::value &&
                               (is_builtin_binary<G>::value || is_builtin_compare<G>::value)>::type
functor_expr(const G &, std::string *d, std::string *e) {
  const std::string s = G::source();  // spelled with a and b
  d->clear();
  e->clear();
  for (char c : s) {
    if (c == 'a') *e += "_1";
    else if (c == 'b') *e += "_2";
    else *e += c;
  }
}
template <class G>
inline typename std::enable_if<!is_jit_functor<G>::value && !is_builtin_binary<G>::value &&
                               !is_builtin_compare<G>::value>::type
functor_expr(const G &, std::string *d, std::string *e) {
  d->clear();
  *e = builtin_unary_expr<G>();
}

// out = [init op] fold(op, f(a[i] [, b[i]])), one generated kernel.
template <class T, class A, class B, class F, class Op>
inline void fused_transform_reduce(const A *a, const B *b, size_t n, F f, Op op, T *out, command_queue &queue,
                                   const T *init = nullptr) {
  std::string fd, fe, od, oe;
  functor_expr(f, &fd, &fe);
  functor_expr(op, &od, &oe);
  std::string load = "const auto _1 = a[i]; ";
  if (b) load += "const auto _2 = b[i]; ";
  load += "return (T)(" + fe + ");";
  jit_fold(fd + "\n" + od, oe, cuda_type_name<T>::get(), sizeof(T), load, cuda_type_name<A>::get(),
           b ? cuda_type_name<B>::get() : nullptr, a, b, n, init, out, queue);
}

}  // namespace detail

template <class InputIterator, class T, class UnaryTransformFunction, class BinaryReduceFunction>
inline void transform_reduce(InputIterator first, InputIterator last, buffer_iterator<T> result,
                             UnaryTransformFunction transform_function, BinaryReduceFunction reduce_function,
                             command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type A;
  if (first == last) return;
  detail::device_range<InputIterator> in(first, last, queue);
  detail::fused_transform_reduce<T, A, A>(in.ptr, static_cast<const A *>(nullptr), in.n, transform_function,
                                          reduce_function, result.get_ptr(), queue);
  if (!std::is_same<InputIterator, buffer_iterator<A> >::value) queue.finish();  // keep the temporary alive
}

template <class InputIterator, class T, class UnaryTransformFunction, class BinaryReduceFunction>
inline void transform_reduce(InputIterator first, InputIterator last, T *result,
                             UnaryTransformFunction transform_function, BinaryReduceFunction reduce_function,
                             command_queue &queue = system::default_queue()) {
  if (first == last) return;
  vector<T> tmp(1, queue.get_context());
  ::boost::compute::transform_reduce(first, last, tmp.begin(), transform_function, reduce_function, queue);
  *result = tmp.begin().read(queue);
}

template <class InputIterator1, class InputIterator2, class T, class BinaryTransformFunction,
          class BinaryReduceFunction>
inline void transform_reduce(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2,
                             buffer_iterator<T> result, BinaryTransformFunction transform_function,
                             BinaryReduceFunction reduce_function, command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator1>::value_type A;
  typedef typename std::iterator_traits<InputIterator2>::value_type B;
  if (first1 == last1) return;
  detail::device_range<InputIterator1> a(first1, last1, queue);
  detail::device_range<InputIterator2> b(first2, first2 + std::ptrdiff_t(a.n), queue);
  detail::fused_transform_reduce<T, A, B>(a.ptr, b.ptr, a.n, transform_function, reduce_function, result.get_ptr(),
                                          queue);
  if (!std::is_same<InputIterator1, buffer_iterator<A> >::value ||
      !std::is_same<InputIterator2, buffer_iterator<B> >::value)
    queue.finish();  // keep the temporaries alive
}

template <class InputIterator1, class InputIterator2, class T, class BinaryTransformFunction,
          class BinaryReduceFunction>
inline void transform_reduce(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2, T *result,
                             BinaryTransformFunction transform_function, BinaryReduceFunction reduce_function,
                             command_queue &queue = system::default_queue()) {
  if (first1 == last1) return;
  vector<T> tmp(1, queue.get_context());
  ::boost::compute::transform_reduce(first1, last1, first2, tmp.begin(), transform_function, reduce_function,
                                     queue);
  *result = tmp.begin().read(queue);
}

}  // namespace compute
}  // namespace boost

#endif
