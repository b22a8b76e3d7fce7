// boost/compute/algorithm/transform.hpp -- transform with built-in functors.
//
// Reference: transform(first, last, result, op) = copy of a
// transform_iterator; the binary form zips both inputs (transform.hpp:38-82).
// Built-in functors forward to bcx_transform_unary / bcx_transform_binary;
// lambda expressions and BOOST_COMPUTE_FUNCTION bodies go through the NVRTC
// path in boost/compute/lambda.hpp and boost/compute/function.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_TRANSFORM_HPP
#define BOOST_COMPUTE_ALGORITHM_TRANSFORM_HPP

#include <type_traits>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>
#include <boost/compute/types/tuple.hpp>

namespace boost {
namespace compute {

template <class InputIterator, class T, class UnaryFunction>
inline typename std::enable_if<detail::is_builtin_unary<UnaryFunction>::value, buffer_iterator<T> >::type
transform(InputIterator first, InputIterator last, buffer_iterator<T> result, UnaryFunction,
          command_queue &queue = system::default_queue()) {
  detail::device_range<InputIterator> in(first, last, queue);
  detail::check(bcx_transform_unary(queue.get(), bcx_dtype(detail::bcx_dtype_of<T>()),
                                    bcx_unary_op(UnaryFunction::bcx_unary_op), in.ptr, result.get_ptr(), in.n));
  if (!std::is_same<InputIterator, buffer_iterator<T> >::value) queue.finish();
  return result + std::ptrdiff_t(in.n);
}

template <class InputIterator1, class InputIterator2, class T, class BinaryFunction>
inline typename std::enable_if<detail::is_builtin_binary<BinaryFunction>::value, buffer_iterator<T> >::type
transform(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2, buffer_iterator<T> result,
          BinaryFunction, command_queue &queue = system::default_queue()) {
  detail::device_range<InputIterator1> a(first1, last1, queue);
  detail::device_range<InputIterator2> b(first2, first2 + std::ptrdiff_t(a.n), queue);
  detail::check(bcx_transform_binary(queue.get(), bcx_dtype(detail::bcx_dtype_of<T>()),
                                     bcx_op(BinaryFunction::bcx_op), a.ptr, b.ptr, result.get_ptr(), a.n));
  queue.finish();
  return result + std::ptrdiff_t(a.n);
}

// Lambda expressions and BOOST_COMPUTE_FUNCTIONs: one generated kernel.
template <class InputIterator, class T, class F>
inline typename std::enable_if<detail::is_jit_functor<F>::value, buffer_iterator<T> >::type
transform(InputIterator first, InputIterator last, buffer_iterator<T> result, F f,
          command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type A;
  detail::device_range<InputIterator> in(first, last, queue);
  detail::jit_transform(detail::type_definition<A>::get() + detail::type_definition<T>::get() + f.defs(), f.print(),
                        detail::cuda_type_name<A>::get(), "", detail::cuda_type_name<T>::get(), sizeof(A), 0,
                        sizeof(T), in.ptr, nullptr, result.get_ptr(), in.n, queue);
  if (!std::is_same<InputIterator, buffer_iterator<A> >::value) queue.finish();
  return result + std::ptrdiff_t(in.n);
}

template <class InputIterator1, class InputIterator2, class T, class F>
inline typename std::enable_if<detail::is_jit_functor<F>::value, buffer_iterator<T> >::type
transform(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2, buffer_iterator<T> result, F f,
          command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator1>::value_type A;
  typedef typename std::iterator_traits<InputIterator2>::value_type B;
  detail::device_range<InputIterator1> a(first1, last1, queue);
  detail::device_range<InputIterator2> b(first2, first2 + std::ptrdiff_t(a.n), queue);
  detail::jit_transform(detail::type_definition<A>::get() + detail::type_definition<B>::get() +
                            detail::type_definition<T>::get() + f.defs(),
                        f.print(), detail::cuda_type_name<A>::get(), detail::cuda_type_name<B>::get(),
                        detail::cuda_type_name<T>::get(), sizeof(A), sizeof(B), sizeof(T), a.ptr, b.ptr,
                        result.get_ptr(), a.n, queue);
  queue.finish();
  return result + std::ptrdiff_t(a.n);
}

}  // namespace compute
}  // namespace boost

#endif
