// boost/compute/algorithm/exclusive_scan.hpp / inclusive_scan.hpp content.
//
// Reference: exclusive_scan.hpp:55-104, inclusive_scan.hpp:53-87 ->
// detail::scan_on_gpu (detail/scan_on_gpu.hpp:187-324).  Both forward to
// bcx_scan (single-pass decoupled look-back; in place allowed).  Float plus
// uses the compensated variant.
#ifndef BOOST_COMPUTE_ALGORITHM_SCAN_HPP
#define BOOST_COMPUTE_ALGORITHM_SCAN_HPP

#include <type_traits>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>

namespace boost {
namespace compute {
namespace detail {

template <class InputIterator, class T, class F>
inline typename std::enable_if<is_jit_functor<F>::value, buffer_iterator<T> >::type
scan(InputIterator first, InputIterator last, buffer_iterator<T> result, bool exclusive, T init, F f,
     command_queue &queue) {
  device_range<InputIterator> in(first, last, queue);
  jit_scan(f.defs(), f.print(), cuda_type_name<T>::get(), sizeof(T), in.ptr, result.get_ptr(), in.n, exclusive,
           &init, queue);
  if (!std::is_same<InputIterator, buffer_iterator<T> >::value) queue.finish();  // keep the temporary alive
  return result + std::ptrdiff_t(in.n);
}

template <class InputIterator, class T, class BinaryOperator>
inline typename std::enable_if<is_builtin_binary<BinaryOperator>::value, buffer_iterator<T> >::type
scan(InputIterator first, InputIterator last, buffer_iterator<T> result, bool exclusive, T init, BinaryOperator,
     command_queue &queue) {
  device_range<InputIterator> in(first, last, queue);
  const int comp = std::is_floating_point<T>::value && BinaryOperator::bcx_op == BCX_PLUS;
  detail::check(bcx_scan(queue.get(), bcx_dtype(bcx_dtype_of<T>()), bcx_op(BinaryOperator::bcx_op),
                         exclusive ? 1 : 0, &init, in.ptr, result.get_ptr(), in.n, comp, nullptr, nullptr));
  if (!std::is_same<InputIterator, buffer_iterator<T> >::value) queue.finish();  // keep the temporary alive
  return result + std::ptrdiff_t(in.n);
}

}  // namespace detail

template <class InputIterator, class T, class BinaryOperator>
inline buffer_iterator<T> exclusive_scan(InputIterator first, InputIterator last, buffer_iterator<T> result, T init,
                                         BinaryOperator op, command_queue &queue = system::default_queue()) {
  return detail::scan(first, last, result, true, init, op, queue);
}
template <class InputIterator, class T>
inline buffer_iterator<T> exclusive_scan(InputIterator first, InputIterator last, buffer_iterator<T> result, T init,
                                         command_queue &queue = system::default_queue()) {
  return detail::scan(first, last, result, true, init, plus<T>(), queue);
}
template <class InputIterator, class T>
inline buffer_iterator<T> exclusive_scan(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                         command_queue &queue = system::default_queue()) {
  return detail::scan(first, last, result, true, T(0), plus<T>(), queue);
}
template <class InputIterator, class T, class BinaryOperator>
inline buffer_iterator<T> inclusive_scan(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                         BinaryOperator op, command_queue &queue = system::default_queue()) {
  return detail::scan(first, last, result, false, T(0), op, queue);
}
template <class InputIterator, class T>
inline buffer_iterator<T> inclusive_scan(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                         command_queue &queue = system::default_queue()) {
  return detail::scan(first, last, result, false, T(0), plus<T>(), queue);
}

}  // namespace compute
}  // namespace boost

#endif
