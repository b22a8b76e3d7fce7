// boost/compute/algorithm/inner_product.hpp
//
// Reference: inner_product(first1, last1, first2, init [, op1, op2])
// (inner_product.hpp:33-110) reduces the products into a temporary and adds
// init on the host.  Here it is the fused binary transform_reduce: one
// generated kernel folds op2(a[i], b[i]) with op1, then init op1 result.
#ifndef BOOST_COMPUTE_ALGORITHM_INNER_PRODUCT_HPP
#define BOOST_COMPUTE_ALGORITHM_INNER_PRODUCT_HPP

#include <iterator>

#include <boost/compute/algorithm/transform_reduce.hpp>

namespace boost {
namespace compute {

template <class InputIterator1, class InputIterator2, class T, class BinaryAccumulateFunction,
          class BinaryTransformFunction>
inline T inner_product(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2, T init,
                       BinaryAccumulateFunction accumulate_function, BinaryTransformFunction transform_function,
                       command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator1>::value_type A;
  typedef typename std::iterator_traits<InputIterator2>::value_type B;
  if (first1 == last1) return init;
  detail::device_range<InputIterator1> a(first1, last1, queue);
  detail::device_range<InputIterator2> b(first2, first2 + std::ptrdiff_t(a.n), queue);
  vector<T> out(1, queue.get_context());
  detail::fused_transform_reduce<T, A, B>(a.ptr, b.ptr, a.n, transform_function, accumulate_function, out.data(),
                                          queue, &init);
  return out.begin().read(queue);
}

template <class InputIterator1, class InputIterator2, class T>
inline T inner_product(InputIterator1 first1, InputIterator1 last1, InputIterator2 first2, T init,
                       command_queue &queue = system::default_queue()) {
  return ::boost::compute::inner_product(first1, last1, first2, init, plus<T>(), multiplies<T>(), queue);
}

}  // namespace compute
}  // namespace boost

#endif
