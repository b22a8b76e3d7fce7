// boost/compute/algorithm/count_if.hpp and count.hpp content.
//
// Reference: count_if(first, last, predicate) (count_if.hpp:28-60) picks a
// work-group counting kernel, and count(first, last, value) counts
// `_1 == value` (count.hpp:35-60).  Here both are one generated reduce kernel
// that folds `predicate(x) ? 1 : 0` in 64 bits (the transform_reduce path), so
// nothing is written besides the result.
#ifndef BOOST_COMPUTE_ALGORITHM_COUNT_IF_HPP
#define BOOST_COMPUTE_ALGORITHM_COUNT_IF_HPP

#include <cstddef>
#include <iterator>
#include <string>

#include <boost/compute/algorithm/transform_reduce.hpp>
#include <boost/compute/types/tuple.hpp>

namespace boost {
namespace compute {
namespace detail {

// Number of elements for which the kernel-side expression `pred` (of _1) holds.
template <class InputIterator>
inline size_t count_where(InputIterator first, InputIterator last, const std::string &defs, const std::string &pred,
                          command_queue &queue) {
  typedef typename std::iterator_traits<InputIterator>::value_type A;
  if (first == last) return 0;
  device_range<InputIterator> in(first, last, queue);
  vector<ulong_> out(1, queue.get_context());
  jit_fold(type_definition<A>::get() + defs, "_1 + _2", "unsigned long long", sizeof(unsigned long long),
           "const auto _1 = a[i]; return (T)((" + pred + ") ? 1ull : 0ull);", cuda_type_name<A>::get(), nullptr,
           in.ptr, nullptr, in.n, nullptr, out.data(), queue);
  return size_t(out.begin().read(queue));
}

}  // namespace detail

template <class InputIterator, class Predicate>
inline size_t count_if(InputIterator first, InputIterator last, Predicate predicate,
                       command_queue &queue = system::default_queue()) {
  std::string defs, expr;
  detail::functor_expr(predicate, &defs, &expr);
  return detail::count_where(first, last, defs, expr, queue);
}

template <class InputIterator, class T>
inline size_t count(InputIterator first, InputIterator last, const T &value,
                    command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type A;
  return detail::count_where(first, last, "", "_1 == (" + std::string(detail::cuda_type_name<A>::get()) + ")" +
                                                  detail::literal(A(value)),
                             queue);
}

}  // namespace compute
}  // namespace boost

#endif
