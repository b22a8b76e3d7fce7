// boost/compute/algorithm/partition.hpp, stable_partition.hpp, remove_if.hpp
// and remove.hpp content.
//
// Reference: stable_partition(first, last, pred) copies the elements that
// satisfy pred, then the others, into a temporary and back
// (stable_partition.hpp:30-70); partition forwards to it (partition.hpp);
// remove_if / remove keep the elements that do not match, in order, and return
// the new end (remove_if.hpp:30-60, remove.hpp).  Here each is copy_if /
// remove_copy_if (marks, look-back scan, ordered scatter) plus one copy back.
#ifndef BOOST_COMPUTE_ALGORITHM_PARTITION_HPP
#define BOOST_COMPUTE_ALGORITHM_PARTITION_HPP

#include <string>

#include <boost/compute/algorithm/copy_if.hpp>

namespace boost {
namespace compute {

template <class T, class UnaryPredicate>
inline buffer_iterator<T> stable_partition(buffer_iterator<T> first, buffer_iterator<T> last,
                                           UnaryPredicate predicate,
                                           command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  if (n == 0) return first;
  vector<T> tmp(n, queue.get_context());
  auto mid = ::boost::compute::copy_if(first, last, tmp.begin(), predicate, queue);
  ::boost::compute::remove_copy_if(first, last, mid, predicate, queue);
  detail::check(bcx_memcpy_async(first.get_ptr(), tmp.data(), n * sizeof(T), queue.get()));
  queue.finish();
  return first + (mid - tmp.begin());
}

template <class T, class UnaryPredicate>
inline buffer_iterator<T> partition(buffer_iterator<T> first, buffer_iterator<T> last, UnaryPredicate predicate,
                                    command_queue &queue = system::default_queue()) {
  return ::boost::compute::stable_partition(first, last, predicate, queue);
}

template <class T, class Predicate>
inline buffer_iterator<T> remove_if(buffer_iterator<T> first, buffer_iterator<T> last, Predicate predicate,
                                    command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  if (n == 0) return first;
  vector<T> tmp(n, queue.get_context());
  auto end = ::boost::compute::remove_copy_if(first, last, tmp.begin(), predicate, queue);
  const size_t m = size_t(end - tmp.begin());
  detail::check(bcx_memcpy_async(first.get_ptr(), tmp.data(), m * sizeof(T), queue.get()));
  queue.finish();
  return first + std::ptrdiff_t(m);
}

template <class T>
inline buffer_iterator<T> remove(buffer_iterator<T> first, buffer_iterator<T> last, const T &value,
                                 command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  if (n == 0) return first;
  detail::device_range<buffer_iterator<T> > in(first, last, queue);
  vector<uint_> marks(n, queue.get_context()), pos(n, queue.get_context());
  const std::string pred = "!(_1 == (" + std::string(detail::cuda_type_name<T>::get()) + ")" + detail::literal(value) + ")";
  const size_t m = detail::mark_and_scan(in.ptr, n, "", pred, marks, pos, queue);
  vector<T> tmp(n, queue.get_context());
  detail::scatter_marked(in.ptr, marks, pos, n, tmp.data(), queue);
  detail::check(bcx_memcpy_async(first.get_ptr(), tmp.data(), m * sizeof(T), queue.get()));
  queue.finish();
  return first + std::ptrdiff_t(m);
}

}  // namespace compute
}  // namespace boost

#endif
