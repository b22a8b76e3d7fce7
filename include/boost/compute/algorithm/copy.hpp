// boost/compute/algorithm/copy.hpp -- copy between host and device ranges
// (the reference's algorithm/copy.hpp:656-854 dispatch).  Host<->device copies
// block until done (like the reference's blocking enqueue_read/write);
// device->device copies are asynchronous on the queue.
#ifndef BOOST_COMPUTE_ALGORITHM_COPY_HPP
#define BOOST_COMPUTE_ALGORITHM_COPY_HPP

#include <algorithm>
#include <iterator>
#include <vector>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/system.hpp>

namespace boost {
namespace compute {

// device -> device
template <class T>
inline buffer_iterator<T> copy(buffer_iterator<T> first, buffer_iterator<T> last, buffer_iterator<T> result,
                               command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  if (n) detail::check(bcx_memcpy_async(result.get_ptr(), first.get_ptr(), n * sizeof(T), queue.get()));
  return result + std::ptrdiff_t(n);
}

// device -> host
template <class T, class OutputIterator>
inline OutputIterator copy(buffer_iterator<T> first, buffer_iterator<T> last, OutputIterator result,
                           command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  std::vector<T> host(n);
  if (n) detail::check(bcx_memcpy_async(host.data(), first.get_ptr(), n * sizeof(T), queue.get()));
  queue.finish();
  return std::copy(host.begin(), host.end(), result);
}

// host (or counting/constant iterator) -> device
template <class InputIterator, class T>
inline buffer_iterator<T> copy(InputIterator first, InputIterator last, buffer_iterator<T> result,
                               command_queue &queue = system::default_queue()) {
  std::vector<T> host(first, last);
  if (!host.empty())
    detail::check(bcx_memcpy_async(result.get_ptr(), host.data(), host.size() * sizeof(T), queue.get()));
  queue.finish();
  return result + std::ptrdiff_t(host.size());
}

template <class InputIterator, class Size, class OutputIterator>
inline OutputIterator copy_n(InputIterator first, Size count, OutputIterator result,
                             command_queue &queue = system::default_queue()) {
  return ::boost::compute::copy(first, first + std::ptrdiff_t(count), result, queue);
}

template <class T>
inline void fill(buffer_iterator<T> first, buffer_iterator<T> last, const T &value,
                 command_queue &queue = system::default_queue()) {
  std::vector<T> host(size_t(last - first), value);
  ::boost::compute::copy(host.begin(), host.end(), first, queue);
}

template <class T>
inline void iota(buffer_iterator<T> first, buffer_iterator<T> last, const T &value,
                 command_queue &queue = system::default_queue()) {
  std::vector<T> host(size_t(last - first));
  T v = value;
  for (auto &h : host) h = v++;
  ::boost::compute::copy(host.begin(), host.end(), first, queue);
}

}  // namespace compute
}  // namespace boost

#endif
