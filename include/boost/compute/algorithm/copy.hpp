// boost/compute/algorithm/copy.hpp -- copy between host and device ranges
// (the reference's algorithm/copy.hpp:656-854 dispatch).  Host<->device copies
// block until done (like the reference's blocking enqueue_read/write);
// device->device copies are asynchronous on the queue.  copy_async and
// fill_async return futures; fill is queued on the device.
#ifndef BOOST_COMPUTE_ALGORITHM_COPY_HPP
#define BOOST_COMPUTE_ALGORITHM_COPY_HPP

#include <algorithm>
#include <cstring>
#include <iterator>
#include <type_traits>
#include <vector>

#include <boost/compute/async/future.hpp>
#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/event.hpp>
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

// ---- copy_async (reference: algorithm/copy.hpp:852-875, dispatch :102-148,
// :366-412, :717-760) --------------------------------------------------------
// Queues the copy and returns at once with a future of the output end; the
// future's event completes when the copy has.  Host ranges must be contiguous
// (pointers, std::vector iterators) and hold the device's element type, as in
// the reference.  The host memory must stay valid until the future completes.
// Copies to or from page-locked memory (bcx_malloc_host) overlap other work;
// for pageable memory the CUDA runtime stages the data, so a host-to-device
// copy returns once its data is staged and a device-to-host copy returns when
// it is done.
namespace detail {
template <class Iterator>
struct host_contiguous {
  typedef typename std::remove_cv<typename std::iterator_traits<Iterator>::value_type>::type V;
  static const bool value =
      !std::is_same<V, bool>::value &&
      (std::is_pointer<Iterator>::value || std::is_same<Iterator, typename std::vector<V>::iterator>::value ||
       std::is_same<Iterator, typename std::vector<V>::const_iterator>::value);
};
}  // namespace detail

// host -> device
template <class InputIterator, class T>
inline typename std::enable_if<detail::host_contiguous<InputIterator>::value, future<buffer_iterator<T> > >::type
copy_async(InputIterator first, InputIterator last, buffer_iterator<T> result,
           command_queue &queue = system::default_queue()) {
  static_assert(std::is_same<typename detail::host_contiguous<InputIterator>::V, T>::value,
                "copy_async: host and device element types must match");
  const size_t n = size_t(std::distance(first, last));
  const T *src = n ? &*first : nullptr;
  event e = event::around(queue, [&](command_queue &q) {
    if (n) detail::check(bcx_memcpy_async(result.get_ptr(), src, n * sizeof(T), q.get()));
  });
  return future<buffer_iterator<T> >(result + std::ptrdiff_t(n), e);
}

// device -> host
template <class T, class OutputIterator>
inline typename std::enable_if<detail::host_contiguous<OutputIterator>::value, future<OutputIterator> >::type
copy_async(buffer_iterator<T> first, buffer_iterator<T> last, OutputIterator result,
           command_queue &queue = system::default_queue()) {
  static_assert(std::is_same<typename detail::host_contiguous<OutputIterator>::V, T>::value,
                "copy_async: host and device element types must match");
  const size_t n = size_t(last - first);
  T *dst = n ? &*result : nullptr;
  event e = event::around(queue, [&](command_queue &q) {
    if (n) detail::check(bcx_memcpy_async(dst, first.get_ptr(), n * sizeof(T), q.get()));
  });
  return future<OutputIterator>(result + std::ptrdiff_t(n), e);
}

// device -> device
template <class T>
inline future<buffer_iterator<T> > copy_async(buffer_iterator<T> first, buffer_iterator<T> last,
                                              buffer_iterator<T> result,
                                              command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  event e = event::around(queue, [&](command_queue &q) {
    if (n) detail::check(bcx_memcpy_async(result.get_ptr(), first.get_ptr(), n * sizeof(T), q.get()));
  });
  return future<buffer_iterator<T> >(result + std::ptrdiff_t(n), e);
}

template <class InputIterator, class Size, class OutputIterator>
inline OutputIterator copy_n(InputIterator first, Size count, OutputIterator result,
                             command_queue &queue = system::default_queue()) {
  return ::boost::compute::copy(first, first + std::ptrdiff_t(count), result, queue);
}

namespace detail {
// Queues dst[0, n) = value on the device: a byte memset when every byte of
// value is the same, else one element copied in and then doubled by
// device-to-device copies (ceil(log2 n) of them; each copies the filled prefix
// right after itself, so source and destination never overlap).
template <class T>
inline void enqueue_fill(T *dst, size_t n, const T &value, command_queue &queue) {
  if (n == 0) return;
  unsigned char b[sizeof(T)];
  std::memcpy(b, &value, sizeof(T));
  bool uniform = true;
  for (size_t i = 1; i < sizeof(T); ++i) uniform = uniform && b[i] == b[0];
  if (uniform) {
    check(bcx_memset_async(dst, int(b[0]), n * sizeof(T), queue.get()));
    return;
  }
  check(bcx_memcpy_async(dst, &value, sizeof(T), queue.get()));
  for (size_t done = 1; done < n;) {
    const size_t m = done < n - done ? done : n - done;
    check(bcx_memcpy_async(dst + done, dst, m * sizeof(T), queue.get()));
    done += m;
  }
}
}  // namespace detail

// Reference: algorithm/fill.hpp:281 (fill) and :296 (fill_async, which
// returns a future<void> completed when the fill is done).
template <class T>
inline void fill(buffer_iterator<T> first, buffer_iterator<T> last, const T &value,
                 command_queue &queue = system::default_queue()) {
  detail::enqueue_fill(first.get_ptr(), size_t(last - first), value, queue);
}

template <class T>
inline future<void> fill_async(buffer_iterator<T> first, buffer_iterator<T> last, const T &value,
                               command_queue &queue = system::default_queue()) {
  return future<void>(event::around(
      queue, [&](command_queue &q) { detail::enqueue_fill(first.get_ptr(), size_t(last - first), value, q); }));
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
