// boost/compute/algorithm/sort.hpp, sort_by_key, stable_sort(_by_key).
//
// Reference dispatch: sort.hpp:34-202 and sort_by_key.hpp:33-163 -- for
// less<T>/greater<T> on radix-sortable T, n <= 32 (sort) / n < 32
// (sort_by_key) runs a serial insertion sort and larger n the radix sort;
// stable_sort(_by_key) takes the same route (stable_sort_by_key.hpp:29-54).
// All of that is inside bcx_sort_keys / bcx_sort_pairs; this header only
// forwards the device pointers.  Host iterators are copied to the device,
// sorted and copied back (sort.hpp:125-148).
#ifndef BOOST_COMPUTE_ALGORITHM_SORT_HPP
#define BOOST_COMPUTE_ALGORITHM_SORT_HPP

#include <iterator>
#include <type_traits>
#include <vector>

#include <boost/compute/algorithm/copy.hpp>
#include <boost/compute/detail/merge_sort.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>

namespace boost {
namespace compute {
namespace detail {

template <class T> inline int sort_direction(less<T>) { return 0; }
template <class T> inline int sort_direction(greater<T>) { return 1; }

template <class T>
inline void device_sort(buffer_iterator<T> first, buffer_iterator<T> last, int desc, command_queue &queue) {
  const size_t n = size_t(last - first);
  detail::check(bcx_sort_keys(queue.get(), bcx_dtype(bcx_dtype_of<T>()), first.get_ptr(), n, desc, nullptr, nullptr));
}

template <class K, class V>
inline void device_sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, int desc,
                               command_queue &queue) {
  const size_t n = size_t(kl - kf);
  detail::check(bcx_sort_pairs(queue.get(), bcx_dtype(bcx_dtype_of<K>()), sizeof(V), kf.get_ptr(), vf.get_ptr(),
                               n, desc, nullptr, nullptr));
}

}  // namespace detail

template <class T, class Compare>
inline typename std::enable_if<!detail::is_jit_functor<Compare>::value>::type
sort(buffer_iterator<T> first, buffer_iterator<T> last, Compare compare,
     command_queue &queue = system::default_queue()) {
  detail::device_sort(first, last, detail::sort_direction(compare), queue);
}
// A lambda or BOOST_COMPUTE_FUNCTION comparator: the generated stable merge
// sort (detail/merge_sort.hpp).
template <class T, class Compare>
inline typename std::enable_if<detail::is_jit_functor<Compare>::value>::type
sort(buffer_iterator<T> first, buffer_iterator<T> last, Compare compare,
     command_queue &queue = system::default_queue()) {
  detail::jit_merge_sort<T, unsigned char>(first.get_ptr(), nullptr, size_t(last - first), compare.defs(),
                                           compare.print(), queue);
}
template <class T>
inline void sort(buffer_iterator<T> first, buffer_iterator<T> last, command_queue &queue = system::default_queue()) {
  detail::device_sort(first, last, 0, queue);
}
// Host iterators: copy in, sort on the device, copy back (blocking).
template <class Iterator, class Compare>
inline typename std::enable_if<!is_buffer_iterator<Iterator>::value>::type
sort(Iterator first, Iterator last, Compare compare, command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<Iterator>::value_type T;
  vector<T> dev(first, last, queue);
  ::boost::compute::sort(dev.begin(), dev.end(), compare, queue);
  ::boost::compute::copy(dev.begin(), dev.end(), first, queue);
}
template <class Iterator>
inline typename std::enable_if<!is_buffer_iterator<Iterator>::value>::type
sort(Iterator first, Iterator last, command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<Iterator>::value_type T;
  ::boost::compute::sort(first, last, less<T>(), queue);
}

template <class K, class V, class Compare>
inline typename std::enable_if<!detail::is_jit_functor<Compare>::value>::type
sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, Compare compare,
            command_queue &queue = system::default_queue()) {
  detail::device_sort_by_key(kf, kl, vf, detail::sort_direction(compare), queue);
}
template <class K, class V, class Compare>
inline typename std::enable_if<detail::is_jit_functor<Compare>::value>::type
sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, Compare compare,
            command_queue &queue = system::default_queue()) {
  detail::jit_merge_sort<K, V>(kf.get_ptr(), vf.get_ptr(), size_t(kl - kf), compare.defs(), compare.print(), queue);
}
template <class K, class V>
inline void sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf,
                        command_queue &queue = system::default_queue()) {
  detail::device_sort_by_key(kf, kl, vf, 0, queue);
}

template <class Iterator, class Compare>
inline void stable_sort(Iterator first, Iterator last, Compare compare, command_queue &queue = system::default_queue()) {
  ::boost::compute::sort(first, last, compare, queue);
}
template <class Iterator>
inline void stable_sort(Iterator first, Iterator last, command_queue &queue = system::default_queue()) {
  ::boost::compute::sort(first, last, queue);
}
template <class KI, class VI, class Compare>
inline void stable_sort_by_key(KI kf, KI kl, VI vf, Compare compare, command_queue &queue = system::default_queue()) {
  ::boost::compute::sort_by_key(kf, kl, vf, compare, queue);
}
template <class KI, class VI>
inline void stable_sort_by_key(KI kf, KI kl, VI vf, command_queue &queue = system::default_queue()) {
  ::boost::compute::sort_by_key(kf, kl, vf, queue);
}

// is_sorted: checked on the host after one copy (not a hot-path algorithm).
template <class T, class Compare>
inline bool is_sorted(buffer_iterator<T> first, buffer_iterator<T> last, Compare compare,
                      command_queue &queue = system::default_queue()) {
  std::vector<T> host(size_t(last - first));
  ::boost::compute::copy(first, last, host.begin(), queue);
  for (size_t i = 1; i < host.size(); ++i)
    if (compare(host[i], host[i - 1])) return false;
  return true;
}
template <class T>
inline bool is_sorted(buffer_iterator<T> first, buffer_iterator<T> last, command_queue &queue = system::default_queue()) {
  return ::boost::compute::is_sorted(first, last, less<T>(), queue);
}

namespace detail {
// detail::radix_sort / radix_sort_by_key (radix_sort.hpp:429-462): the radix
// path for any n, as the reference's own tests call it.
template <class T>
inline void radix_sort(buffer_iterator<T> first, buffer_iterator<T> last, command_queue &queue) {
  detail::check(bcx_radix_sort_keys(queue.get(), bcx_dtype(bcx_dtype_of<T>()), first.get_ptr(),
                                    size_t(last - first), 0, nullptr, nullptr));
}
template <class T>
inline void radix_sort(buffer_iterator<T> first, buffer_iterator<T> last, bool ascending, command_queue &queue) {
  detail::check(bcx_radix_sort_keys(queue.get(), bcx_dtype(bcx_dtype_of<T>()), first.get_ptr(),
                                    size_t(last - first), ascending ? 0 : 1, nullptr, nullptr));
}
template <class K, class V>
inline void radix_sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf,
                              command_queue &queue) {
  detail::check(bcx_radix_sort_pairs(queue.get(), bcx_dtype(bcx_dtype_of<K>()), sizeof(V), kf.get_ptr(),
                                     vf.get_ptr(), size_t(kl - kf), 0, nullptr, nullptr));
}
template <class K, class V>
inline void radix_sort_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, bool ascending,
                              command_queue &queue) {
  detail::check(bcx_radix_sort_pairs(queue.get(), bcx_dtype(bcx_dtype_of<K>()), sizeof(V), kf.get_ptr(),
                                     vf.get_ptr(), size_t(kl - kf), ascending ? 0 : 1, nullptr, nullptr));
}
}  // namespace detail

}  // namespace compute
}  // namespace boost

#endif
