// boost/compute/algorithm/reduce_by_key.hpp -- one output per run of equal
// consecutive keys (reduce_by_key.hpp; detail/reduce_by_key_with_scan.hpp:
// 432-486).  Like the reference, it blocks to read the run count and returns
// the ends of the two output ranges.
#ifndef BOOST_COMPUTE_ALGORITHM_REDUCE_BY_KEY_HPP
#define BOOST_COMPUTE_ALGORITHM_REDUCE_BY_KEY_HPP

#include <type_traits>
#include <utility>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/discard_iterator.hpp>

namespace boost {
namespace compute {

template <class K, class V, class BinaryFunction, class BinaryPredicate>
inline std::pair<buffer_iterator<K>, buffer_iterator<V> >
reduce_by_key(buffer_iterator<K> keys_first, buffer_iterator<K> keys_last, buffer_iterator<V> values_first,
              buffer_iterator<K> keys_result, buffer_iterator<V> values_result, BinaryFunction, BinaryPredicate,
              command_queue &queue = system::default_queue()) {
  static_assert(detail::is_builtin_binary<BinaryFunction>::value, "reduce_by_key: built-in functors only");
  static_assert(std::is_same<BinaryPredicate, equal_to<K> >::value, "reduce_by_key: equal_to<K> only");
  const size_t n = size_t(keys_last - keys_first);
  vector<ulong_> count(1, queue.get_context());
  const int comp = std::is_floating_point<V>::value && BinaryFunction::bcx_op == BCX_PLUS;
  detail::check(bcx_reduce_by_key(queue.get(), bcx_dtype(detail::bcx_dtype_of<K>()),
                                  bcx_dtype(detail::bcx_dtype_of<V>()), bcx_op(BinaryFunction::bcx_op),
                                  keys_first.get_ptr(), values_first.get_ptr(), n, keys_result.get_ptr(),
                                  values_result.get_ptr(), reinterpret_cast<uint64_t *>(count.data()), comp,
                                  nullptr, nullptr));
  const std::ptrdiff_t m = n ? std::ptrdiff_t(count.begin().read(queue)) : 0;
  return std::make_pair(keys_result + m, values_result + m);
}
// Run keys discarded: only the reduced values are written.
template <class K, class V, class BinaryFunction>
inline std::pair<discard_iterator, buffer_iterator<V> >
reduce_by_key(buffer_iterator<K> keys_first, buffer_iterator<K> keys_last, buffer_iterator<V> values_first,
              discard_iterator keys_result, buffer_iterator<V> values_result, BinaryFunction,
              command_queue &queue = system::default_queue()) {
  static_assert(detail::is_builtin_binary<BinaryFunction>::value, "reduce_by_key: built-in functors only");
  const size_t n = size_t(keys_last - keys_first);
  vector<ulong_> count(1, queue.get_context());
  const int comp = std::is_floating_point<V>::value && BinaryFunction::bcx_op == BCX_PLUS;
  detail::check(bcx_reduce_by_key(queue.get(), bcx_dtype(detail::bcx_dtype_of<K>()),
                                  bcx_dtype(detail::bcx_dtype_of<V>()), bcx_op(BinaryFunction::bcx_op),
                                  keys_first.get_ptr(), values_first.get_ptr(), n, nullptr, values_result.get_ptr(),
                                  reinterpret_cast<uint64_t *>(count.data()), comp, nullptr, nullptr));
  const std::ptrdiff_t m = n ? std::ptrdiff_t(count.begin().read(queue)) : 0;
  return std::make_pair(keys_result + m, values_result + m);
}
template <class K, class V>
inline std::pair<discard_iterator, buffer_iterator<V> >
reduce_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, discard_iterator kr,
              buffer_iterator<V> vr, command_queue &queue = system::default_queue()) {
  return ::boost::compute::reduce_by_key(kf, kl, vf, kr, vr, plus<V>(), queue);
}

template <class K, class V, class BinaryFunction>
inline std::pair<buffer_iterator<K>, buffer_iterator<V> >
reduce_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, buffer_iterator<K> kr,
              buffer_iterator<V> vr, BinaryFunction op, command_queue &queue = system::default_queue()) {
  return ::boost::compute::reduce_by_key(kf, kl, vf, kr, vr, op, equal_to<K>(), queue);
}
template <class K, class V>
inline std::pair<buffer_iterator<K>, buffer_iterator<V> >
reduce_by_key(buffer_iterator<K> kf, buffer_iterator<K> kl, buffer_iterator<V> vf, buffer_iterator<K> kr,
              buffer_iterator<V> vr, command_queue &queue = system::default_queue()) {
  return ::boost::compute::reduce_by_key(kf, kl, vf, kr, vr, plus<V>(), equal_to<K>(), queue);
}

}  // namespace compute
}  // namespace boost

#endif
