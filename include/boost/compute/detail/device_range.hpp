// boost/compute/detail/device_range.hpp -- how the algorithms of this layer
// get a device pointer for an input range: buffer iterators pass straight
// through; counting and constant iterators are materialised in a temporary
// device array.
#ifndef BOOST_COMPUTE_DETAIL_DEVICE_RANGE_HPP
#define BOOST_COMPUTE_DETAIL_DEVICE_RANGE_HPP

#include <vector>

#include <boost/compute/container/vector.hpp>
#include <boost/compute/iterator/buffer_iterator.hpp>
#include <boost/compute/iterator/counting_iterator.hpp>
#include <boost/compute/types.hpp>

namespace boost {
namespace compute {
namespace detail {

template <class Iterator>
struct device_range {
  typedef typename std::iterator_traits<Iterator>::value_type T;
  // Any other iterator: evaluate on the host and upload.
  device_range(Iterator first, Iterator last, command_queue &queue) {
    std::vector<T> host;
    for (Iterator it = first; it != last; ++it) host.push_back(*it);
    n = host.size();
    tmp = vector<T>(host.begin(), host.end(), queue);
    ptr = tmp.data();
  }
  const T *ptr;
  size_t n;
  vector<T> tmp;
};

template <class T>
struct device_range<buffer_iterator<T> > {
  device_range(buffer_iterator<T> first, buffer_iterator<T> last, command_queue &)
      : ptr(first.get_ptr()), n(size_t(last - first)) {}
  const T *ptr;
  size_t n;
};

template <class T>
inline int bcx_dtype_of() {
  static_assert(bcx_type_of<T>::value >= 0, "element type is not one of the bcx scalar types");
  return bcx_type_of<T>::value;
}

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
