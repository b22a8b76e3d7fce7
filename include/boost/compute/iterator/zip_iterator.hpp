// boost/compute/iterator/zip_iterator.hpp -- iterate several ranges in step
// (the reference's iterator/zip_iterator.hpp:40-130, where the binary
// transform is built on it, transform.hpp:56-82).
//
// make_zip_iterator(std::make_tuple(a.begin(), b.begin(), ...)) gives an
// iterator whose value_type is std::tuple<A, B, ...>.  Algorithms read a
// zipped range through one generated gather kernel that builds the tuple
// structs (boost/compute/types/tuple.hpp) from the component ranges; a copy
// into a vector of tuples writes them straight to the destination.  The
// reference zips boost::tuple; this drop-in zips std::tuple (the reference
// also accepts std::tuple element types, types/tuple.hpp:162).
#ifndef BOOST_COMPUTE_ITERATOR_ZIP_ITERATOR_HPP
#define BOOST_COMPUTE_ITERATOR_ZIP_ITERATOR_HPP

#include <cstddef>
#include <iterator>
#include <memory>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>

#include <boost/compute/container/vector.hpp>
#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/detail/jit.hpp>
#include <boost/compute/functional/get.hpp>
#include <boost/compute/types/tuple.hpp>

namespace boost {
namespace compute {

template <class IteratorTuple>
class zip_iterator;

template <class... Its>
class zip_iterator<std::tuple<Its...> > {
 public:
  typedef std::tuple<Its...> iterator_tuple;
  typedef std::tuple<typename std::iterator_traits<Its>::value_type...> value_type;
  typedef std::random_access_iterator_tag iterator_category;
  typedef std::ptrdiff_t difference_type;
  typedef value_type *pointer;
  typedef value_type reference;

  zip_iterator() {}
  explicit zip_iterator(const iterator_tuple &its) : m_its(its) {}
  const iterator_tuple &get_iterator_tuple() const { return m_its; }

  zip_iterator operator+(difference_type d) const { return zip_iterator(advance(d, idx())); }
  zip_iterator operator-(difference_type d) const { return zip_iterator(advance(-d, idx())); }
  zip_iterator &operator+=(difference_type d) { return *this = *this + d; }
  zip_iterator &operator-=(difference_type d) { return *this = *this - d; }
  zip_iterator &operator++() { return *this += 1; }
  zip_iterator &operator--() { return *this -= 1; }
  zip_iterator operator++(int) {
    zip_iterator t = *this;
    *this += 1;
    return t;
  }
  // The ranges move in step, so the first component gives the distance.
  difference_type operator-(const zip_iterator &o) const {
    return difference_type(std::get<0>(m_its) - std::get<0>(o.m_its));
  }
  bool operator==(const zip_iterator &o) const { return std::get<0>(m_its) == std::get<0>(o.m_its); }
  bool operator!=(const zip_iterator &o) const { return !(*this == o); }

 private:
  static std::index_sequence_for<Its...> idx() { return {}; }
  template <std::size_t... I>
  iterator_tuple advance(difference_type d, std::index_sequence<I...>) const {
    return iterator_tuple((std::get<I>(m_its) + d)...);
  }
  iterator_tuple m_its;
};

template <class... Its>
inline zip_iterator<std::tuple<Its...> > make_zip_iterator(const std::tuple<Its...> &its) {
  return zip_iterator<std::tuple<Its...> >(its);
}

namespace detail {

// Source of the gather kernel: out[i] = {c0[i], c1[i], ...} as the tuple
// struct of the zipped value type.
template <class... V>
inline std::string zip_gather_source() {
  typedef std::tuple<V...> Tuple;
  const char *types[] = {cuda_type_name<V>::get()...};
  std::ostringstream src;
  src << jit_prelude() << type_definition<Tuple>::get() << "extern \"C\" __global__ void bcx_jit_zip_gather(";
  for (std::size_t i = 0; i < sizeof...(V); ++i) src << "const " << types[i] << " *__restrict__ c" << i << ", ";
  src << cuda_type_name<Tuple>::get() << " *__restrict__ out, unsigned long long n) {\n"
      << "  const unsigned long long s = (unsigned long long)gridDim.x * blockDim.x;\n"
      << "  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += s) {\n"
      << "    " << cuda_type_name<Tuple>::get() << " t;\n";
  for (std::size_t i = 0; i < sizeof...(V); ++i) src << "    t.v" << i << " = c" << i << "[i];\n";
  src << "    out[i] = t;\n  }\n}\n";
  return src.str();
}

template <class... Its>
struct zip_gather {
  typedef std::tuple<typename std::iterator_traits<Its>::value_type...> Tuple;
  // Component ranges as device arrays (buffer iterators pass through; other
  // iterators are materialised by their own device_range).
  template <std::size_t... I>
  static void run(const std::tuple<Its...> &first, std::size_t n, void *out, command_queue &queue,
                  std::index_sequence<I...>) {
    std::tuple<std::unique_ptr<device_range<Its> >...> parts(
        std::unique_ptr<device_range<Its> >(new device_range<Its>(
            std::get<I>(first), std::get<I>(first) + std::ptrdiff_t(n), queue))...);
    const void *ptrs[] = {static_cast<const void *>(std::get<I>(parts)->ptr)...};
    unsigned long long nn = n;
    void *args[sizeof...(Its) + 2];
    for (std::size_t i = 0; i < sizeof...(Its); ++i) args[i] = &ptrs[i];
    args[sizeof...(Its)] = &out;
    args[sizeof...(Its) + 1] = &nn;
    jit_launch(zip_gather_source<typename std::iterator_traits<Its>::value_type...>(), "bcx_jit_zip_gather",
               grid_for(n, 256), 256, queue, args);
    queue.finish();  // the component temporaries go out of scope here
  }
};

// A zipped range as a device array of tuple structs.
template <class... Its>
struct device_range<zip_iterator<std::tuple<Its...> > > {
  typedef zip_iterator<std::tuple<Its...> > It;
  typedef typename It::value_type T;
  device_range(It first, It last, command_queue &queue) {
    n = std::size_t(last - first);
    tmp = vector<T>(n, queue.get_context());
    if (n) zip_gather<Its...>::run(first.get_iterator_tuple(), n, tmp.data(), queue, std::index_sequence_for<Its...>());
    ptr = tmp.data();
  }
  const T *ptr;
  std::size_t n;
  vector<T> tmp;
};

}  // namespace detail

// A zipped range into a device array of tuples: one gather kernel writing the
// destination directly.
template <class... Its>
inline buffer_iterator<typename zip_iterator<std::tuple<Its...> >::value_type> copy(
    zip_iterator<std::tuple<Its...> > first, zip_iterator<std::tuple<Its...> > last,
    buffer_iterator<typename zip_iterator<std::tuple<Its...> >::value_type> result,
    command_queue &queue = system::default_queue()) {
  const std::size_t n = std::size_t(last - first);
  if (n)
    detail::zip_gather<Its...>::run(first.get_iterator_tuple(), n, result.get_ptr(), queue,
                                    std::index_sequence_for<Its...>());
  return result + std::ptrdiff_t(n);
}

}  // namespace compute
}  // namespace boost

#endif
