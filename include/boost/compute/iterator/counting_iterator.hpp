// boost/compute/iterator/counting_iterator.hpp and constant_iterator: the
// reference's iterator/counting_iterator.hpp and constant_iterator.hpp.  The
// algorithms of this layer materialise them into a device array first (one
// small upload), then run the normal device path.
#ifndef BOOST_COMPUTE_ITERATOR_COUNTING_ITERATOR_HPP
#define BOOST_COMPUTE_ITERATOR_COUNTING_ITERATOR_HPP

#include <cstddef>
#include <iterator>

namespace boost {
namespace compute {

template <class T>
class counting_iterator {
 public:
  typedef std::random_access_iterator_tag iterator_category;
  typedef T value_type;
  typedef std::ptrdiff_t difference_type;
  typedef T *pointer;
  typedef T reference;
  counting_iterator() : m_value(0) {}
  explicit counting_iterator(T v) : m_value(v) {}
  T operator*() const { return m_value; }
  T operator[](difference_type i) const { return T(m_value + i); }
  counting_iterator &operator++() { ++m_value; return *this; }
  counting_iterator operator+(difference_type d) const { return counting_iterator(T(m_value + d)); }
  difference_type operator-(const counting_iterator &o) const { return difference_type(m_value - o.m_value); }
  bool operator==(const counting_iterator &o) const { return m_value == o.m_value; }
  bool operator!=(const counting_iterator &o) const { return m_value != o.m_value; }

 private:
  T m_value;
};
template <class T>
inline counting_iterator<T> make_counting_iterator(T v) { return counting_iterator<T>(v); }

template <class T>
class constant_iterator {
 public:
  typedef std::random_access_iterator_tag iterator_category;
  typedef T value_type;
  typedef std::ptrdiff_t difference_type;
  typedef T *pointer;
  typedef T reference;
  constant_iterator() : m_value(), m_index(0) {}
  constant_iterator(const T &v, size_t index) : m_value(v), m_index(index) {}
  T operator*() const { return m_value; }
  T operator[](difference_type) const { return m_value; }
  constant_iterator &operator++() { ++m_index; return *this; }
  constant_iterator operator+(difference_type d) const { return constant_iterator(m_value, size_t(difference_type(m_index) + d)); }
  difference_type operator-(const constant_iterator &o) const { return difference_type(m_index) - difference_type(o.m_index); }
  bool operator==(const constant_iterator &o) const { return m_index == o.m_index; }
  bool operator!=(const constant_iterator &o) const { return m_index != o.m_index; }

 private:
  T m_value;
  size_t m_index;
};
template <class T>
inline constant_iterator<T> make_constant_iterator(const T &v, size_t index = 0) { return constant_iterator<T>(v, index); }

}  // namespace compute
}  // namespace boost

#endif
