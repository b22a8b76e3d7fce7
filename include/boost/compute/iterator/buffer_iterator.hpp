// boost/compute/iterator/buffer_iterator.hpp -- random-access iterator over a
// buffer of T (the reference's iterator/buffer_iterator.hpp:136-260): a
// (buffer, index) pair whose device address feeds the bcx_* calls directly.
#ifndef BOOST_COMPUTE_ITERATOR_BUFFER_ITERATOR_HPP
#define BOOST_COMPUTE_ITERATOR_BUFFER_ITERATOR_HPP

#include <cstddef>
#include <iterator>

#include <bcx.h>
#include <boost/compute/buffer.hpp>
#include <boost/compute/command_queue.hpp>

namespace boost {
namespace compute {

template <class T>
class buffer_iterator {
 public:
  typedef std::random_access_iterator_tag iterator_category;
  typedef T value_type;
  typedef std::ptrdiff_t difference_type;
  typedef T *pointer;
  typedef T reference;

  buffer_iterator() : m_index(0) {}
  buffer_iterator(const buffer &b, size_t index) : m_buffer(b), m_index(index) {}

  const buffer &get_buffer() const { return m_buffer; }
  size_t get_index() const { return m_index; }
  // Device address of the element this iterator points at.
  T *get_ptr() const { return static_cast<T *>(m_buffer.get()) + m_index; }

  T read(command_queue &queue) const {
    T v;
    detail::check(bcx_memcpy_async(&v, get_ptr(), sizeof(T), queue.get()));
    queue.finish();
    return v;
  }
  void write(const T &v, command_queue &queue) const {
    detail::check(bcx_memcpy_async(get_ptr(), &v, sizeof(T), queue.get()));
    queue.finish();
  }

  buffer_iterator &operator++() { ++m_index; return *this; }
  buffer_iterator operator++(int) { buffer_iterator r = *this; ++m_index; return r; }
  buffer_iterator &operator--() { --m_index; return *this; }
  buffer_iterator &operator+=(difference_type d) { m_index = size_t(difference_type(m_index) + d); return *this; }
  buffer_iterator &operator-=(difference_type d) { m_index = size_t(difference_type(m_index) - d); return *this; }
  buffer_iterator operator+(difference_type d) const { buffer_iterator r = *this; r += d; return r; }
  buffer_iterator operator-(difference_type d) const { buffer_iterator r = *this; r -= d; return r; }
  difference_type operator-(const buffer_iterator &o) const {
    return difference_type(m_index) - difference_type(o.m_index);
  }
  bool operator==(const buffer_iterator &o) const { return m_buffer == o.m_buffer && m_index == o.m_index; }
  bool operator!=(const buffer_iterator &o) const { return !(*this == o); }
  bool operator<(const buffer_iterator &o) const { return m_index < o.m_index; }

 private:
  buffer m_buffer;
  size_t m_index;
};

template <class T>
inline buffer_iterator<T> make_buffer_iterator(const buffer &b, size_t index = 0) {
  return buffer_iterator<T>(b, index);
}

template <class Iterator> struct is_buffer_iterator { static const bool value = false; };
template <class T> struct is_buffer_iterator<buffer_iterator<T> > { static const bool value = true; };

}  // namespace compute
}  // namespace boost

#endif
