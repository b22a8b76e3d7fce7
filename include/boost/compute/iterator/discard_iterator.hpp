// boost/compute/iterator/discard_iterator.hpp -- an output range that drops
// what is written to it (the reference's iterator/discard_iterator.hpp:
// 67-150).  Algorithms that accept it as an output skip that output
// (reduce_by_key does not write its run keys).
#ifndef BOOST_COMPUTE_ITERATOR_DISCARD_ITERATOR_HPP
#define BOOST_COMPUTE_ITERATOR_DISCARD_ITERATOR_HPP

#include <cstddef>
#include <iterator>

namespace boost {
namespace compute {

class discard_iterator {
 public:
  typedef void value_type;
  typedef std::random_access_iterator_tag iterator_category;
  typedef std::ptrdiff_t difference_type;
  explicit discard_iterator(size_t index = 0) : m_index(index) {}
  size_t get_index() const { return m_index; }
  discard_iterator operator+(difference_type d) const { return discard_iterator(size_t(difference_type(m_index) + d)); }
  difference_type operator-(const discard_iterator &o) const { return difference_type(m_index) - difference_type(o.m_index); }
  bool operator==(const discard_iterator &o) const { return m_index == o.m_index; }
  bool operator!=(const discard_iterator &o) const { return m_index != o.m_index; }

 private:
  size_t m_index;
};

inline discard_iterator make_discard_iterator(size_t index = 0) { return discard_iterator(index); }

}  // namespace compute
}  // namespace boost

#endif
