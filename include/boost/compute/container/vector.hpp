// boost/compute/container/vector.hpp -- contiguous device array of T
// (the reference's container/vector.hpp:104-250), backed by one buffer.
#ifndef BOOST_COMPUTE_CONTAINER_VECTOR_HPP
#define BOOST_COMPUTE_CONTAINER_VECTOR_HPP

#include <algorithm>
#include <iterator>
#include <vector>

#include <boost/compute/buffer.hpp>
#include <boost/compute/iterator/buffer_iterator.hpp>
#include <boost/compute/system.hpp>

namespace boost {
namespace compute {
namespace detail {

// Reference to one device element: reads and writes block on the default
// queue, like the reference's buffer_value<T>.
template <class T>
class buffer_value {
 public:
  buffer_value(const buffer_iterator<T> &it) : m_it(it) {}
  operator T() const { return m_it.read(system::default_queue()); }
  buffer_value &operator=(const T &v) {
    m_it.write(v, system::default_queue());
    return *this;
  }

 private:
  buffer_iterator<T> m_it;
};

}  // namespace detail

template <class T>
class vector {
 public:
  typedef T value_type;
  typedef buffer_iterator<T> iterator;
  typedef buffer_iterator<T> const_iterator;
  typedef size_t size_type;

  explicit vector(const context &ctx = system::default_context()) : m_size(0), m_context(ctx) {}
  explicit vector(size_t n, const context &ctx = system::default_context())
      : m_size(n), m_context(ctx), m_buffer(ctx, n * sizeof(T)) {}
  vector(size_t n, const T &value, command_queue &queue = system::default_queue())
      : m_size(n), m_context(queue.get_context()), m_buffer(m_context, n * sizeof(T)) {
    std::vector<T> host(n, value);
    upload(host.data(), n, queue);
  }
  template <class InputIterator>
  vector(InputIterator first, InputIterator last, command_queue &queue = system::default_queue())
      : m_context(queue.get_context()) {
    std::vector<T> host(first, last);
    m_size = host.size();
    m_buffer = buffer(m_context, m_size * sizeof(T));
    upload(host.data(), m_size, queue);
  }
  vector(const std::vector<T> &host, command_queue &queue = system::default_queue())
      : vector(host.begin(), host.end(), queue) {}
  vector(const vector &o) : m_size(o.m_size), m_context(o.m_context), m_buffer(o.m_context, o.m_size * sizeof(T)) {
    command_queue &q = system::default_queue();
    if (m_size) detail::check(bcx_memcpy_async(m_buffer.get(), o.m_buffer.get(), m_size * sizeof(T), q.get()));
    q.finish();
  }
  vector &operator=(const vector &o) {
    if (this != &o) {
      vector tmp(o);
      std::swap(m_size, tmp.m_size);
      std::swap(m_buffer, tmp.m_buffer);
      m_context = tmp.m_context;
    }
    return *this;
  }

  iterator begin() const { return iterator(m_buffer, 0); }
  iterator end() const { return iterator(m_buffer, m_size); }
  size_t size() const { return m_size; }
  bool empty() const { return m_size == 0; }
  const buffer &get_buffer() const { return m_buffer; }
  T *data() const { return static_cast<T *>(m_buffer.get()); }
  detail::buffer_value<T> operator[](size_t i) { return detail::buffer_value<T>(begin() + std::ptrdiff_t(i)); }
  T operator[](size_t i) const { return (begin() + std::ptrdiff_t(i)).read(system::default_queue()); }

  void resize(size_t n, command_queue &queue = system::default_queue()) {
    if (n == m_size) return;
    buffer nb(m_context, n * sizeof(T));
    const size_t keep = std::min(n, m_size);
    if (keep) detail::check(bcx_memcpy_async(nb.get(), m_buffer.get(), keep * sizeof(T), queue.get()));
    queue.finish();
    m_buffer = nb;
    m_size = n;
  }
  void clear() { resize(0); }

 private:
  void upload(const T *host, size_t n, command_queue &queue) {
    if (n) detail::check(bcx_memcpy_async(m_buffer.get(), host, n * sizeof(T), queue.get()));
    queue.finish();
  }
  size_t m_size;
  context m_context;
  buffer m_buffer;
};

}  // namespace compute
}  // namespace boost

#endif
