// boost/compute/container/mapped_view.hpp -- a host array used in place by
// device algorithms (the reference's container/mapped_view.hpp:44-220, a
// buffer created with CL_MEM_USE_HOST_PTR over the caller's memory).
//
// The host memory is page-locked and mapped into the device's address space
// for the view's lifetime; kernels read and write it directly (on a Grace
// host, over the CPU-GPU link), so no copy is made.  As in the reference,
// the host must not touch the memory while device work on it is queued:
// map(queue) waits for that work, unmap(queue) hands the memory back.
#ifndef BOOST_COMPUTE_CONTAINER_MAPPED_VIEW_HPP
#define BOOST_COMPUTE_CONTAINER_MAPPED_VIEW_HPP

#include <cstddef>

#include <boost/compute/buffer.hpp>
#include <boost/compute/command_queue.hpp>
#include <boost/compute/iterator/buffer_iterator.hpp>
#include <boost/compute/system.hpp>

namespace boost {
namespace compute {

template <class T>
class mapped_view {
 public:
  typedef T value_type;
  typedef std::size_t size_type;
  typedef buffer_iterator<T> iterator;
  typedef buffer_iterator<T> const_iterator;

  mapped_view() : m_host(nullptr), m_size(0) {}
  mapped_view(T *host_ptr, size_type n, const context &ctx = system::default_context())
      : m_host(host_ptr), m_size(n), m_buffer(ctx, n * sizeof(T), buffer::read_write | buffer::use_host_ptr, host_ptr) {}
  mapped_view(const T *host_ptr, size_type n, const context &ctx = system::default_context())
      : m_host(const_cast<T *>(host_ptr)),
        m_size(n),
        m_buffer(ctx, n * sizeof(T), buffer::read_only | buffer::use_host_ptr, const_cast<T *>(host_ptr)) {}

  iterator begin() { return iterator(m_buffer, 0); }
  iterator end() { return iterator(m_buffer, m_size); }
  const_iterator begin() const { return const_iterator(m_buffer, 0); }
  const_iterator end() const { return const_iterator(m_buffer, m_size); }
  const_iterator cbegin() const { return begin(); }
  const_iterator cend() const { return end(); }
  size_type size() const { return m_size; }
  bool empty() const { return m_size == 0; }
  T *get_host_ptr() const { return m_host; }
  const buffer &get_buffer() const { return m_buffer; }

  // Waits until queued device work on the view has finished, so the host can
  // read what the device wrote.
  void map(command_queue &queue) { queue.finish(); }
  void unmap(command_queue &) {}

 private:
  T *m_host;
  size_type m_size;
  buffer m_buffer;
};

}  // namespace compute
}  // namespace boost

#endif
