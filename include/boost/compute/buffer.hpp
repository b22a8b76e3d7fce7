// boost/compute/buffer.hpp -- reference-counted device allocation
// (the reference's buffer.hpp wraps a cl_mem; here a cudaMalloc'd block).
#ifndef BOOST_COMPUTE_BUFFER_HPP
#define BOOST_COMPUTE_BUFFER_HPP

#include <memory>

#include <bcx.h>
#include <boost/compute/context.hpp>
#include <boost/compute/exception.hpp>

namespace boost {
namespace compute {

class buffer {
 public:
  enum mem_flags { read_write = 1 << 0, write_only = 1 << 1, read_only = 1 << 2, use_host_ptr = 1 << 3 };
  buffer() : m_size(0) {}
  // With use_host_ptr the host memory itself is the storage (mapped into the
  // device's address space, CL_MEM_USE_HOST_PTR); otherwise host_ptr, if
  // given, is the initial contents.
  buffer(const context &ctx, size_t size, int flags = read_write, void *host_ptr = nullptr)
      : m_context(ctx), m_size(size) {
    if ((flags & use_host_ptr) && host_ptr && size) {
      void *dev = nullptr;
      detail::check(bcx_host_register(host_ptr, size, (flags & read_only) ? 1 : 0, &dev));
      m_mem = std::shared_ptr<void>(dev, [host_ptr](void *) { bcx_host_unregister(host_ptr); });
      return;
    }
    void *p = nullptr;
    if (size) detail::check(bcx_malloc(&p, size));
    m_mem = std::shared_ptr<void>(p, [](void *q) { if (q) bcx_free(q); });
    if (host_ptr && size) {
      detail::check(bcx_memcpy_async(p, host_ptr, size, nullptr));
      detail::check(bcx_stream_synchronize(nullptr));
    }
  }
  void *get() const { return m_mem.get(); }
  size_t size() const { return m_size; }
  context get_context() const { return m_context; }
  bool operator==(const buffer &o) const { return m_mem == o.m_mem; }
  bool operator!=(const buffer &o) const { return !(*this == o); }

 private:
  context m_context;
  std::shared_ptr<void> m_mem;
  size_t m_size;
};

}  // namespace compute
}  // namespace boost

#endif
