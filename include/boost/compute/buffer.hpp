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
  buffer(const context &ctx, size_t size, int /*flags*/ = read_write, void *host_ptr = nullptr)
      : m_context(ctx), m_size(size) {
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
