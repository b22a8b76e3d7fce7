// boost/compute/command_queue.hpp -- an in-order queue is a CUDA stream.
//
// Reference: command_queue.hpp:78-1570.  Algorithms enqueue work on the
// queue's stream and return; finish() (command_queue.hpp:1564) synchronizes.
#ifndef BOOST_COMPUTE_COMMAND_QUEUE_HPP
#define BOOST_COMPUTE_COMMAND_QUEUE_HPP

#include <memory>

#include <bcx.h>
#include <boost/compute/context.hpp>
#include <boost/compute/exception.hpp>

namespace boost {
namespace compute {

class command_queue {
 public:
  enum properties { enable_profiling = 1 << 1 };
  command_queue() {}
  command_queue(const context &ctx, const device &dev, int /*properties*/ = 0) : m_context(ctx), m_device(dev) {
    detail::check(bcx_set_device(dev.id()));
    bcx_stream s = nullptr;
    detail::check(bcx_stream_create(&s));
    m_stream = std::shared_ptr<void>(s, [](void *p) { bcx_stream_destroy(p); });
  }
  // Wraps an existing stream (not owned), e.g. one from another CUDA library.
  static command_queue from_stream(const context &ctx, bcx_stream s) {
    command_queue q;
    q.m_context = ctx;
    q.m_device = ctx.get_device();
    q.m_stream = std::shared_ptr<void>(s, [](void *) {});
    return q;
  }
  bcx_stream get() const { return m_stream.get(); }
  context get_context() const { return m_context; }
  device get_device() const { return m_device; }
  void finish() const { detail::check(bcx_stream_synchronize(get())); }
  void flush() const {}
  // Raises opencl_error(BCX_DEVICE_TIMEOUT) if a bounded device-side wait of
  // this library expired in work already finished on the device.
  void check_device_errors() const { detail::check(bcx_device_error_check(get())); }

 private:
  context m_context;
  device m_device;
  std::shared_ptr<void> m_stream;
};

}  // namespace compute
}  // namespace boost

#endif
