// boost/compute/event.hpp -- the completion of queued work, as a pair of CUDA
// events recorded around it.
//
// Reference: event.hpp:47-300 wraps a cl_event: wait() (:213) blocks until the
// command completes, status() (:173) reports whether it has, and duration()
// reads the command's start/end profiling stamps.  A CUDA event is a point in
// a stream rather than a command, so an event here holds the marker recorded
// after the work (completion) and, for work this layer enqueued itself (copy,
// enqueue_marker pairs), a marker recorded before it (for duration()).
#ifndef BOOST_COMPUTE_EVENT_HPP
#define BOOST_COMPUTE_EVENT_HPP

#include <chrono>
#include <memory>

#include <bcx.h>
#include <boost/compute/command_queue.hpp>
#include <boost/compute/exception.hpp>

namespace boost {
namespace compute {

class event {
 public:
  // status() values, as the reference's CL_COMPLETE / CL_RUNNING.
  enum { complete = 0, running = 2 };

  event() {}

  // Records a marker at the current end of `queue` (enqueue_marker).
  static event marker(command_queue &queue) {
    event e;
    e.m_end = make();
    detail::check(bcx_event_record(e.m_end.get(), queue.get()));
    return e;
  }
  // Records a marker before and after `enqueue(queue)`; duration() then spans
  // the work it queued.
  template <class Enqueue>
  static event around(command_queue &queue, Enqueue enqueue) {
    event e;
    e.m_start = make();
    e.m_end = make();
    detail::check(bcx_event_record(e.m_start.get(), queue.get()));
    enqueue(queue);
    detail::check(bcx_event_record(e.m_end.get(), queue.get()));
    return e;
  }

  // An event that was never recorded is complete.
  bool valid() const { return bool(m_end); }
  void wait() const {
    if (m_end) detail::check(bcx_event_synchronize(m_end.get()));
  }
  int status() const {
    if (!m_end) return complete;
    int done = 0;
    detail::check(bcx_event_query(m_end.get(), &done));
    return done ? complete : running;
  }
  // Device time between the markers around the work (blocks until done).
  template <class Duration>
  Duration duration() const {
    if (!m_start || !m_end) throw opencl_error(BCX_INVALID_VALUE);
    wait();
    float ms = 0.f;
    detail::check(bcx_event_elapsed_ms(m_start.get(), m_end.get(), &ms));
    return std::chrono::duration_cast<Duration>(std::chrono::duration<double, std::milli>(ms));
  }
  // Makes later work on `queue` wait for this event, without blocking the
  // host (enqueue_barrier with a wait list).
  void enqueue_wait(command_queue &queue) const {
    if (m_end) detail::check(bcx_stream_wait_event(queue.get(), m_end.get()));
  }
  bcx_event get() const { return m_end.get(); }

 private:
  static std::shared_ptr<void> make() {
    bcx_event ev = nullptr;
    detail::check(bcx_event_create(&ev));
    return std::shared_ptr<void>(ev, [](void *p) { bcx_event_destroy(p); });
  }
  std::shared_ptr<void> m_start, m_end;
};

}  // namespace compute
}  // namespace boost

#endif
