// boost/compute/async/future.hpp -- the result of an asynchronous operation
// together with the event that completes it.
//
// Reference: async/future.hpp:24-105 (future<T>: get() waits then returns the
// result, valid(), wait(), get_event()) and :107-160 (future<void>).
#ifndef BOOST_COMPUTE_ASYNC_FUTURE_HPP
#define BOOST_COMPUTE_ASYNC_FUTURE_HPP

#include <boost/compute/event.hpp>

namespace boost {
namespace compute {

template <class T>
class future {
 public:
  future() {}
  future(const T &result, const event &ev) : m_result(result), m_event(ev) {}

  // Blocks until the operation has completed, then returns its result.
  T get() {
    wait();
    return m_result;
  }
  bool valid() const { return m_event.valid(); }
  void wait() const { m_event.wait(); }
  event get_event() const { return m_event; }

 private:
  T m_result{};
  event m_event;
};

template <>
class future<void> {
 public:
  future() {}
  explicit future(const event &ev) : m_event(ev) {}
  template <class T>
  future(const future<T> &other) : m_event(other.get_event()) {}

  void get() { wait(); }
  bool valid() const { return m_event.valid(); }
  void wait() const { m_event.wait(); }
  event get_event() const { return m_event; }

 private:
  event m_event;
};

}  // namespace compute
}  // namespace boost

#endif
