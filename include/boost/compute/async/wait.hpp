// boost/compute/async/wait.hpp -- block until several events or futures have
// completed.
//
// Reference: async/wait.hpp:45 wait_for_all(events...), which waits on a
// wait_list built from events and futures.
#ifndef BOOST_COMPUTE_ASYNC_WAIT_HPP
#define BOOST_COMPUTE_ASYNC_WAIT_HPP

#include <boost/compute/async/future.hpp>
#include <boost/compute/event.hpp>

namespace boost {
namespace compute {

inline void wait_for_all() {}

template <class First, class... Rest>
inline void wait_for_all(First &&first, Rest &&...rest) {
  first.wait();  // an event, or a future
  wait_for_all(static_cast<Rest &&>(rest)...);
}

}  // namespace compute
}  // namespace boost

#endif
