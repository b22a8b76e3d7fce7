// boost/compute/system.hpp -- default device/context/queue selection.
//
// Reference: system::default_device/default_context/default_queue
// (system.hpp:181-298) pick a device from BOOST_COMPUTE_DEFAULT_DEVICE* env
// vars.  Here BOOST_COMPUTE_DEFAULT_DEVICE may hold a CUDA device index.
#ifndef BOOST_COMPUTE_SYSTEM_HPP
#define BOOST_COMPUTE_SYSTEM_HPP

#include <cstdlib>
#include <vector>

#include <boost/compute/command_queue.hpp>

namespace boost {
namespace compute {

class system {
 public:
  static std::vector<device> devices() {
    int n = 0;
    detail::check(bcx_device_count(&n));
    std::vector<device> d;
    for (int i = 0; i < n; ++i) d.push_back(device(i));
    return d;
  }
  static size_t device_count() { return devices().size(); }
  static device default_device() {
    static device d = pick();
    return d;
  }
  static context default_context() {
    static context c(default_device());
    return c;
  }
  static command_queue &default_queue() {
    static command_queue q(default_context(), default_device());
    return q;
  }
  static void finish() { default_queue().finish(); }

 private:
  static device pick() {
    std::vector<device> d = devices();
    if (d.empty()) throw no_device_found();
    const char *env = std::getenv("BOOST_COMPUTE_DEFAULT_DEVICE");
    if (env) {
      char *end = nullptr;
      long idx = std::strtol(env, &end, 10);
      if (end && *end == 0 && idx >= 0 && size_t(idx) < d.size()) return d[size_t(idx)];
    }
    return d[0];
  }
};

}  // namespace compute
}  // namespace boost

#endif
