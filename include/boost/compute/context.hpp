// boost/compute/context.hpp -- one device's CUDA primary context
// (the reference's context.hpp wraps cl_context).
#ifndef BOOST_COMPUTE_CONTEXT_HPP
#define BOOST_COMPUTE_CONTEXT_HPP

#include <boost/compute/device.hpp>

namespace boost {
namespace compute {

class context {
 public:
  context() {}
  explicit context(const device &d) : m_device(d) {}
  device get_device() const { return m_device; }
  bool operator==(const context &o) const { return m_device == o.m_device; }
  bool operator!=(const context &o) const { return !(*this == o); }

 private:
  device m_device;
};

}  // namespace compute
}  // namespace boost

#endif
