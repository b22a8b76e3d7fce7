// boost/compute/device.hpp -- a CUDA device seen through the reference's
// device interface (device.hpp: name(), compute_units(), type(),
// global_memory_size()).  Every device this library drives is a CUDA GPU.
#ifndef BOOST_COMPUTE_DEVICE_HPP
#define BOOST_COMPUTE_DEVICE_HPP

#include <string>

#include <bcx.h>
#include <boost/compute/exception.hpp>

namespace boost {
namespace compute {

class device {
 public:
  enum type { cpu = 1 << 1, gpu = 1 << 2, accelerator = 1 << 3 };
  device() : m_id(-1) {}
  explicit device(int id) : m_id(id) {}
  int id() const { return m_id; }
  std::string name() const {
    char buf[256] = {0};
    detail::check(bcx_device_info(m_id, buf, sizeof(buf), nullptr, nullptr));
    return buf;
  }
  std::string vendor() const { return "NVIDIA Corporation"; }
  unsigned compute_units() const {
    int cu = 0;
    detail::check(bcx_device_info(m_id, nullptr, 0, &cu, nullptr));
    return unsigned(cu);
  }
  size_t global_memory_size() const {
    size_t bytes = 0;
    detail::check(bcx_device_info(m_id, nullptr, 0, nullptr, &bytes));
    return bytes;
  }
  int type() const { return gpu; }
  bool supports_extension(const std::string &) const { return true; }
  bool operator==(const device &o) const { return m_id == o.m_id; }
  bool operator!=(const device &o) const { return m_id != o.m_id; }

 private:
  int m_id;
};

}  // namespace compute
}  // namespace boost

#endif
