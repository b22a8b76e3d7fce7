// boost/compute/exception.hpp -- error types of the drop-in layer.
//
// Same names and meaning as the reference's exception/opencl_error.hpp:30,
// exception/program_build_failure.hpp:28 and exception/no_device_found.hpp:25:
// every failing bcx_* call is rethrown as opencl_error carrying the status,
// which equals the OpenCL cl_int code wherever one exists.
#ifndef BOOST_COMPUTE_EXCEPTION_HPP
#define BOOST_COMPUTE_EXCEPTION_HPP

#include <exception>
#include <string>

#include <bcx.h>

namespace boost {
namespace compute {

class opencl_error : public std::exception {
 public:
  explicit opencl_error(int error) : m_error(error), m_error_string(to_string(error)) {
    const char *detail = bcx_last_error_string();
    if (detail && *detail) m_error_string += std::string(": ") + detail;
  }
  opencl_error(int error, const std::string &what) : m_error(error), m_error_string(what) {}
  ~opencl_error() throw() {}
  int error_code() const throw() { return m_error; }
  std::string error_string() const throw() { return m_error_string; }
  const char *what() const throw() { return m_error_string.c_str(); }

  static std::string to_string(int error) {
    switch (error) {
      case BCX_SUCCESS: return "Success";
      case BCX_DEVICE_NOT_FOUND: return "Device Not Found";
      case BCX_MEM_ALLOCATION_FAILURE: return "Memory Object Allocation Failure";
      case BCX_OUT_OF_RESOURCES: return "Out of Resources";
      case BCX_BUILD_PROGRAM_FAILURE: return "Build Program Failure";
      case BCX_INVALID_VALUE: return "Invalid Value";
      case BCX_INVALID_KERNEL_NAME: return "Invalid Kernel Name";
      case BCX_INVALID_BUFFER_SIZE: return "Invalid Buffer Size";
      case BCX_DEVICE_TIMEOUT: return "Device Wait Timeout";
      case BCX_UNSUPPORTED: return "Unsupported Type or Functor";
    }
    return "Unknown OpenCL Error (" + std::to_string(error) + ")";
  }

 private:
  int m_error;
  std::string m_error_string;
};

class program_build_failure : public opencl_error {
 public:
  program_build_failure(int error, const std::string &build_log)
      : opencl_error(error, "Build Program Failure"), m_build_log(build_log) {}
  ~program_build_failure() throw() {}
  std::string build_log() const { return m_build_log; }

 private:
  std::string m_build_log;
};

class no_device_found : public std::exception {
 public:
  const char *what() const throw() { return "No OpenCL device found"; }
};

namespace detail {
inline void check(int status) {
  if (status != BCX_SUCCESS) throw opencl_error(status);
}
}  // namespace detail

}  // namespace compute
}  // namespace boost

#endif
