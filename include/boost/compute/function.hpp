// boost/compute/function.hpp -- user functions compiled into the kernels.
//
// Reference: BOOST_COMPUTE_FUNCTION(return_type, name, (arguments), { body })
// (function.hpp:458-463) stringifies the body into a function<Signature>
// whose source is emitted into every kernel that uses it (function.hpp:
// 337-420); BOOST_COMPUTE_CLOSURE (closure.hpp:334-340) also captures host
// values.  Here the body is CUDA C++ (the usual C subset of OpenCL C bodies
// compiles as is; OpenCL-only syntax such as (int2)(a, b) vector literals is
// rejected by NVRTC with program_build_failure).  Captured values are emitted
// as exact literals.
#ifndef BOOST_COMPUTE_FUNCTION_HPP
#define BOOST_COMPUTE_FUNCTION_HPP

#include <string>

#include <boost/compute/detail/jit.hpp>

namespace boost {
namespace compute {

template <class Signature>
class function;

template <class R, class... Args>
class function<R(Args...)> {
 public:
  typedef R result_type;
  static const int arity = int(sizeof...(Args));
  function(const std::string &name, const std::string &definition) : m_name(name), m_definition(definition) {}
  std::string name() const { return m_name; }
  std::string source() const { return m_definition; }
  // Kernel-side call on the placeholders _1, _2, ...
  std::string print() const {
    std::string s = m_name + "(";
    for (int i = 0; i < arity; ++i) s += (i ? ", _" : "_") + std::to_string(i + 1);
    return s + ")";
  }
  std::string defs() const { return m_definition + "\n"; }

 private:
  std::string m_name;
  std::string m_definition;
};

namespace detail {

template <class Signature>
inline function<Signature> make_function(const char *name, const char *return_type, const char *arguments,
                                         const char *body) {
  return function<Signature>(name, std::string("__device__ __forceinline__ ") + return_type + " " + name +
                                       arguments + " " + body);
}

inline void closure_captures(std::string &, const char *, int) {}
template <class T, class... Rest>
inline void closure_captures(std::string &out, const char *names, int index, const T &v, const Rest &...rest) {
  // names is "(a, b, c)": take the index-th identifier.
  std::string list(names);
  std::string cur;
  int k = 0;
  std::string id;
  for (char c : list) {
    if (c == '(' || c == ' ') continue;
    if (c == ',' || c == ')') {
      if (k == index) id = cur;
      cur.clear();
      ++k;
      continue;
    }
    cur += c;
  }
  out += "  const auto " + id + " = " + literal(v) + ";\n";
  closure_captures(out, names, index + 1, rest...);
}

template <class Signature, class... Captured>
inline function<Signature> make_closure(const char *name, const char *return_type, const char *arguments,
                                        const char *capture_names, const char *body, const Captured &...values) {
  std::string caps;
  closure_captures(caps, capture_names, 0, values...);
  return function<Signature>(name, std::string("__device__ __forceinline__ ") + return_type + " " + name +
                                       arguments + " {\n" + caps + body + "\n}");
}

template <class F> struct is_user_function { static const bool value = false; };
template <class S> struct is_user_function<function<S> > { static const bool value = true; };

}  // namespace detail

#define BOOST_COMPUTE_DETAIL_UNPAREN(...) __VA_ARGS__

#define BOOST_COMPUTE_FUNCTION(return_type, name, arguments, ...)                              \
  ::boost::compute::function<return_type arguments> name =                                      \
      ::boost::compute::detail::make_function<return_type arguments>(#name, #return_type,       \
                                                                     #arguments, #__VA_ARGS__)

#define BOOST_COMPUTE_CLOSURE(return_type, name, arguments, capture, ...)                       \
  ::boost::compute::function<return_type arguments> name =                                      \
      ::boost::compute::detail::make_closure<return_type arguments>(                            \
          #name, #return_type, #arguments, #capture, #__VA_ARGS__, BOOST_COMPUTE_DETAIL_UNPAREN capture)

}  // namespace compute
}  // namespace boost

#endif
