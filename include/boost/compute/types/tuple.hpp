// boost/compute/types/tuple.hpp -- std::tuple elements in generated kernels.
//
// Reference: types/tuple.hpp:61-170 declares an OpenCL struct for every
// tuple type used in a kernel (members v0, v1, ...) and names it after its
// element types; get<N>() reads member vN.  Here kernel source gets a
// specialization of std::tuple<V...> itself (the generated code has no
// standard library), a plain struct with members v0..vK placed exactly where
// the host's std::tuple keeps them (offsets measured on the host; the
// generated source asserts each offset and the size, so a layout mismatch
// fails to compile instead of corrupting data).  Device arrays of tuples
// therefore copy to and from std::vector<std::tuple<...>> byte for byte, and a
// BOOST_COMPUTE_FUNCTION may take std::tuple<...> arguments.  Element N is read
// in kernel source with bcx_get<N>(x) (also spelled boost_tuple_get(x, N)).
#ifndef BOOST_COMPUTE_TYPES_TUPLE_HPP
#define BOOST_COMPUTE_TYPES_TUPLE_HPP

#include <algorithm>
#include <cstddef>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include <boost/compute/types.hpp>

namespace boost {
namespace compute {
namespace detail {

// Extra kernel source a type needs (none for the built-in scalar and vector
// types).
template <class T>
struct type_definition {
  static std::string get() { return ""; }
};

template <class... V>
struct cuda_type_name<std::tuple<V...> > {
  static const char *get() {
    static const std::string name = [] {
      std::string s = "std::tuple<";
      const char *parts[] = {cuda_type_name<V>::get()...};
      for (std::size_t i = 0; i < sizeof...(V); ++i) s += std::string(i ? ", " : "") + parts[i];
      return s + ">";
    }();
    return name.c_str();
  }
};

// Identifier-safe form of a tuple's element types (include guards).
template <class... V>
inline std::string tuple_guard() {
  std::string s = "BCX_TUPLE";
  const char *parts[] = {cuda_type_name<V>::get()...};
  for (const char *p : parts) {
    s += "_";
    for (const char *c = p; *c; ++c) s += ((*c >= 'a' && *c <= 'z') || (*c >= 'A' && *c <= 'Z') || (*c >= '0' && *c <= '9')) ? *c : '_';
  }
  return s;
}

template <class Tuple, std::size_t... I>
inline std::vector<std::size_t> tuple_offsets(std::index_sequence<I...>) {
  Tuple t;
  const char *base = reinterpret_cast<const char *>(&t);
  return {std::size_t(reinterpret_cast<const char *>(&std::get<I>(t)) - base)...};
}

template <class... V>
struct type_definition<std::tuple<V...> > {
  static std::string get() {
    typedef std::tuple<V...> Tuple;
    const std::string name = cuda_type_name<Tuple>::get();
    const char *types[] = {cuda_type_name<V>::get()...};
    const std::string defs[] = {type_definition<V>::get()...};
    const std::vector<std::size_t> off = tuple_offsets<Tuple>(std::index_sequence_for<V...>());
    const std::size_t k = sizeof...(V);
    std::vector<std::size_t> order(k);
    for (std::size_t i = 0; i < k; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](std::size_t a, std::size_t b) { return off[a] < off[b]; });
    const std::string guard = tuple_guard<V...>();
    const std::size_t sizes[] = {sizeof(V)...};
    std::string s;
    for (const std::string &d : defs) s += d;
    s += "#ifndef " + guard + "\n#define " + guard + "\n";
    s += "namespace std { template <class...> struct tuple; }\n";
    // Members in the host's memory order with explicit padding up to each
    // host offset: every member then sits where the host keeps it (its offset
    // is a multiple of its alignment there too, so no extra padding arises).
    s += "template <> struct alignas(" + std::to_string(alignof(Tuple)) + ") " + name + " {\n";
    std::size_t cur = 0;
    for (std::size_t i : order) {
      if (off[i] > cur) s += "  unsigned char bcx_pad" + std::to_string(i) + "[" + std::to_string(off[i] - cur) + "];\n";
      s += "  " + std::string(types[i]) + " v" + std::to_string(i) + ";\n";
      cur = off[i] + sizes[i];
    }
    if (sizeof(Tuple) > cur) s += "  unsigned char bcx_pad_tail[" + std::to_string(sizeof(Tuple) - cur) + "];\n";
    for (int konst = 0; konst < 2; ++konst) {
      s += std::string("  template <int N> __device__ __forceinline__ ") + (konst ? "const auto &bcx_at() const {\n"
                                                                                 : "auto &bcx_at() {\n");
      for (std::size_t i = 0; i < k; ++i)
        s += std::string(i ? "    else " : "    ") +
             (i + 1 < k ? "if constexpr (N == " + std::to_string(i) + ") " : "") + "return v" + std::to_string(i) +
             ";\n";
      s += "  }\n";
    }
    s += "};\n";
    s += "static_assert(sizeof(" + name + ") == " + std::to_string(sizeof(Tuple)) +
         ", \"device tuple size differs from the host's\");\n";
    s += "#endif\n";
    return s;
  }
};

}  // namespace detail
}  // namespace compute
}  // namespace boost

#endif
