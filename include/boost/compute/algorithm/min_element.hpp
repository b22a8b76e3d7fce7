// boost/compute/algorithm/min_element.hpp and max_element.hpp content.
//
// Reference: min_element / max_element(first, last [, compare]) return an
// iterator to the FIRST smallest / largest element (min_element.hpp:40-120,
// max_element.hpp:40-120, detail/find_extrema*.hpp).  Here one generated
// reduce kernel folds (value, index) pairs in index order and keeps the earlier
// pair on ties, so the first extremum wins as in the reference.
#ifndef BOOST_COMPUTE_ALGORITHM_MIN_ELEMENT_HPP
#define BOOST_COMPUTE_ALGORITHM_MIN_ELEMENT_HPP

#include <cstring>
#include <iterator>
#include <string>

#include <boost/compute/algorithm/transform_reduce.hpp>

namespace boost {
namespace compute {
namespace detail {

// Index of the first extremum under `less_expr` (a kernel-side expression of
// _1, _2 meaning "_1 orders before _2"); max selects the largest.
template <class InputIterator>
inline size_t find_extremum(InputIterator first, InputIterator last, const std::string &defs,
                            const std::string &less_expr, bool max, command_queue &queue) {
  typedef typename std::iterator_traits<InputIterator>::value_type V;
  device_range<InputIterator> in(first, last, queue);
  const std::string vt = cuda_type_name<V>::get();
  std::string d = defs + "\nstruct BcxArg { " + vt + " v; unsigned long long i; };\n" +
                  "__device__ __forceinline__ bool bcx_before(const " + vt + " &_1, const " + vt + " &_2) { return (" +
                  less_expr + "); }\n";
  // the later pair replaces the earlier only when strictly better
  const std::string op = max ? "bcx_before(_1.v, _2.v) ? _2 : _1" : "bcx_before(_2.v, _1.v) ? _2 : _1";
  unsigned char result[16] = {0};
  vector<ulong_> out(2, queue.get_context());
  jit_fold(d, op, "BcxArg", 16, "BcxArg r; r.v = a[i]; r.i = i; return r;", vt.c_str(), nullptr, in.ptr, nullptr,
           in.n, nullptr, out.data(), queue);
  check(bcx_memcpy_async(result, out.data(), 16, queue.get()));
  queue.finish();
  unsigned long long idx;
  std::memcpy(&idx, result + 8, 8);
  return size_t(idx);
}

}  // namespace detail

template <class InputIterator, class Compare>
inline InputIterator min_element(InputIterator first, InputIterator last, Compare compare,
                                 command_queue &queue = system::default_queue()) {
  if (first == last) return last;
  std::string defs, expr;
  detail::functor_expr(compare, &defs, &expr);
  return first + std::ptrdiff_t(detail::find_extremum(first, last, defs, expr, false, queue));
}
template <class InputIterator>
inline InputIterator min_element(InputIterator first, InputIterator last,
                                 command_queue &queue = system::default_queue()) {
  if (first == last) return last;
  return first + std::ptrdiff_t(detail::find_extremum(first, last, "", "_1 < _2", false, queue));
}

template <class InputIterator, class Compare>
inline InputIterator max_element(InputIterator first, InputIterator last, Compare compare,
                                 command_queue &queue = system::default_queue()) {
  if (first == last) return last;
  std::string defs, expr;
  detail::functor_expr(compare, &defs, &expr);
  return first + std::ptrdiff_t(detail::find_extremum(first, last, defs, expr, true, queue));
}
template <class InputIterator>
inline InputIterator max_element(InputIterator first, InputIterator last,
                                 command_queue &queue = system::default_queue()) {
  if (first == last) return last;
  return first + std::ptrdiff_t(detail::find_extremum(first, last, "", "_1 < _2", true, queue));
}

}  // namespace compute
}  // namespace boost

#endif
