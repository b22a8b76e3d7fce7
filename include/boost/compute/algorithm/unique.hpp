// boost/compute/algorithm/unique.hpp and unique_copy content.
//
// Reference: unique_copy(first, last, result [, op]) keeps the first element of
// every run of equal elements (unique_copy.hpp:30-160: flags, scan, scatter);
// unique(first, last [, op]) does the same in place through a temporary
// (unique.hpp:30-70).  Here: one generated kernel marks run heads (comparing
// each element with its predecessor), bcx_scan turns marks into positions,
// one generated kernel scatters the heads in order.
#ifndef BOOST_COMPUTE_ALGORITHM_UNIQUE_HPP
#define BOOST_COMPUTE_ALGORITHM_UNIQUE_HPP

#include <iterator>
#include <string>

#include <boost/compute/algorithm/copy_if.hpp>

namespace boost {
namespace compute {
namespace detail {

template <class A, class T>
inline size_t unique_copy_impl(const A *in, size_t n, T *out, const std::string &defs, const std::string &eq,
                               command_queue &queue) {
  vector<uint_> marks(n, queue.get_context()), pos(n, queue.get_context());
  // _0 is the previous element: a head when it differs (or for element 0)
  std::string e = eq;
  std::string expr;
  for (size_t i = 0; i < e.size(); ++i) {
    if (e[i] == '_' && i + 1 < e.size() && e[i + 1] == '2') {
      expr += "_1";
      ++i;
    } else if (e[i] == '_' && i + 1 < e.size() && e[i + 1] == '1') {
      expr += "_0";
      ++i;
    } else {
      expr += e[i];
    }
  }
  const size_t count = mark_adjacent_and_scan(in, n, defs, "first || !(" + expr + ")", marks, pos, queue);
  scatter_marked(in, marks, pos, n, out, queue);
  queue.finish();
  return count;
}

}  // namespace detail

template <class InputIterator, class T, class BinaryPredicate>
inline buffer_iterator<T> unique_copy(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                      BinaryPredicate op, command_queue &queue = system::default_queue()) {
  if (first == last) return result;
  detail::device_range<InputIterator> in(first, last, queue);
  std::string defs, expr;
  detail::functor_expr(op, &defs, &expr);  // spelled with _1 (earlier) and _2 (later)
  return result + std::ptrdiff_t(detail::unique_copy_impl(in.ptr, in.n, result.get_ptr(), defs, expr, queue));
}
template <class InputIterator, class T>
inline buffer_iterator<T> unique_copy(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                      command_queue &queue = system::default_queue()) {
  if (first == last) return result;
  detail::device_range<InputIterator> in(first, last, queue);
  return result + std::ptrdiff_t(detail::unique_copy_impl(in.ptr, in.n, result.get_ptr(), "", "_1 == _2", queue));
}

template <class T, class BinaryPredicate>
inline buffer_iterator<T> unique(buffer_iterator<T> first, buffer_iterator<T> last, BinaryPredicate op,
                                 command_queue &queue = system::default_queue()) {
  const size_t n = size_t(last - first);
  if (n == 0) return first;
  vector<T> tmp(n, queue.get_context());
  auto end = ::boost::compute::unique_copy(first, last, tmp.begin(), op, queue);
  const size_t m = size_t(end - tmp.begin());
  detail::check(bcx_memcpy_async(first.get_ptr(), tmp.data(), m * sizeof(T), queue.get()));
  queue.finish();
  return first + std::ptrdiff_t(m);
}
template <class T>
inline buffer_iterator<T> unique(buffer_iterator<T> first, buffer_iterator<T> last,
                                 command_queue &queue = system::default_queue()) {
  return ::boost::compute::unique(first, last, equal_to<T>(), queue);
}

}  // namespace compute
}  // namespace boost

#endif
