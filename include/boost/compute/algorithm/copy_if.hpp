// boost/compute/algorithm/copy_if.hpp
//
// Reference: copy_if(first, last, result, predicate) (copy_if.hpp:30-80)
// marks each element with the predicate, scans the marks and scatters the
// kept elements (detail/compact.hpp).  Here: one generated kernel writes the
// marks, bcx_scan (single-pass look-back) turns them into output positions,
// and one generated kernel scatters the kept elements in order.  Returns the
// end of the written range (it reads the count back, as the reference does).
#ifndef BOOST_COMPUTE_ALGORITHM_COPY_IF_HPP
#define BOOST_COMPUTE_ALGORITHM_COPY_IF_HPP

#include <iterator>
#include <sstream>
#include <string>

#include <boost/compute/algorithm/transform_reduce.hpp>

namespace boost {
namespace compute {
namespace detail {

// Positions of the elements for which the kernel-side expression `pred` (of
// _1) holds: marks[i] in {0, 1} and their exclusive scan; returns the count.
template <class A>
inline size_t mark_and_scan(const A *in, size_t n, const std::string &defs, const std::string &pred,
                            vector<uint_> &marks, vector<uint_> &pos, command_queue &queue) {
  jit_transform(defs, "((" + pred + ") ? 1u : 0u)", cuda_type_name<A>::get(), "", "unsigned int", sizeof(A), 0, 4,
                in, nullptr, marks.data(), n, queue);
  const uint_ zero = 0;
  check(bcx_scan(queue.get(), BCX_UINT, BCX_PLUS, 1, &zero, marks.data(), pos.data(), n, 0, nullptr, nullptr));
  const uint_ last_pos = (pos.begin() + std::ptrdiff_t(n - 1)).read(queue);
  const uint_ last_mark = (marks.begin() + std::ptrdiff_t(n - 1)).read(queue);
  return size_t(last_pos) + size_t(last_mark);
}

// marks[i] = EXPR ? 1 : 0 where _1 = in[i], _0 = in[i - 1] (in[i] for i == 0)
// and first = (i == 0): predicates that look at the previous element.
template <class A>
inline size_t mark_adjacent_and_scan(const A *in, size_t n, const std::string &defs, const std::string &expr,
                                     vector<uint_> &marks, vector<uint_> &pos, command_queue &queue) {
  std::ostringstream src;
  src << jit_prelude() << defs << "\nextern \"C\" __global__ void bcx_jit_mark_adjacent(const "
      << cuda_type_name<A>::get() << " *__restrict__ in, unsigned *__restrict__ marks, unsigned long long n) {\n"
      << "  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;"
      << " i += (unsigned long long)gridDim.x * blockDim.x) {\n"
      << "    const auto _1 = in[i];\n    const auto _0 = in[i > 0 ? i - 1 : 0];\n    const bool first = i == 0;\n"
      << "    marks[i] = (" << expr << ") ? 1u : 0u;\n  }\n}\n";
  unsigned *m = marks.data();
  unsigned long long nn = n;
  void *args[] = {(void *)&in, (void *)&m, (void *)&nn};
  jit_launch(src.str(), "bcx_jit_mark_adjacent", grid_for(n, 256), 256, queue, args);
  const uint_ zero = 0;
  check(bcx_scan(queue.get(), BCX_UINT, BCX_PLUS, 1, &zero, marks.data(), pos.data(), n, 0, nullptr, nullptr));
  const uint_ last_pos = (pos.begin() + std::ptrdiff_t(n - 1)).read(queue);
  const uint_ last_mark = (marks.begin() + std::ptrdiff_t(n - 1)).read(queue);
  return size_t(last_pos) + size_t(last_mark);
}

template <class A, class T>
inline void scatter_marked(const A *in, const vector<uint_> &marks, const vector<uint_> &pos, size_t n, T *out,
                           command_queue &queue) {
  std::ostringstream src;
  src << jit_prelude() << "extern \"C\" __global__ void bcx_jit_scatter_if(const " << cuda_type_name<A>::get()
      << " *__restrict__ in, const unsigned *__restrict__ marks, const unsigned *__restrict__ pos, "
      << cuda_type_name<T>::get() << " *__restrict__ out, unsigned long long n) {\n"
      << "  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;"
      << " i += (unsigned long long)gridDim.x * blockDim.x)\n"
      << "    if (marks[i]) out[pos[i]] = (" << cuda_type_name<T>::get() << ")in[i];\n}\n";
  const unsigned *m = marks.data(), *p = pos.data();
  unsigned long long nn = n;
  void *args[] = {(void *)&in, (void *)&m, (void *)&p, (void *)&out, (void *)&nn};
  jit_launch(src.str(), "bcx_jit_scatter_if", grid_for(n, 256), 256, queue, args);
}

}  // namespace detail

template <class InputIterator, class T, class Predicate>
inline buffer_iterator<T> copy_if(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                  Predicate predicate, command_queue &queue = system::default_queue()) {
  if (first == last) return result;
  detail::device_range<InputIterator> in(first, last, queue);
  std::string defs, expr;
  detail::functor_expr(predicate, &defs, &expr);
  vector<uint_> marks(in.n, queue.get_context()), pos(in.n, queue.get_context());
  const size_t count = detail::mark_and_scan(in.ptr, in.n, defs, expr, marks, pos, queue);
  detail::scatter_marked(in.ptr, marks, pos, in.n, result.get_ptr(), queue);
  queue.finish();
  return result + std::ptrdiff_t(count);
}

// remove_copy_if keeps what copy_if drops.
template <class InputIterator, class T, class Predicate>
inline buffer_iterator<T> remove_copy_if(InputIterator first, InputIterator last, buffer_iterator<T> result,
                                         Predicate predicate, command_queue &queue = system::default_queue()) {
  if (first == last) return result;
  detail::device_range<InputIterator> in(first, last, queue);
  std::string defs, expr;
  detail::functor_expr(predicate, &defs, &expr);
  vector<uint_> marks(in.n, queue.get_context()), pos(in.n, queue.get_context());
  const size_t count = detail::mark_and_scan(in.ptr, in.n, defs, "!(" + expr + ")", marks, pos, queue);
  detail::scatter_marked(in.ptr, marks, pos, in.n, result.get_ptr(), queue);
  queue.finish();
  return result + std::ptrdiff_t(count);
}

}  // namespace compute
}  // namespace boost

#endif
