// boost/compute/algorithm/reduce.hpp and accumulate.hpp content.
//
// Reference: reduce(first, last, result, op) (reduce.hpp:205-305) writes to a
// host pointer (blocking) or a device iterator (asynchronous); an empty range
// writes nothing.  accumulate(first, last, init, op) (accumulate.hpp:102-188)
// returns init op ... and blocks.  Both forward to bcx_reduce/bcx_accumulate
// (one pass, fixed association order); float plus is compensated, and
// minus/divides fold left to right exactly like serial_accumulate.
#ifndef BOOST_COMPUTE_ALGORITHM_REDUCE_HPP
#define BOOST_COMPUTE_ALGORITHM_REDUCE_HPP

#include <type_traits>

#include <boost/compute/detail/device_range.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>

namespace boost {
namespace compute {

namespace detail {
template <class F>
using not_queue = typename std::enable_if<!std::is_same<typename std::decay<F>::type, command_queue>::value>::type;
}  // namespace detail

// device result, built-in functor
template <class InputIterator, class T, class BinaryFunction, class = detail::not_queue<BinaryFunction>,
          class = typename std::enable_if<detail::is_builtin_binary<BinaryFunction>::value>::type>
inline void reduce(InputIterator first, InputIterator last, buffer_iterator<T> result, BinaryFunction,
                   command_queue &queue = system::default_queue()) {
  if (first == last) return;
  detail::device_range<InputIterator> in(first, last, queue);
  const int comp = std::is_floating_point<T>::value && BinaryFunction::bcx_op == BCX_PLUS;
  detail::check(bcx_reduce(queue.get(), bcx_dtype(detail::bcx_dtype_of<T>()), bcx_op(BinaryFunction::bcx_op),
                           in.ptr, in.n, result.get_ptr(), comp, nullptr, nullptr));
  if (!std::is_same<InputIterator, buffer_iterator<T> >::value) queue.finish();
}
// host result (blocking)
template <class InputIterator, class T, class BinaryFunction, class = detail::not_queue<BinaryFunction> >
inline void reduce(InputIterator first, InputIterator last, T *result, BinaryFunction op,
                   command_queue &queue = system::default_queue()) {
  if (first == last) return;
  vector<T> tmp(1, queue.get_context());
  ::boost::compute::reduce(first, last, tmp.begin(), op, queue);
  *result = tmp.begin().read(queue);
}
template <class InputIterator, class OutputIterator>
inline void reduce(InputIterator first, InputIterator last, OutputIterator result,
                   command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type T;
  ::boost::compute::reduce(first, last, result, plus<T>(), queue);
}

// device result, lambda or BOOST_COMPUTE_FUNCTION (associative)
template <class InputIterator, class T, class F, class = typename std::enable_if<detail::is_jit_functor<F>::value>::type>
inline void reduce(InputIterator first, InputIterator last, buffer_iterator<T> result, F f,
                   command_queue &queue = system::default_queue()) {
  if (first == last) return;
  detail::device_range<InputIterator> in(first, last, queue);
  detail::jit_reduce(f.defs(), f.print(), detail::cuda_type_name<T>::get(), sizeof(T), in.ptr, in.n, nullptr,
                     result.get_ptr(), queue);
  if (!std::is_same<InputIterator, buffer_iterator<T> >::value) queue.finish();  // keep the temporary alive
}

template <class InputIterator, class T, class F,
          class = typename std::enable_if<detail::is_jit_functor<F>::value>::type>
inline T accumulate(InputIterator first, InputIterator last, T init, F f, command_queue &queue = system::default_queue()) {
  if (first == last) return init;
  detail::device_range<InputIterator> in(first, last, queue);
  vector<T> tmp(1, queue.get_context());
  detail::jit_reduce(f.defs(), f.print(), detail::cuda_type_name<T>::get(), sizeof(T), in.ptr, in.n, &init,
                     tmp.data(), queue);
  return tmp.begin().read(queue);
}

template <class InputIterator, class T, class BinaryFunction, class = detail::not_queue<BinaryFunction>,
          class = typename std::enable_if<detail::is_builtin_binary<BinaryFunction>::value>::type>
inline T accumulate(InputIterator first, InputIterator last, T init, BinaryFunction,
                    command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type IT;
  if (first == last) return init;
  detail::device_range<InputIterator> in(first, last, queue);
  vector<T> tmp(1, queue.get_context());
  if (!std::is_same<IT, T>::value) {
    // init of another type than the elements: the reference's serial fold
    // with a conversion to T at every step (accumulate.hpp:31-55).
    const std::string s = BinaryFunction::source();  // spelled with a and b
    std::string e;
    for (char c : s) e += (c == 'a') ? std::string("_1") : (c == 'b') ? std::string("_2") : std::string(1, c);
    detail::jit_serial_fold("", e, detail::cuda_type_name<T>::get(), sizeof(T), detail::cuda_type_name<IT>::get(),
                            in.ptr, in.n, &init, tmp.data(), queue);
    return tmp.begin().read(queue);
  }
  const int comp = std::is_floating_point<T>::value && BinaryFunction::bcx_op == BCX_PLUS;
  detail::check(bcx_accumulate(queue.get(), bcx_dtype(detail::bcx_dtype_of<T>()), bcx_op(BinaryFunction::bcx_op),
                               in.ptr, in.n, &init, tmp.data(), comp, nullptr, nullptr));
  return tmp.begin().read(queue);
}
template <class InputIterator, class T>
inline T accumulate(InputIterator first, InputIterator last, T init, command_queue &queue = system::default_queue()) {
  typedef typename std::iterator_traits<InputIterator>::value_type IT;
  return ::boost::compute::accumulate(first, last, init, plus<IT>(), queue);
}

}  // namespace compute
}  // namespace boost

#endif
