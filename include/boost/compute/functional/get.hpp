// boost/compute/functional/get.hpp -- get<N>(): element N of a tuple or
// component N of a vector type, as a functor for transform and friends
// (the reference's functional/get.hpp:26-92).  In kernel source it is
// bcx_get<N>(_1); the lambda form get<N>(expr) is in boost/compute/lambda.hpp.
#ifndef BOOST_COMPUTE_FUNCTIONAL_GET_HPP
#define BOOST_COMPUTE_FUNCTIONAL_GET_HPP

#include <cstddef>
#include <string>

#include <boost/compute/lambda.hpp>

namespace boost {
namespace compute {

template <std::size_t N>
struct get : lambda::expr_base<get<N> > {
  std::string print() const { return "bcx_get<" + std::to_string(N) + ">(_1)"; }
  std::string defs() const { return ""; }
};

}  // namespace compute
}  // namespace boost

#endif
