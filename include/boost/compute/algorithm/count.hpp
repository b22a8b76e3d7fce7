// boost/compute/algorithm/count.hpp -- see count_if.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_COUNT_HPP
#define BOOST_COMPUTE_ALGORITHM_COUNT_HPP
#include <boost/compute/algorithm/count_if.hpp>
#endif
