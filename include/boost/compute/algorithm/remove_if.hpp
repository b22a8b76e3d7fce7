// boost/compute/algorithm/remove_if.hpp -- see partition.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_REMOVE_IF_HPP
#define BOOST_COMPUTE_ALGORITHM_REMOVE_IF_HPP
#include <boost/compute/algorithm/partition.hpp>
#endif
