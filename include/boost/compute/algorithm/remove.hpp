// boost/compute/algorithm/remove.hpp -- see partition.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_REMOVE_HPP
#define BOOST_COMPUTE_ALGORITHM_REMOVE_HPP
#include <boost/compute/algorithm/partition.hpp>
#endif
