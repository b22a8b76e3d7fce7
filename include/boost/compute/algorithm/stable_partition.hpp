// boost/compute/algorithm/stable_partition.hpp -- see partition.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_STABLE_PARTITION_HPP
#define BOOST_COMPUTE_ALGORITHM_STABLE_PARTITION_HPP
#include <boost/compute/algorithm/partition.hpp>
#endif
