// boost/compute/algorithm/unique_copy.hpp -- see unique.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_UNIQUE_COPY_HPP
#define BOOST_COMPUTE_ALGORITHM_UNIQUE_COPY_HPP
#include <boost/compute/algorithm/unique.hpp>
#endif
